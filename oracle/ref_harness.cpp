// Test infrastructure (oracle): C API around the reference solver itself.
//
// Built only where the reference sources are present, from the reference's own
// src/solver.cpp, src/FFT.cpp and src/parallel.cpp compiled unmodified against
// the shims in oracle/shim (see oracle/Makefile).  This file replaces the
// reference's main.cpp/IO.cpp: it sets the inline globals of src/setup.hpp
// directly (the values load_params derives, src/IO.cpp:27-34, with PX = PZ = 1
// and one rank) and calls the reference routines.  Arrays cross this API as
// complex128 interleaved in the reference Field layout [z][x][y].
#include <cstring>
#include <iostream>
#include <sstream>
#include <string>
#include "setup.hpp"

namespace {
std::stringstream g_sink;
std::streambuf *g_saved = nullptr;
bool g_quiet = true;
struct Quiet {
  Quiet() { if (g_quiet) { g_saved = std::cout.rdbuf(g_sink.rdbuf()); } }
  ~Quiet() { if (g_quiet) { std::cout.rdbuf(g_saved); g_sink.str(""); } }
};
bool g_fft_ready = false;

Field<Complex> *field_by_name(const char *n) {
  struct E { const char *name; Field<Complex> *f; };
  static const E tab[] = {
      {"velx", &velx}, {"vely", &vely}, {"velz", &velz}, {"vorx", &vorx}, {"vory", &vory},
      {"vorz", &vorz}, {"lmbx", &lmbx}, {"lmby", &lmby}, {"lmbz", &lmbz}, {"Hv", &Hv},
      {"Hg", &Hg}, {"vely_0", &vely_0}, {"vely_1", &vely_1}, {"vely_2", &vely_2},
      {"vory_0", &vory_0}, {"vory_1", &vory_1}, {"vory_2", &vory_2}, {"Hv_0", &Hv_0},
      {"Hv_1", &Hv_1}, {"Hv_2", &Hv_2}, {"Hg_0", &Hg_0}, {"Hg_1", &Hg_1}, {"Hg_2", &Hg_2}};
  for (const E &e : tab) if (std::strcmp(e.name, n) == 0) return e.f;
  return nullptr;
}
Vec<Complex> *cvec_by_name(const char *n) {
  struct E { const char *name; Vec<Complex> *v; };
  static const E tab[] = {
      {"lmbx_mean_0", &lmbx_mean_0}, {"lmbx_mean_1", &lmbx_mean_1}, {"lmbx_mean_2", &lmbx_mean_2},
      {"lmbz_mean_0", &lmbz_mean_0}, {"lmbz_mean_1", &lmbz_mean_1}, {"lmbz_mean_2", &lmbz_mean_2},
      {"velx_mean_0", &velx_mean_0}, {"velx_mean_1", &velx_mean_1}, {"velx_mean_2", &velx_mean_2},
      {"velz_mean_0", &velz_mean_0}, {"velz_mean_1", &velz_mean_1}, {"velz_mean_2", &velz_mean_2}};
  for (const E &e : tab) if (std::strcmp(e.name, n) == 0) return e.v;
  return nullptr;
}
Vec<double> *rvec_by_name(const char *n) {
  struct E { const char *name; Vec<double> *v; };
  static const E tab[] = {{"y", &y}, {"s", &s}, {"dyds1", &dyds1}, {"dyds2", &dyds2}, {"dyds3", &dyds3},
                          {"dyds4", &dyds4}, {"c11", &c11}, {"c21", &c21}, {"c22", &c22}, {"c31", &c31},
                          {"c32", &c32}, {"c33", &c33}, {"c41", &c41}, {"c42", &c42}, {"c43", &c43},
                          {"c44", &c44}, {"kx_local", &kx_local}, {"kz_local", &kz_local}};
  for (const E &e : tab) if (std::strcmp(e.name, n) == 0) return e.v;
  return nullptr;
}
double *scalar_by_name(const char *n) {
  struct E { const char *name; double *p; };
  static const E tab[] = {{"fx_fric", &fx_fric}, {"fz_fric", &fz_fric}, {"fx_fric_0", &fx_fric_0},
                          {"fx_fric_1", &fx_fric_1}, {"fx_fric_2", &fx_fric_2}, {"fz_fric_0", &fz_fric_0},
                          {"fz_fric_1", &fz_fric_1}, {"fz_fric_2", &fz_fric_2}, {"ds", &ds}};
  for (const E &e : tab) if (std::strcmp(e.name, n) == 0) return e.p;
  return nullptr;
}
void copy_in(Field<Complex> &f, const double *src) {
  size_t q = 0;
  for (size_t k = 0; k < f.size_z(); ++k)
    for (size_t i = 0; i < f.size_x(); ++i)
      for (size_t j = 0; j < f.size_y(); ++j, q += 2) f(k, i, j) = Complex(src[q], src[q + 1]);
}
void copy_out(const Field<Complex> &f, double *dst) {
  size_t q = 0;
  for (size_t k = 0; k < f.size_z(); ++k)
    for (size_t i = 0; i < f.size_x(); ++i)
      for (size_t j = 0; j < f.size_y(); ++j, q += 2) {
        dst[q] = f(k, i, j).real();
        dst[q + 1] = f(k, i, j).imag();
      }
}
}  // namespace

extern "C" {

void ref_quiet(int q) { g_quiet = q != 0; }

// Sizes and derived quantities exactly as load_params derives them
// (src/IO.cpp:27-34), one rank: PX = PZ = 1, PXID = PZID = 0.
int ref_init(double dt_, double dkx_, double dkz_, long nx, long ny, long nz, double alpha, double nu_) {
  try {
    Quiet q;
    if (g_fft_ready) { cleanup_fft(); g_fft_ready = false; }
    dt = dt_; dkx = dkx_; dkz = dkz_; NX = nx; NY = ny; NZ = nz; alpha_mesh = alpha; nu = nu_;
    PX = 1; PZ = 1; NT = 0; save_interval = 1; id_step = 0;
    NXH = NX / 2; NZH = NZ / 2; NX2 = NX / 2 * 3; NZ2 = NZ / 2 * 3;
    NXHPX = NXH / PX; NZPZ = NZ / PZ; NYPZ = NY / PZ; NZ2PX = NZ2 / PX;
    my_rank = 0; numProcs = 1; PZID = 0; PXID = 0; MPI_COMM_X = 0; MPI_COMM_Z = 0;
    allocate_var();
    init_mat();
    init_fft();
    g_fft_ready = true;
    return 0;
  } catch (const std::exception &e) {
    std::cerr << "ref_init: " << e.what() << "\n";
    return 1;
  }
}

// The reference's own initial condition (laminar + TS wave), src/solver.cpp:329-426.
int ref_init_fields_builtin() {
  try { Quiet q; init_fields(); return 0; } catch (...) { return 1; }
}

// A caller-given velocity field, then the same start-up sequence as init_fields
// after its initial-condition block (src/solver.cpp:379-425).
int ref_set_velocity(const double *u, const double *v, const double *w) {
  try {
    Quiet q;
    copy_in(velx, u); copy_in(vely, v); copy_in(velz, w);
    get_vor_from_vel();
    Lamb_vec();
    nonlinear_source();
    vely_0 = vely; vely_1 = vely; vely_2 = vely;
    vory_0 = vory; vory_1 = vory; vory_2 = vory;
    Hv_0 = Hv; Hv_1 = Hv; Hv_2 = Hv;
    Hg_0 = Hg; Hg_1 = Hg; Hg_2 = Hg;
    solve_friction_force();
    fx_fric_0 = fx_fric; fx_fric_1 = fx_fric; fx_fric_2 = fx_fric;
    fz_fric_0 = fz_fric; fz_fric_1 = fz_fric; fz_fric_2 = fz_fric;
    velx_mean_0 = velx(0, 0); velx_mean_1 = velx(0, 0); velx_mean_2 = velx(0, 0);
    velz_mean_0 = velz(0, 0); velz_mean_1 = velz(0, 0); velz_mean_2 = velz(0, 0);
    lmbx_mean_0 = lmbx(0, 0); lmbx_mean_1 = lmbx(0, 0); lmbx_mean_2 = lmbx(0, 0);
    lmbz_mean_0 = lmbz(0, 0); lmbz_mean_1 = lmbz(0, 0); lmbz_mean_2 = lmbz(0, 0);
    return 0;
  } catch (const std::exception &e) {
    std::cerr << "ref_set_velocity: " << e.what() << "\n";
    return 1;
  }
}

int ref_step(int n) {
  try {
    Quiet q;
    for (int i = 0; i < n; ++i) { time_Integration(); id_step += 1; }
    return 0;
  } catch (const std::exception &e) {
    std::cerr << "ref_step: " << e.what() << "\n";
    return 1;
  }
}

// Individual reference routines, for component parity tests.
int ref_call(const char *name) {
  try {
    Quiet q;
    std::string s(name);
    if (s == "get_vor_from_vel") get_vor_from_vel();
    else if (s == "solve_horizontal") solve_horizontal();
    else if (s == "Lamb_vec") Lamb_vec();
    else if (s == "nonlinear_source") nonlinear_source();
    else if (s == "solve_friction_force") solve_friction_force();
    else if (s == "time_Integration") time_Integration();
    else return 2;
    return 0;
  } catch (const std::exception &e) {
    std::cerr << "ref_call: " << e.what() << "\n";
    return 1;
  }
}

int ref_get_field(const char *name, double *out) {
  Field<Complex> *f = field_by_name(name);
  if (!f) return 2;
  copy_out(*f, out);
  return 0;
}
int ref_set_field(const char *name, const double *in) {
  Field<Complex> *f = field_by_name(name);
  if (!f) return 2;
  copy_in(*f, in);
  return 0;
}
int ref_get_cvec(const char *name, double *out) {
  Vec<Complex> *v = cvec_by_name(name);
  if (!v) return 2;
  for (size_t j = 0; j < v->size(); ++j) { out[2 * j] = (*v)[j].real(); out[2 * j + 1] = (*v)[j].imag(); }
  return 0;
}
int ref_set_cvec(const char *name, const double *in) {
  Vec<Complex> *v = cvec_by_name(name);
  if (!v) return 2;
  for (size_t j = 0; j < v->size(); ++j) (*v)[j] = Complex(in[2 * j], in[2 * j + 1]);
  return 0;
}
int ref_get_rvec(const char *name, double *out) {
  Vec<double> *v = rvec_by_name(name);
  if (!v) return 2;
  for (size_t j = 0; j < v->size(); ++j) out[j] = (*v)[j];
  return 0;
}
int ref_get_scalar(const char *name, double *out) {
  double *p = scalar_by_name(name);
  if (!p) return 2;
  *out = *p;
  return 0;
}
int ref_set_scalar(const char *name, double val) {
  double *p = scalar_by_name(name);
  if (!p) return 2;
  *p = val;
  return 0;
}
// DY1..DY4 (src/solver.cpp:171-216), written row-major NY x NY.
int ref_get_dy(int which, double *out) {
  const Mat *m = which == 1 ? &DY1 : which == 2 ? &DY2 : which == 3 ? &DY3 : which == 4 ? &DY4 : nullptr;
  if (!m) return 2;
  for (size_t i = 0; i < NY; ++i)
    for (size_t j = 0; j < NY; ++j) out[i * NY + j] = (*m)(i, j);
  return 0;
}
// Fourier2Physical_dealiased on a caller field: in [z][x][y] complex,
// out physical [z2][x2][y] real (src/FFT.cpp:49-128).
int ref_fourier2physical(const double *in, double *out) {
  Field<Complex> f(NZPZ, NXHPX, NY);
  copy_in(f, in);
  Field<double> p(NZ2PX, NX2, NYPZ);
  Fourier2Physical_dealiased(f, p);
  size_t q = 0;
  for (size_t k = 0; k < NZ2PX; ++k)
    for (size_t i = 0; i < NX2; ++i)
      for (size_t j = 0; j < NYPZ; ++j) out[q++] = p(k, i, j);
  return 0;
}
// Physical2Fourier_dealiased (src/FFT.cpp:130-194).
int ref_physical2fourier(const double *in, double *out) {
  Field<double> p(NZ2PX, NX2, NYPZ);
  size_t q = 0;
  for (size_t k = 0; k < NZ2PX; ++k)
    for (size_t i = 0; i < NX2; ++i)
      for (size_t j = 0; j < NYPZ; ++j) p(k, i, j) = in[q++];
  Field<Complex> f(NZPZ, NXHPX, NY);
  Physical2Fourier_dealiased(p, f);
  copy_out(f, out);
  return 0;
}
}

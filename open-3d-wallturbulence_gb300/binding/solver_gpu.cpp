// GPU drop-in for the reference solver's time step.
//
// Compile this file in place of the reference's src/solver.cpp, src/FFT.cpp
// and src/parallel.cpp, against the reference's own headers (src/setup.hpp,
// src/linalg.hpp), and link libowt_gpu.so (include/owt_gpu.h).  The driver
// src/main.cpp and src/IO.cpp stay unchanged: main calls allocate_var,
// init_mat, init_fft and init_fields, then time_Integration once per step
// and save_instant_field every save_interval steps, and cleanup_fft at the
// end (src/main.cpp:63-90).  Those names, and the other routines declared in
// src/setup.hpp:84-114 that have a stand-alone GPU counterpart, are defined
// here with the reference's meaning on the reference's host globals:
//
//   allocate_var          wavenumbers, grid, metric and the host Fields, as
//                         src/solver.cpp:15-167 (the physical-space Fields
//                         velx_p .. lmbz_p and the dense DY1..DY4 are not
//                         allocated: the GPU path never uses them)
//   init_mat + init_fft   one GPU handle (owt_create), which builds the
//                         operators, the banded factorizations and the FFT
//                         plans on the device; the step is replayed as a
//                         CUDA graph
//   init_fields           the reference's laminar + TS-wave velocity
//                         (src/solver.cpp:329-377) on the host, then
//                         owt_init_fields; every host global is refreshed
//   time_Integration      one GPU step; fx_fric, fz_fric and their
//                         histories are read back and printed as
//                         src/solver.cpp:314 prints them; velx, vely, velz
//                         are copied back to the host before every step
//                         whose start main.cpp saves (id_step + 1 a multiple
//                         of save_interval), so save_instant_field writes the
//                         GPU state without any change to main.cpp
//   cleanup_fft           destroys the handle
//   get_vor_from_vel, Lamb_vec, nonlinear_source, solve_friction_force,
//   Fourier2Physical_dealiased, Physical2Fourier_dealiased
//                         run on the GPU on the host globals' current values
//                         (uploaded first) and leave their results in the
//                         host globals
//   EXCHANGE_*            one rank: the pencils are the whole field, the
//                         exchange is a copy
//
// solve_horizontal and solve_mean are not defined: on the GPU they are fused
// into the time step (the mode kernel and the mean-mode kernel), and nothing
// outside src/solver.cpp calls them.  One MPI rank only (PX = PZ = 1; the
// whole channel lives on one GPU); anything else stops in allocate_var with
// std::runtime_error, as the reference stops on its own size checks.
// Environment: OWT_DEVICE (CUDA device ordinal, default 0), OWT_PRECISION
// ("fp64", the default and the reference's arithmetic, or "mixed").
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "owt_gpu.h"
#include "setup.hpp"

namespace {

owt_handle *g_gpu = nullptr;
std::vector<double> g_stage;  // one spectral field, [z][x][y] complex interleaved

void ok(int rc, const char *what) {
  if (rc != OWT_OK) throw std::runtime_error(std::string(what) + ": " + owt_last_error(g_gpu));
}

// Host Field<Complex> <-> the [z][x][y] interleaved layout of the C ABI.
const double *flat(Field<Complex> &f) {
  g_stage.resize(2 * NZ * NXH * NY);
  size_t o = 0;
  for (size_t k = 0; k < NZ; ++k)
    for (size_t i = 0; i < NXH; ++i, o += 2 * NY) std::memcpy(&g_stage[o], f(k, i).data(), NY * sizeof(Complex));
  return g_stage.data();
}
void unflat(Field<Complex> &f) {
  size_t o = 0;
  for (size_t k = 0; k < NZ; ++k)
    for (size_t i = 0; i < NXH; ++i, o += 2 * NY) std::memcpy(f(k, i).data(), &g_stage[o], NY * sizeof(Complex));
}
void put(Field<Complex> &f, int id) { ok(owt_set_field(g_gpu, id, flat(f)), "owt_set_field"); }
void get(Field<Complex> &f, int id) {
  g_stage.resize(2 * NZ * NXH * NY);
  ok(owt_get_field(g_gpu, id, g_stage.data()), "owt_get_field");
  unflat(f);
}

struct FieldId {
  Field<Complex> *f;
  int id;
};
std::vector<FieldId> state_fields() {
  return {{&velx, OWT_VELX},     {&vely, OWT_VELY},     {&velz, OWT_VELZ},     {&vorx, OWT_VORX},
          {&vory, OWT_VORY},     {&vorz, OWT_VORZ},     {&lmbx, OWT_LMBX},     {&lmby, OWT_LMBY},
          {&lmbz, OWT_LMBZ},     {&Hv, OWT_HV},         {&Hg, OWT_HG},         {&vely_0, OWT_VELY_0},
          {&vely_1, OWT_VELY_1}, {&vely_2, OWT_VELY_2}, {&vory_0, OWT_VORY_0}, {&vory_1, OWT_VORY_1},
          {&vory_2, OWT_VORY_2}, {&Hv_0, OWT_HV_0},     {&Hv_1, OWT_HV_1},     {&Hv_2, OWT_HV_2},
          {&Hg_0, OWT_HG_0},     {&Hg_1, OWT_HG_1},     {&Hg_2, OWT_HG_2}};
}
struct MeanId {
  Vec<Complex> *v;
  int id;
};
std::vector<MeanId> mean_vectors() {
  return {{&lmbx_mean_0, OWT_LMBX_MEAN_0}, {&lmbx_mean_1, OWT_LMBX_MEAN_1}, {&lmbx_mean_2, OWT_LMBX_MEAN_2},
          {&lmbz_mean_0, OWT_LMBZ_MEAN_0}, {&lmbz_mean_1, OWT_LMBZ_MEAN_1}, {&lmbz_mean_2, OWT_LMBZ_MEAN_2},
          {&velx_mean_0, OWT_VELX_MEAN_0}, {&velx_mean_1, OWT_VELX_MEAN_1}, {&velx_mean_2, OWT_VELX_MEAN_2},
          {&velz_mean_0, OWT_VELZ_MEAN_0}, {&velz_mean_1, OWT_VELZ_MEAN_1}, {&velz_mean_2, OWT_VELZ_MEAN_2}};
}

// fx_fric, fz_fric and their three history levels from the GPU.
void read_friction() {
  double f[6];
  ok(owt_get_friction(g_gpu, f), "owt_get_friction");
  fx_fric_0 = f[0]; fx_fric_1 = f[1]; fx_fric_2 = f[2];
  fz_fric_0 = f[3]; fz_fric_1 = f[4]; fz_fric_2 = f[5];
  fx_fric = fx_fric_0;
  fz_fric = fz_fric_0;
}
void print_friction() {
  if (my_rank == 0) std::cout << "fx_fric, " << fx_fric << "\n";
}

// Every host global of the step from the GPU state.
void refresh_all() {
  for (const FieldId &q : state_fields()) get(*q.f, q.id);
  for (const MeanId &q : mean_vectors()) ok(owt_get_mean(g_gpu, q.id, reinterpret_cast<double *>(q.v->data())), "owt_get_mean");
  read_friction();
}

double sech_(double x) { return 1.0 / std::cosh(x); }

}  // namespace

void allocate_var() {
  if (numProcs != 1 || PX != 1 || PZ != 1)
    throw std::runtime_error("the GPU time step runs the whole channel on one GPU: one MPI rank, PX = PZ = 1");
  // wavenumbers (src/solver.cpp:25-37, one rank)
  kx_local = Vec<double>(NXHPX);
  kz_local = Vec<double>(NZPZ);
  for (size_t i = 0; i < NXHPX; ++i) kx_local[i] = (double)i * dkx;
  for (size_t k = 0; k < NZPZ; ++k) {
    double t = (double)k;
    if (t >= NZH) t -= NZ;
    kz_local[k] = t * dkz;
  }
  // grid and metric (src/solver.cpp:57-106)
  for (Vec<double> *v : {&s, &y, &dyds1, &dyds2, &dyds3, &dyds4, &c11, &c21, &c22, &c31, &c32, &c33, &c41, &c42, &c43, &c44})
    *v = Vec<double>(NY);
  ds = 2.0 / (NY - 1.0);
  const double ap = alpha_mesh, cth = 1.0 / std::tanh(ap);
  for (size_t i = 0; i < NY; ++i) {
    s[i] = 2 * i / (NY - 1.0) - 1.0;
    const double as = ap * s[i];
    y[i] = std::tanh(as) / std::tanh(ap);
    dyds1[i] = ap * cth * std::pow(sech_(as), 2);
    dyds2[i] = -2 * std::pow(ap, 2) * cth * std::pow(sech_(as), 2) * std::tanh(as);
    dyds3[i] = 2 * std::pow(ap, 3) * (-2 + std::cosh(2 * as)) * cth * std::pow(sech_(as), 4);
    dyds4[i] = -2 * std::pow(ap, 4) * cth * std::pow(sech_(as), 5) * (-11 * std::sinh(as) + std::sinh(3 * as));
  }
  c11 = dyds1.pow(-1);
  c21 = -dyds2 * dyds1.pow(-3);
  c22 = dyds1.pow(-2);
  c31 = -dyds3 * dyds1.pow(-4) + 3.0 * dyds2.pow(2) * dyds1.pow(-5);
  c32 = -3.0 * dyds2 * dyds1.pow(-4);
  c33 = dyds1.pow(-3);
  c41 = -dyds4 * dyds1.pow(-5) + 10.0 * dyds3 * dyds2 * dyds1.pow(-6) - 15.0 * dyds2.pow(3) * dyds1.pow(-7);
  c42 = -4.0 * dyds3 * dyds1.pow(-5) + 15.0 * dyds2.pow(2) * dyds1.pow(-6);
  c43 = -6.0 * dyds2 * dyds1.pow(-5);
  c44 = dyds1.pow(-4);
  // spectral Fields and mean histories, the reference's shapes
  for (const FieldId &q : state_fields()) *q.f = Field<Complex>(NZPZ, NXHPX, NY);
  for (const MeanId &q : mean_vectors()) *q.v = Vec<Complex>(NY);
}

void init_mat() {
  owt_params p{};
  p.dt = dt;
  p.dkx = dkx;
  p.dkz = dkz;
  p.alpha_mesh = alpha_mesh;
  p.nu = nu;
  p.NX = (int64_t)NX;
  p.NY = (int64_t)NY;
  p.NZ = (int64_t)NZ;
  const char *prec = std::getenv("OWT_PRECISION");
  p.precision = (prec && std::string(prec) == "mixed") ? OWT_PREC_MIXED : OWT_PREC_FP64;
  const char *dev = std::getenv("OWT_DEVICE");
  p.device = dev ? std::atoi(dev) : 0;
  p.fd_order = 0;  // the reference's compact schemes
  if (g_gpu) owt_destroy(g_gpu);
  g_gpu = nullptr;
  ok(owt_create(&p, &g_gpu), "owt_create");
  ok(owt_use_graph(g_gpu, 1), "owt_use_graph");
}

// The FFT plans are made by owt_create (init_mat); nothing is left to plan.
void init_fft() {}

void cleanup_fft() {
  if (g_gpu) owt_destroy(g_gpu);
  g_gpu = nullptr;
}

void init_fields() {
  // laminar flow + TS-wave perturbation, src/solver.cpp:336-377
  for (size_t j = 0; j < NY; ++j) velx(0, 0, j) = Complex(1.5 * (1 - std::pow(y[j], 2)), 0.0);
  const double k1 = 2.0, k2 = 2.0, alpha = 1.0;
  for (size_t k = 0; k < NZPZ; ++k)
    for (size_t i = 0; i < NXHPX; ++i)
      for (size_t j = 0; j < NY; ++j) {
        const double y_ = y[j];
        if (kz_local[k] == k2 && kx_local[i] == k1) {
          velx(k, i, j) += alpha / k1 * (y_ - std::pow(y_, 3)) * (-0.25 * IUNIT);
          vely(k, i, j) += alpha * (0.5 * std::pow(y_, 2) - 0.25 * std::pow(y_, 4) - 0.25) * (0.25);
          velz(k, i, j) += -2 * alpha / k2 * (y_ - std::pow(y_, 3)) * (-0.25 * IUNIT);
        }
        if (kz_local[k] == -k2 && kx_local[i] == k1) {
          velx(k, i, j) += alpha / k1 * (y_ - std::pow(y_, 3)) * (-0.25 * IUNIT);
          vely(k, i, j) += alpha * (0.5 * std::pow(y_, 2) - 0.25 * std::pow(y_, 4) - 0.25) * (0.25);
          velz(k, i, j) += -2 * alpha / k2 * (y_ - std::pow(y_, 3)) * (0.25 * IUNIT);
        }
      }
  const size_t n = 2 * NZ * NXH * NY;
  const double *fu = flat(velx);
  std::vector<double> u(fu, fu + n);
  const double *fv = flat(vely);
  std::vector<double> v(fv, fv + n);
  ok(owt_init_fields(g_gpu, u.data(), v.data(), flat(velz)), "owt_init_fields");
  refresh_all();
  print_friction();
}

void time_Integration() {
  ok(owt_time_integration(g_gpu, 1), "owt_time_integration");
  read_friction();  // also reports a device-side numeric failure of the step
  print_friction();
  if (save_interval > 0 && (id_step + 1) % save_interval == 0) {
    get(velx, OWT_VELX);
    get(vely, OWT_VELY);
    get(velz, OWT_VELZ);
  }
}

void get_vor_from_vel() {
  put(velx, OWT_VELX);
  put(vely, OWT_VELY);
  put(velz, OWT_VELZ);
  ok(owt_call(g_gpu, OWT_CALL_GET_VOR_FROM_VEL), "get_vor_from_vel");
  get(vorx, OWT_VORX);
  get(vory, OWT_VORY);
  get(vorz, OWT_VORZ);
}

void Lamb_vec() {
  for (const FieldId &q : state_fields())
    if (q.id <= OWT_VORZ) put(*q.f, q.id);
  for (const MeanId &q : mean_vectors())
    if (q.id <= OWT_LMBZ_MEAN_2) ok(owt_set_mean(g_gpu, q.id, reinterpret_cast<const double *>(q.v->data())), "owt_set_mean");
  ok(owt_call(g_gpu, OWT_CALL_LAMB_VEC), "Lamb_vec");
  get(lmbx, OWT_LMBX);
  get(lmby, OWT_LMBY);
  get(lmbz, OWT_LMBZ);
  for (const MeanId &q : mean_vectors())
    if (q.id <= OWT_LMBZ_MEAN_2) ok(owt_get_mean(g_gpu, q.id, reinterpret_cast<double *>(q.v->data())), "owt_get_mean");
}

void nonlinear_source() {
  put(lmbx, OWT_LMBX);
  put(lmby, OWT_LMBY);
  put(lmbz, OWT_LMBZ);
  ok(owt_call(g_gpu, OWT_CALL_NONLINEAR_SOURCE), "nonlinear_source");
  get(Hv, OWT_HV);
  get(Hg, OWT_HG);
}

void solve_friction_force() {
  put(velx, OWT_VELX);
  put(velz, OWT_VELZ);
  double f[6] = {fx_fric_0, fx_fric_1, fx_fric_2, fz_fric_0, fz_fric_1, fz_fric_2};
  ok(owt_set_friction(g_gpu, f), "owt_set_friction");
  ok(owt_call(g_gpu, OWT_CALL_SOLVE_FRICTION_FORCE), "solve_friction_force");
  read_friction();
  print_friction();
}

void Fourier2Physical_dealiased(const Field<Complex> &u_, Field<double> &up_) {
  Field<Complex> &u = const_cast<Field<Complex> &>(u_);  // read only
  std::vector<double> phys(NZ2 * NX2 * NY);
  ok(owt_fourier2physical(g_gpu, flat(u), phys.data()), "Fourier2Physical_dealiased");
  if (up_.size_z() != NZ2 || up_.size_x() != NX2 || up_.size_y() != NY) up_ = Field<double>(NZ2, NX2, NY);
  size_t o = 0;
  for (size_t k = 0; k < NZ2; ++k)
    for (size_t i = 0; i < NX2; ++i, o += NY) std::memcpy(up_(k, i).data(), &phys[o], NY * sizeof(double));
}

void Physical2Fourier_dealiased(const Field<double> &up_, Field<Complex> &u_) {
  std::vector<double> phys(NZ2 * NX2 * NY);
  size_t o = 0;
  for (size_t k = 0; k < NZ2; ++k)
    for (size_t i = 0; i < NX2; ++i, o += NY) std::memcpy(&phys[o], up_(k, i).data(), NY * sizeof(double));
  g_stage.resize(2 * NZ * NXH * NY);
  ok(owt_physical2fourier(g_gpu, phys.data(), g_stage.data()), "Physical2Fourier_dealiased");
  if (u_.size_z() != NZ || u_.size_x() != NXH || u_.size_y() != NY) u_ = Field<Complex>(NZ, NXH, NY);
  unflat(u_);
}

// One rank: every pencil is the whole field, so each exchange is a copy
// (src/parallel.cpp:4-285 with PX = PZ = 1).
void EXCHANGE_Y2Z(const Field<Complex> &a, Field<Complex> &b) { b = a; }
void EXCHANGE_Z2X(const Field<Complex> &a, Field<Complex> &b) { b = a; }
void EXCHANGE_X2Z(const Field<Complex> &a, Field<Complex> &b) { b = a; }
void EXCHANGE_Z2Y(const Field<Complex> &a, Field<Complex> &b) { b = a; }

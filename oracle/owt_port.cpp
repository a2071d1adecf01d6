// Test infrastructure (oracle): CPU restatement of the reference channel-DNS
// time step, written from the reference's algorithm, not copied from it.
//
// This library is the checker and the timed CPU baseline wherever the
// reference itself cannot be built (the reference needs MPI/FFTW/LAPACK, and
// its sources are not shipped with this repository).  It restates, function by
// function, what the reference computes, including its dense operators and its
// per-mode dense LU solves, so that its results agree with the reference build
// to round-off:
//
//   wavenumbers, grid, metric ...... src/solver.cpp:25-37, 57-106
//   compact-FD stencils A_n, B_n ... src/compdiff.hpp:11-357 (as coded, with the
//                                    B2/B3 top-row duplicate writes, :164-165,
//                                    :257-258)
//   DY1..DY4 = diag(c) A^-1 B ...... src/solver.cpp:171-216
//   get_vor_from_vel ............... src/solver.cpp:218-238
//   nonlinear_source ............... src/solver.cpp:240-260
//   Lamb_vec ....................... src/solver.cpp:262-304
//   solve_friction_force ........... src/solver.cpp:306-327
//   start-up sequence .............. src/solver.cpp:379-425
//   solve_mean ..................... src/solver.cpp:428-514
//   solve_horizontal ............... src/solver.cpp:516-539
//   time_Integration ............... src/solver.cpp:541-627 (optionally with
//                                    wall blowing/suction values in the v
//                                    boundary rows, :593-596)
//   Fourier2Physical_dealiased ..... src/FFT.cpp:49-128
//   Physical2Fourier_dealiased ..... src/FFT.cpp:130-194
//   dense mat-vec (j outer) ........ src/linalg.hpp:434-453
//   Mat::solve (getrf + getrs) ..... src/linalg.hpp:616-690
//
// One process, no MPI: the pencil exchanges (src/parallel.cpp) are identity
// permutations for one rank.  Mode loops and transform lines run under OpenMP.
// Arrays cross the C API as complex128 interleaved in the Field layout
// [z][x][y] (src/linalg.hpp:695-745).
#include <omp.h>

#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "cpu_fft.hpp"

namespace {

using cplx = std::complex<double>;
using owt_oracle::CpuFft;
const cplx I1(0.0, 1.0);

// Dense row-major matrix helpers -----------------------------------------------
struct Dense {
  long n = 0;
  std::vector<double> a;  // row-major
  Dense() = default;
  explicit Dense(long n_) : n(n_), a((size_t)n_ * n_, 0.0) {}
  double &operator()(long i, long j) { return a[(size_t)i * n + j]; }
  double operator()(long i, long j) const { return a[(size_t)i * n + j]; }
};

// LU with partial pivoting in LAPACK dgetf2 order (first maximal |a| as pivot,
// swap whole rows, scale the column, rank-1 update).  In place, row-major.
void lu_factor(Dense &m, std::vector<int> &piv) {
  const long n = m.n;
  piv.assign(n, 0);
  for (long j = 0; j < n; ++j) {
    long p = j;
    double best = std::fabs(m(j, j));
    for (long i = j + 1; i < n; ++i) {
      double v = std::fabs(m(i, j));
      if (v > best) { best = v; p = i; }
    }
    piv[j] = (int)p;
    if (m(p, j) == 0.0) throw std::runtime_error("LU factorization failed. Matrix A may be singular.");
    if (p != j)
      for (long c = 0; c < n; ++c) std::swap(m(j, c), m(p, c));
    const double inv = 1.0 / m(j, j);
    for (long i = j + 1; i < n; ++i) m(i, j) *= inv;
    for (long i = j + 1; i < n; ++i) {
      const double l = m(i, j);
      if (l != 0.0) {
        double *ri = &m.a[(size_t)i * n];
        const double *rj = &m.a[(size_t)j * n];
        for (long c = j + 1; c < n; ++c) ri[c] -= l * rj[c];
      }
    }
  }
}
template <typename T>
void lu_solve(const Dense &m, const std::vector<int> &piv, T *x) {
  const long n = m.n;
  for (long i = 0; i < n; ++i)
    if (piv[i] != i) std::swap(x[i], x[piv[i]]);
  for (long j = 0; j < n; ++j) {
    const T xj = x[j];
    for (long i = j + 1; i < n; ++i) x[i] -= m(i, j) * xj;
  }
  for (long j = n - 1; j >= 0; --j) {
    x[j] /= m(j, j);
    const T xj = x[j];
    for (long i = 0; i < j; ++i) x[i] -= m(i, j) * xj;
  }
}
// out = M * v with the reference's summation order (column j outer).
void matvec(const Dense &m, const cplx *v, cplx *out) {
  const long n = m.n;
  for (long i = 0; i < n; ++i) out[i] = 0.0;
  for (long j = 0; j < n; ++j) {
    const cplx vj = v[j];
    for (long i = 0; i < n; ++i) out[i] += m(i, j) * vj;
  }
}

// Interior order of D1-D3: 8 = the reference's schemes; 6 = the sixth-order
// tridiagonal schemes (alpha 1/3, 2/11, 7/16) on the interior rows (D2 from
// row 3 inward), every boundary row as the reference's.  Not in the reference
// (hard-wired 8th order); the GPU library's fd_order option.
int g_fd_order = 8;

// Compact finite-difference stencils (src/compdiff.hpp), written into dense
// matrices on the uniform s-grid with spacing h.
void stencils(long N, double h, Dense A[4], Dense B[4]) {
  const bool six = g_fd_order == 6;
  for (int q = 0; q < 4; ++q) { A[q] = Dense(N); B[q] = Dense(N); }
  // 1st derivative: 8th-order interior, 4th-order closures (compdiff.hpp:11-69).
  {
    Dense &a = A[0], &b = B[0];
    const double al = six ? 1.0 / 3.0 : 4.0 / 9.0, be = six ? 0.0 : 1.0 / 36.0;
    const double ca = six ? 14.0 / 9.0 : 40.0 / 27.0, cb = six ? 1.0 / 9.0 : 25.0 / 54.0;
    for (long i = 2; i < N - 2; ++i) {
      a(i, i - 2) = be; a(i, i - 1) = al; a(i, i) = 1.0; a(i, i + 1) = al; a(i, i + 2) = be;
      b(i, i - 2) = -cb / (4 * h); b(i, i - 1) = -ca / (2 * h); b(i, i + 1) = ca / (2 * h); b(i, i + 2) = cb / (4 * h);
    }
    for (long i : {1L, N - 2}) {
      a(i, i - 1) = 0.25; a(i, i) = 1.0; a(i, i + 1) = 0.25;
      b(i, i - 1) = -1.5 / (2 * h); b(i, i + 1) = 1.5 / (2 * h);
    }
    const double a0 = -17.0 / 6.0, b0 = 1.5, c0 = 1.5, d0 = -1.0 / 6.0;
    a(0, 0) = 1.0; a(0, 1) = 3.0; a(N - 1, N - 1) = 1.0; a(N - 1, N - 2) = 3.0;
    b(0, 0) = a0 / h; b(0, 1) = b0 / h; b(0, 2) = c0 / h; b(0, 3) = d0 / h;
    b(N - 1, N - 1) = -a0 / h; b(N - 1, N - 2) = -b0 / h; b(N - 1, N - 3) = -c0 / h; b(N - 1, N - 4) = -d0 / h;
  }
  // 2nd derivative (compdiff.hpp:71-166); rows 1 and N-2 centred on 2 and N-3.
  {
    Dense &a = A[1], &b = B[1];
    const double h2 = std::pow(h, 2);
    // sixth order on rows 3..N-4 only: rows 1, N-2 are the sixth-order scheme
    // centred on nodes 2, N-3, so rows 2, N-3 keep the reference's scheme
    for (long i = 2; i < N - 2; ++i) {
      const bool s6 = six && i >= 3 && i <= N - 4;
      const double al = s6 ? 2.0 / 11.0 : 344.0 / 1179.0, be = s6 ? 0.0 : 23.0 / 2358.0;
      const double ca = s6 ? 12.0 / 11.0 : 320.0 / 393.0, cb = s6 ? 3.0 / 11.0 : 310.0 / 393.0;
      a(i, i - 2) = be; a(i, i - 1) = al; a(i, i) = 1.0; a(i, i + 1) = al; a(i, i + 2) = be;
      b(i, i - 2) = cb / (4 * h2); b(i, i - 1) = ca / h2; b(i, i) = -2 * cb / (4 * h2) - 2 * ca / h2;
      b(i, i + 1) = ca / h2; b(i, i + 2) = cb / (4 * h2);
    }
    const double al1 = 2.0 / 11.0, a1 = 12.0 / 11.0, b1 = 3.0 / 11.0;
    for (long i : {1L, N - 2}) {
      const long c = (i == 1) ? 2 : N - 3;
      a(i, c - 1) = al1; a(i, c) = 1.0; a(i, c + 1) = al1;
      b(i, c - 2) = b1 / (4 * h2); b(i, c - 1) = a1 / h2; b(i, c) = -2 * b1 / (4 * h2) - 2 * a1 / h2;
      b(i, c + 1) = a1 / h2; b(i, c + 2) = b1 / (4 * h2);
    }
    a(0, 0) = 1.0; a(0, 1) = 10.0; a(0, 2) = 1.0;
    a(N - 1, N - 1) = 1.0; a(N - 1, N - 2) = 10.0; a(N - 1, N - 3) = 1.0;
    b(0, 0) = 12.0 / h2; b(0, 1) = -24.0 / h2; b(0, 2) = 12.0 / h2; b(0, 3) = 0.0; b(0, 4) = 0.0;
    // Top row: the reference writes (N-1, N-4) twice (d_0 then e_0, both 0)
    // and never (N-1, N-5); the value is 0 either way.
    b(N - 1, N - 1) = 12.0 / h2; b(N - 1, N - 2) = -24.0 / h2; b(N - 1, N - 3) = 12.0 / h2; b(N - 1, N - 4) = 0.0;
  }
  // 3rd derivative (compdiff.hpp:168-259).
  {
    Dense &a = A[2], &b = B[2];
    const double h3 = std::pow(h, 3);
    const double al = six ? 7.0 / 16.0 : 147.0 / 332.0, be = six ? 0.0 : 1.0 / 166.0;
    const double ca = six ? 2.0 : 160.0 / 83.0, cb = six ? -1.0 / 8.0 : -5.0 / 166.0;
    for (long i = 3; i < N - 3; ++i) {
      a(i, i - 2) = be; a(i, i - 1) = al; a(i, i) = 1.0; a(i, i + 1) = al; a(i, i + 2) = be;
      b(i, i - 3) = -cb / (8 * h3); b(i, i - 2) = -ca / (2 * h3); b(i, i - 1) = ca / h3 + 3 * cb / (8 * h3);
      b(i, i + 1) = -ca / h3 - 3 * cb / (8 * h3); b(i, i + 2) = ca / (2 * h3); b(i, i + 3) = cb / (8 * h3);
    }
    const double al2 = 4.0 / 9.0, be2 = 1.0 / 126.0, a2 = 40.0 / 21.0;
    for (long i : {2L, N - 3}) {
      a(i, i - 2) = be2; a(i, i - 1) = al2; a(i, i) = 1.0; a(i, i + 1) = al2; a(i, i + 2) = be2;
      b(i, i - 2) = -a2 / (2 * h3); b(i, i - 1) = a2 / h3; b(i, i + 1) = -a2 / h3; b(i, i + 2) = a2 / (2 * h3);
    }
    a(1, 1) = 0.5; a(1, 2) = 1.0; a(1, 3) = 0.5;
    a(N - 2, N - 4) = 0.5; a(N - 2, N - 3) = 1.0; a(N - 2, N - 2) = 0.5;
    b(1, 0) = -2.0 / (2 * h3); b(1, 1) = 2.0 / h3; b(1, 3) = -2.0 / h3; b(1, 4) = 2.0 / (2 * h3);
    b(N - 2, N - 5) = -2.0 / (2 * h3); b(N - 2, N - 4) = 2.0 / h3; b(N - 2, N - 2) = -2.0 / h3;
    b(N - 2, N - 1) = 2.0 / (2 * h3);
    a(0, 0) = 1.0; a(0, 1) = -7.0; a(N - 1, N - 1) = 1.0; a(N - 1, N - 2) = -7.0;
    b(0, 0) = 8.0 / h3; b(0, 1) = -26.0 / h3; b(0, 2) = 30.0 / h3; b(0, 3) = -14.0 / h3; b(0, 4) = 2.0 / h3;
    // Top row as coded (compdiff.hpp:254-258): (N-1, N-4) is written with
    // -d_0/h3 and then overwritten with -e_0/h3; (N-1, N-5) stays 0.
    b(N - 1, N - 1) = -8.0 / h3; b(N - 1, N - 2) = 26.0 / h3; b(N - 1, N - 3) = -30.0 / h3;
    b(N - 1, N - 4) = -2.0 / h3;
  }
  // 4th derivative (compdiff.hpp:261-357).
  {
    Dense &a = A[3], &b = B[3];
    const double h4 = std::pow(h, 4);
    const double al = 7.0 / 26.0, ca = 19.0 / 13.0, cb = 1.0 / 13.0;
    for (long i = 3; i < N - 3; ++i) {
      a(i, i - 1) = al; a(i, i) = 1.0; a(i, i + 1) = al;
      b(i, i - 3) = cb / (6 * h4); b(i, i - 2) = ca / h4; b(i, i - 1) = -4 * ca / h4 - 9 * cb / (6 * h4);
      b(i, i) = 6 * ca / h4 + 16 * cb / (6 * h4); b(i, i + 1) = -4 * ca / h4 - 9 * cb / (6 * h4);
      b(i, i + 2) = ca / h4; b(i, i + 3) = cb / (6 * h4);
    }
    for (long i : {2L, N - 3}) {
      a(i, i - 1) = 0.25; a(i, i) = 1.0; a(i, i + 1) = 0.25;
      b(i, i - 2) = 1.5 / h4; b(i, i - 1) = -4 * 1.5 / h4; b(i, i) = 6 * 1.5 / h4; b(i, i + 1) = -4 * 1.5 / h4;
      b(i, i + 2) = 1.5 / h4;
    }
    const double r1[5] = {6.0, -24.0, 36.0, -24.0, 6.0};
    a(1, 0) = 1.0; a(1, 1) = -2.0; a(1, 2) = 7.0;
    for (int c = 0; c < 5; ++c) b(1, c) = r1[c] / h4;
    a(N - 2, N - 1) = 1.0; a(N - 2, N - 2) = -2.0; a(N - 2, N - 3) = 7.0;
    for (int c = 0; c < 5; ++c) b(N - 2, N - 1 - c) = r1[c] / h4;
    const double r0[5] = {-1.0, 4.0, -6.0, 4.0, -1.0};
    a(0, 0) = 1.0; a(0, 1) = -2.0;
    for (int c = 0; c < 5; ++c) b(0, c) = r0[c] / h4;
    a(N - 1, N - 1) = 1.0; a(N - 1, N - 2) = -2.0;
    for (int c = 0; c < 5; ++c) b(N - 1, N - 1 - c) = r0[c] / h4;
  }
}

struct Port {
  // parameters
  double dt = 0, dkx = 0, dkz = 0, alpha = 0, nu = 0;
  long NX = 0, NY = 0, NZ = 0, NXH = 0, NZH = 0, NX2 = 0, NZ2 = 0;
  // grid, metric, wavenumbers
  std::vector<double> kx, kz, y, s, dyds[4];
  std::map<std::string, std::vector<double>> cvec_r;  // c11..c44
  double ds = 0;
  Dense DY[4];
  Dense Amean;  // solve_mean's matrix, factored once (it is constant)
  std::vector<int> Amean_piv;
  // fields [z][x][y]
  std::map<std::string, std::vector<cplx>> F;
  std::map<std::string, std::vector<cplx>> V;  // mean-mode vectors
  std::map<std::string, double> S;
  CpuFft fzb, fzf, fxb, fxf;
  // wall blowing/suction [z][x]: the values the v boundary rows take in place
  // of the reference's zeros (solver.cpp:593-596); empty = no-slip
  std::vector<cplx> vw_bot, vw_top;

  size_t nfield() const { return (size_t)NZ * NXH * NY; }
  cplx *f(const std::string &n) { return F.at(n).data(); }
  cplx *line(const std::string &n, long k, long i) { return F.at(n).data() + ((size_t)k * NXH + i) * NY; }

  void init(double dt_, double dkx_, double dkz_, long nx, long ny, long nz, double al, double nu_) {
    dt = dt_; dkx = dkx_; dkz = dkz_; NX = nx; NY = ny; NZ = nz; alpha = al; nu = nu_;
    vw_bot.clear();  // a wall velocity belongs to one grid: no-slip after init
    vw_top.clear();
    if (NY < 7) throw std::invalid_argument("N must be at least 7 for 3rd derivative scheme");
    NXH = NX / 2; NZH = NZ / 2; NX2 = NX / 2 * 3; NZ2 = NZ / 2 * 3;
    // wavenumbers (solver.cpp:25-37), one rank
    kx.assign(NXH, 0.0);
    kz.assign(NZ, 0.0);
    for (long i = 0; i < NXH; ++i) kx[i] = (double)i * dkx;
    for (long k = 0; k < NZ; ++k) {
      double t = (double)k;
      if (t >= (double)NZH) t -= (double)NZ;
      kz[k] = t * dkz;
    }
    // stretched grid and analytic metric derivatives (solver.cpp:57-81)
    s.assign(NY, 0); y.assign(NY, 0);
    for (auto &d : dyds) d.assign(NY, 0);
    ds = 2.0 / (NY - 1.0);
    const double ap = alpha, ap2 = std::pow(alpha, 2), ap3 = std::pow(alpha, 3), ap4 = std::pow(alpha, 4);
    const double coth_ap = 1.0 / std::tanh(ap);
    for (long i = 0; i < NY; ++i) {
      s[i] = 2 * i / (NY - 1.0) - 1.0;
      const double as = ap * s[i];
      const double sech = 1.0 / std::cosh(as);
      y[i] = std::tanh(as) / std::tanh(ap);
      dyds[0][i] = ap * coth_ap * std::pow(sech, 2);
      dyds[1][i] = -2 * ap2 * coth_ap * std::pow(sech, 2) * std::tanh(as);
      dyds[2][i] = 2 * ap3 * (-2 + std::cosh(2 * as)) * coth_ap * std::pow(sech, 4);
      dyds[3][i] = -2 * ap4 * coth_ap * std::pow(sech, 5) * (-11 * std::sinh(as) + std::sinh(3 * as));
    }
    // chain-rule coefficients (solver.cpp:94-106)
    auto P = [&](int q, int e) { std::vector<double> r(NY); for (long i = 0; i < NY; ++i) r[i] = std::pow(dyds[q][i], (double)e); return r; };
    std::vector<double> d1m1 = P(0, -1), d1m2 = P(0, -2), d1m3 = P(0, -3), d1m4 = P(0, -4), d1m5 = P(0, -5),
                        d1m6 = P(0, -6), d1m7 = P(0, -7), d2p2 = P(1, 2), d2p3 = P(1, 3);
    std::vector<double> c11(NY), c21(NY), c22(NY), c31(NY), c32(NY), c33(NY), c41(NY), c42(NY), c43(NY), c44(NY);
    for (long i = 0; i < NY; ++i) {
      const double d2 = dyds[1][i], d3 = dyds[2][i], d4 = dyds[3][i];
      c11[i] = d1m1[i];
      c21[i] = -d2 * d1m3[i];
      c22[i] = d1m2[i];
      c31[i] = -d3 * d1m4[i] + 3.0 * d2p2[i] * d1m5[i];
      c32[i] = -3.0 * d2 * d1m4[i];
      c33[i] = d1m3[i];
      c41[i] = -d4 * d1m5[i] + 10.0 * d3 * d2 * d1m6[i] - 15.0 * d2p3[i] * d1m7[i];
      c42[i] = -4.0 * d3 * d1m5[i] + 15.0 * d2p2[i] * d1m6[i];
      c43[i] = -6.0 * d2 * d1m5[i];
      c44[i] = d1m4[i];
    }
    cvec_r = {{"c11", c11}, {"c21", c21}, {"c22", c22}, {"c31", c31}, {"c32", c32}, {"c33", c33},
              {"c41", c41}, {"c42", c42}, {"c43", c43}, {"c44", c44}};
    // D_n = A_n^-1 B_n, DYn as in init_mat (solver.cpp:171-216)
    Dense A[4], B[4], D[4];
    stencils(NY, ds, A, B);
    for (int q = 0; q < 4; ++q) {
      Dense lu = A[q];
      std::vector<int> piv;
      lu_factor(lu, piv);
      D[q] = Dense(NY);
      std::vector<double> col(NY);
      for (long c = 0; c < NY; ++c) {
        for (long r = 0; r < NY; ++r) col[r] = B[q](r, c);
        lu_solve(lu, piv, col.data());
        for (long r = 0; r < NY; ++r) D[q](r, c) = col[r];
      }
    }
    for (int q = 0; q < 4; ++q) DY[q] = Dense(NY);
    for (long i = 0; i < NY; ++i)
      for (long j = 0; j < NY; ++j) {
        DY[0](i, j) = c11[i] * D[0](i, j);
        DY[1](i, j) = c21[i] * D[0](i, j) + c22[i] * D[1](i, j);
        DY[2](i, j) = c31[i] * D[0](i, j) + c32[i] * D[1](i, j) + c33[i] * D[2](i, j);
        DY[3](i, j) = c41[i] * D[0](i, j) + c42[i] * D[1](i, j) + c43[i] * D[2](i, j) + c44[i] * D[3](i, j);
      }
    // solve_mean's matrix (solver.cpp:448-476) is constant: factor it once.
    const double g0 = 11.0 / 6.0;
    Amean = Dense(NY);
    for (long i = 0; i < NY; ++i)
      for (long j = 0; j < NY; ++j) Amean(i, j) = -nu * DY[1](i, j) + (i == j ? g0 / dt : 0.0);
    for (long j = 0; j < NY; ++j) { Amean(0, j) = 0.0; Amean(NY - 1, j) = 0.0; }
    Amean(0, 0) = 1.0; Amean(NY - 1, NY - 1) = 1.0;
    lu_factor(Amean, Amean_piv);
    // fields
    F.clear(); V.clear(); S.clear();
    for (const char *n : {"velx", "vely", "velz", "vorx", "vory", "vorz", "lmbx", "lmby", "lmbz", "Hv", "Hg",
                          "vely_0", "vely_1", "vely_2", "vory_0", "vory_1", "vory_2", "Hv_0", "Hv_1", "Hv_2",
                          "Hg_0", "Hg_1", "Hg_2"})
      F[n].assign(nfield(), cplx(0.0, 0.0));
    for (const char *n : {"lmbx_mean_0", "lmbx_mean_1", "lmbx_mean_2", "lmbz_mean_0", "lmbz_mean_1", "lmbz_mean_2",
                          "velx_mean_0", "velx_mean_1", "velx_mean_2", "velz_mean_0", "velz_mean_1", "velz_mean_2"})
      V[n].assign(NY, cplx(0.0, 0.0));
    for (const char *n : {"fx_fric", "fz_fric", "fx_fric_0", "fx_fric_1", "fx_fric_2", "fz_fric_0", "fz_fric_1",
                          "fz_fric_2"})
      S[n] = 0.0;
    fzb = CpuFft((int)NZ2, +1); fzf = CpuFft((int)NZ2, -1);
    fxb = CpuFft((int)NX2, +1); fxf = CpuFft((int)NX2, -1);
  }

  // ---- transforms (FFT.cpp:49-194), physical layout [z2][x2][y] ------------
  void fourier2physical(const cplx *u, double *up) {
    std::vector<cplx> zt((size_t)NZ2 * NXH * NY);
#pragma omp parallel
    {
      std::vector<cplx> a(NZ2), b(NZ2), w(NZ2);
#pragma omp for collapse(2) schedule(static)
      for (long i = 0; i < NXH; ++i)
        for (long j = 0; j < NY; ++j) {
          std::fill(a.begin(), a.end(), cplx(0.0, 0.0));
          for (long k = 0; k < NZH; ++k) {
            a[k] = u[((size_t)k * NXH + i) * NY + j];
            a[k + NZ] = u[((size_t)(k + NZH) * NXH + i) * NY + j];
          }
          a[NZ] = 0.0;  // Nyquist (-NZH) dropped on the way to physical space
          fzb.exec(a.data(), b.data(), w.data());
          for (long k = 0; k < NZ2; ++k) zt[((size_t)k * NXH + i) * NY + j] = b[k];
        }
    }
#pragma omp parallel
    {
      std::vector<cplx> a(NX2), b(NX2), w(NX2);
#pragma omp for collapse(2) schedule(static)
      for (long j = 0; j < NY; ++j)
        for (long k = 0; k < NZ2; ++k) {
          std::fill(a.begin(), a.end(), cplx(0.0, 0.0));
          for (long i = 0; i < NXH; ++i) {
            a[i] = zt[((size_t)k * NXH + i) * NY + j];
            if (i > 0) a[i + NX] = std::conj(zt[((size_t)k * NXH + (NXH - i)) * NY + j]);
          }
          fxb.exec(a.data(), b.data(), w.data());
          for (long i = 0; i < NX2; ++i) up[((size_t)k * NX2 + i) * NY + j] = b[i].real();
        }
    }
  }
  void physical2fourier(const double *up, cplx *u) {
    std::vector<cplx> xt((size_t)NZ2 * NXH * NY);
#pragma omp parallel
    {
      std::vector<cplx> a(NX2), b(NX2), w(NX2);
#pragma omp for collapse(2) schedule(static)
      for (long k = 0; k < NZ2; ++k)
        for (long j = 0; j < NY; ++j) {
          for (long i = 0; i < NX2; ++i) a[i] = cplx(up[((size_t)k * NX2 + i) * NY + j], 0.0);
          fxf.exec(a.data(), b.data(), w.data());
          for (long i = 0; i < NXH; ++i) xt[((size_t)k * NXH + i) * NY + j] = b[i] / (double)NX2;
        }
    }
#pragma omp parallel
    {
      std::vector<cplx> a(NZ2), b(NZ2), w(NZ2);
#pragma omp for collapse(2) schedule(static)
      for (long i = 0; i < NXH; ++i)
        for (long j = 0; j < NY; ++j) {
          for (long k = 0; k < NZ2; ++k) a[k] = xt[((size_t)k * NXH + i) * NY + j];
          fzf.exec(a.data(), b.data(), w.data());
          for (long k = 0; k < NZH; ++k) {
            u[((size_t)k * NXH + i) * NY + j] = b[k] / (double)NZ2;
            u[((size_t)(k + NZH) * NXH + i) * NY + j] = b[k + NZ] / (double)NZ2;
          }
        }
    }
  }

  // ---- physics --------------------------------------------------------------
  void get_vor_from_vel() {
#pragma omp parallel
    {
      std::vector<cplx> t(NY);
#pragma omp for collapse(2) schedule(static)
      for (long k = 0; k < NZ; ++k)
        for (long i = 0; i < NXH; ++i) {
          const double kxv = kx[i], kzv = kz[k];
          cplx *u = line("velx", k, i), *v = line("vely", k, i), *w = line("velz", k, i);
          cplx *ox = line("vorx", k, i), *oy = line("vory", k, i), *oz = line("vorz", k, i);
          matvec(DY[0], w, t.data());
          for (long j = 0; j < NY; ++j) ox[j] = t[j] - I1 * kzv * v[j];
          for (long j = 0; j < NY; ++j) oy[j] = I1 * kzv * u[j] - I1 * kxv * w[j];
          matvec(DY[0], u, t.data());
          for (long j = 0; j < NY; ++j) oz[j] = I1 * kxv * v[j] - t[j];
        }
    }
  }
  void nonlinear_source() {
#pragma omp parallel
    {
      std::vector<cplx> t(NY), d(NY);
#pragma omp for collapse(2) schedule(static)
      for (long k = 0; k < NZ; ++k)
        for (long i = 0; i < NXH; ++i) {
          const double kzv = kz[k], kxv = kx[i], k2 = std::pow(kxv, 2) + std::pow(kzv, 2);
          cplx *lx = line("lmbx", k, i), *ly = line("lmby", k, i), *lz = line("lmbz", k, i);
          cplx *hv = line("Hv", k, i), *hg = line("Hg", k, i);
          for (long j = 0; j < NY; ++j) t[j] = I1 * kxv * lx[j] + I1 * kzv * lz[j];
          matvec(DY[0], t.data(), d.data());
          for (long j = 0; j < NY; ++j) hv[j] = -k2 * ly[j] - d[j];
          for (long j = 0; j < NY; ++j) hg[j] = I1 * kzv * lx[j] - I1 * kxv * lz[j];
        }
    }
  }
  void lamb_vec() {
    const size_t np = (size_t)NZ2 * NX2 * NY;
    std::vector<double> p[6];
    const char *src[6] = {"velx", "vely", "velz", "vorx", "vory", "vorz"};
    for (int q = 0; q < 6; ++q) { p[q].resize(np); fourier2physical(f(src[q]), p[q].data()); }
    std::vector<double> lx(np), ly(np), lz(np);
    const double *u = p[0].data(), *v = p[1].data(), *w = p[2].data();
    const double *ox = p[3].data(), *oy = p[4].data(), *oz = p[5].data();
#pragma omp parallel for schedule(static)
    for (size_t n = 0; n < np; ++n) {
      lx[n] = v[n] * oz[n] - w[n] * oy[n];
      ly[n] = w[n] * ox[n] - u[n] * oz[n];
      lz[n] = u[n] * oy[n] - v[n] * ox[n];
    }
    physical2fourier(lx.data(), f("lmbx"));
    physical2fourier(ly.data(), f("lmby"));
    physical2fourier(lz.data(), f("lmbz"));
    V["lmbx_mean_2"] = V["lmbx_mean_1"]; V["lmbx_mean_1"] = V["lmbx_mean_0"];
    V["lmbx_mean_0"].assign(line("lmbx", 0, 0), line("lmbx", 0, 0) + NY);
    V["lmbz_mean_2"] = V["lmbz_mean_1"]; V["lmbz_mean_1"] = V["lmbz_mean_0"];
    V["lmbz_mean_0"].assign(line("lmbz", 0, 0), line("lmbz", 0, 0) + NY);
  }
  void solve_friction_force() {
    std::vector<cplx> du(NY), dw(NY);
    matvec(DY[0], line("velx", 0, 0), du.data());
    matvec(DY[0], line("velz", 0, 0), dw.data());
    const double Ly = y[NY - 1] - y[0];
    S["fx_fric"] = -nu / Ly * (du[NY - 1].real() - du[0].real());
    S["fz_fric"] = -nu / Ly * (dw[NY - 1].real() - dw[0].real());
    S["fx_fric_2"] = S["fx_fric_1"]; S["fx_fric_1"] = S["fx_fric_0"]; S["fx_fric_0"] = S["fx_fric"];
    S["fz_fric_2"] = S["fz_fric_1"]; S["fz_fric_1"] = S["fz_fric_0"]; S["fz_fric_0"] = S["fz_fric"];
  }
  void solve_mean() {
    const double a0 = 3.0, a1 = -1.5, a2 = 1.0 / 3.0, b0 = 3.0, b1 = -3.0, b2 = 1.0;
    std::vector<cplx> su(NY), sw(NY);
    const cplx *lx0 = V["lmbx_mean_0"].data(), *lx1 = V["lmbx_mean_1"].data(), *lx2 = V["lmbx_mean_2"].data();
    const cplx *lz0 = V["lmbz_mean_0"].data(), *lz1 = V["lmbz_mean_1"].data(), *lz2 = V["lmbz_mean_2"].data();
    const cplx *u0 = V["velx_mean_0"].data(), *u1 = V["velx_mean_1"].data(), *u2 = V["velx_mean_2"].data();
    const cplx *w0 = V["velz_mean_0"].data(), *w1 = V["velz_mean_1"].data(), *w2 = V["velz_mean_2"].data();
    for (long j = 0; j < NY; ++j) {
      su[j] = b0 * (lx0[j] + S["fx_fric_0"]) + b1 * (lx1[j] + S["fx_fric_1"]) + b2 * (lx2[j] + S["fx_fric_2"]);
      su[j] = su[j] + (a0 * u0[j] + a1 * u1[j] + a2 * u2[j]) / dt;
      sw[j] = b0 * (lz0[j] + S["fz_fric_0"]) + b1 * (lz1[j] + S["fz_fric_1"]) + b2 * (lz2[j] + S["fz_fric_2"]);
      sw[j] = sw[j] + (a0 * w0[j] + a1 * w1[j] + a2 * w2[j]) / dt;
    }
    su[0] = 0.0; su[NY - 1] = 0.0; sw[0] = 0.0; sw[NY - 1] = 0.0;
    lu_solve(Amean, Amean_piv, su.data());
    lu_solve(Amean, Amean_piv, sw.data());
    std::copy(su.begin(), su.end(), line("velx", 0, 0));
    std::copy(sw.begin(), sw.end(), line("velz", 0, 0));
    V["velx_mean_2"] = V["velx_mean_1"]; V["velx_mean_1"] = V["velx_mean_0"]; V["velx_mean_0"] = su;
    V["velz_mean_2"] = V["velz_mean_1"]; V["velz_mean_1"] = V["velz_mean_0"]; V["velz_mean_0"] = sw;
    solve_friction_force();
    std::vector<cplx> t(NY);
    matvec(DY[0], line("velz", 0, 0), line("vorx", 0, 0));
    matvec(DY[0], line("velx", 0, 0), t.data());
    for (long j = 0; j < NY; ++j) line("vorz", 0, 0)[j] = -t[j];
  }
  void solve_horizontal() {
#pragma omp parallel
    {
      std::vector<cplx> d1v(NY), d2v(NY), d1g(NY);
#pragma omp for collapse(2) schedule(static)
      for (long k = 0; k < NZ; ++k)
        for (long i = 0; i < NXH; ++i) {
          const double kxv = kx[i], kzv = kz[k], k2 = std::pow(kxv, 2) + std::pow(kzv, 2);
          if (k2 < 1.e-8) continue;  // the mean mode is handled by solve_mean below
          cplx *v = line("vely", k, i), *g = line("vory", k, i);
          matvec(DY[0], v, d1v.data());
          matvec(DY[1], v, d2v.data());
          matvec(DY[0], g, d1g.data());
          cplx *u = line("velx", k, i), *w = line("velz", k, i), *ox = line("vorx", k, i), *oz = line("vorz", k, i);
          for (long j = 0; j < NY; ++j) {
            u[j] = I1 * kxv / k2 * d1v[j] - I1 * kzv / k2 * g[j];
            w[j] = I1 * kxv / k2 * g[j] + I1 * kzv / k2 * d1v[j];
            ox[j] = I1 / k2 * (kxv * d1g[j] + kzv * d2v[j] - kzv * k2 * v[j]);
            oz[j] = I1 / k2 * (kzv * d1g[j] - kxv * d2v[j] + kxv * k2 * v[j]);
          }
        }
    }
    solve_mean();
  }
  // One slice of the mode loop (solver.cpp:561-605): modes with flat index
  // m = k*NXH + i in [m0, m1) stepping by stride.
  void mode_loop(long m0, long m1, long stride) {
    const double g0 = 11.0 / 6.0, a0 = 3.0, a1 = -1.5, a2 = 1.0 / 3.0, b0 = 3.0, b1 = -3.0, b2 = 1.0;
    const long N = NY;
#pragma omp parallel
    {
      Dense Av(N), Ag(N);
      std::vector<int> pv, pg;
      std::vector<cplx> sv(N), sg(N), vs(N), d2(N);
#pragma omp for schedule(dynamic, 4)
      for (long m = m0; m < m1; m += stride) {
        const long k = m / NXH, i = m % NXH;
        const double k2 = std::pow(kx[i], 2) + std::pow(kz[k], 2), k4 = std::pow(k2, 2);
        const cplx *h0 = line("Hv_0", k, i), *h1 = line("Hv_1", k, i), *h2 = line("Hv_2", k, i);
        const cplx *v0 = line("vely_0", k, i), *v1 = line("vely_1", k, i), *v2 = line("vely_2", k, i);
        const cplx *q0 = line("Hg_0", k, i), *q1 = line("Hg_1", k, i), *q2 = line("Hg_2", k, i);
        const cplx *g0p = line("vory_0", k, i), *g1p = line("vory_1", k, i), *g2p = line("vory_2", k, i);
        for (long j = 0; j < N; ++j) vs[j] = v0[j] * a0 + v1[j] * a1 + v2[j] * a2;
        matvec(DY[1], vs.data(), d2.data());
        for (long j = 0; j < N; ++j) {
          sv[j] = h0[j] * b0 + h1[j] * b1 + h2[j] * b2;
          sv[j] = sv[j] - (k2 / dt) * vs[j];
          sv[j] = sv[j] + d2[j] / dt;
          sg[j] = q0[j] * b0 + q1[j] * b1 + q2[j] * b2;
          sg[j] = sg[j] + (g0p[j] * a0 + g1p[j] * a1 + g2p[j] * a2) / dt;
        }
        const double ca = g0 / dt + 2 * nu * k2, cb = nu * k4 + g0 * k2 / dt, cg = nu * k2 + g0 / dt;
        for (long r = 0; r < N; ++r)
          for (long c = 0; c < N; ++c) {
            Av(r, c) = -nu * DY[3](r, c) + ca * DY[1](r, c) - (r == c ? cb : 0.0);
            Ag(r, c) = -nu * DY[1](r, c) + (r == c ? cg : 0.0);
          }
        // boundary rows (solver.cpp:581-599)
        for (long c = 0; c < N; ++c) {
          Av(0, c) = 0.0; Av(1, c) = DY[0](0, c); Av(N - 2, c) = DY[0](N - 1, c); Av(N - 1, c) = 0.0;
          Ag(0, c) = 0.0; Ag(N - 1, c) = 0.0;
        }
        Av(0, 0) = 1.0; Av(N - 1, N - 1) = 1.0; Ag(0, 0) = 1.0; Ag(N - 1, N - 1) = 1.0;
        sv[0] = 0.0; sv[1] = 0.0; sv[N - 2] = 0.0; sv[N - 1] = 0.0;
        if (!vw_bot.empty()) { sv[0] = vw_bot.at(m); sv[N - 1] = vw_top.at(m); }
        sg[0] = 0.0; sg[N - 1] = 0.0;
        lu_factor(Av, pv);
        lu_solve(Av, pv, sv.data());
        lu_factor(Ag, pg);
        lu_solve(Ag, pg, sg.data());
        std::copy(sv.begin(), sv.end(), line("vely", k, i));
        std::copy(sg.begin(), sg.end(), line("vory", k, i));
      }
    }
  }
  void rotate_history() {
    for (const char *b : {"vely", "vory", "Hv", "Hg"}) {
      std::string n(b);
      std::swap(F[n + "_2"], F[n + "_1"]);
      std::swap(F[n + "_1"], F[n + "_0"]);
      F[n + "_0"] = F[n];
    }
  }
  void time_integration() {
    mode_loop(0, NZ * NXH, 1);
    solve_horizontal();
    lamb_vec();
    nonlinear_source();
    rotate_history();
  }
  void startup() {
    get_vor_from_vel();
    lamb_vec();
    nonlinear_source();
    for (const char *b : {"vely", "vory", "Hv", "Hg"}) {
      std::string n(b);
      F[n + "_0"] = F[n]; F[n + "_1"] = F[n]; F[n + "_2"] = F[n];
    }
    solve_friction_force();
    for (const char *n : {"fx_fric", "fz_fric"}) {
      std::string b(n);
      S[b + "_0"] = S[b]; S[b + "_1"] = S[b]; S[b + "_2"] = S[b];
    }
    for (const char *pair : {"velx", "velz", "lmbx", "lmbz"}) {
      std::string b(pair);
      std::vector<cplx> m(line(b, 0, 0), line(b, 0, 0) + NY);
      V[b + "_mean_0"] = m; V[b + "_mean_1"] = m; V[b + "_mean_2"] = m;
    }
  }
  // The reference's built-in initial condition (solver.cpp:336-377).
  void builtin_ic() {
    for (long j = 0; j < NY; ++j) line("velx", 0, 0)[j] = cplx(1.5 * (1 - std::pow(y[j], 2)), 0.0);
    const double k1 = 2.0, k2 = 2.0, al = 1.0;
    for (long k = 0; k < NZ; ++k)
      for (long i = 0; i < NXH; ++i)
        for (long j = 0; j < NY; ++j) {
          const double yy = y[j];
          if (kz[k] == k2 && kx[i] == k1) {
            line("velx", k, i)[j] += al / k1 * (yy - std::pow(yy, 3)) * (-0.25 * I1);
            line("vely", k, i)[j] += al * (0.5 * std::pow(yy, 2) - 0.25 * std::pow(yy, 4) - 0.25) * (0.25);
            line("velz", k, i)[j] += -2 * al / k2 * (yy - std::pow(yy, 3)) * (-0.25 * I1);
          }
          if (kz[k] == -k2 && kx[i] == k1) {
            line("velx", k, i)[j] += al / k1 * (yy - std::pow(yy, 3)) * (-0.25 * I1);
            line("vely", k, i)[j] += al * (0.5 * std::pow(yy, 2) - 0.25 * std::pow(yy, 4) - 0.25) * (0.25);
            line("velz", k, i)[j] += -2 * al / k2 * (yy - std::pow(yy, 3)) * (0.25 * I1);
          }
        }
  }
};

Port g_port;

void copy_in(std::vector<cplx> &dst, const double *src) {
  std::memcpy(dst.data(), src, dst.size() * sizeof(cplx));
}
void copy_out(const std::vector<cplx> &src, double *dst) {
  std::memcpy(dst, src.data(), src.size() * sizeof(cplx));
}

template <typename F>
int guarded(F &&f) {
  try { f(); return 0; } catch (const std::exception &) { return 1; }
}

}  // namespace

extern "C" {

int port_set_fd_order(int order) {
  if (order != 6 && order != 8) return 1;
  g_fd_order = order;
  return 0;
}
int port_get_stencil(int which, double *a, double *b) {
  return guarded([&] {
    if (which < 1 || which > 4) throw std::invalid_argument("stencil index");
    Dense A[4], B[4];
    stencils(g_port.NY, g_port.ds, A, B);
    std::memcpy(a, A[which - 1].a.data(), A[which - 1].a.size() * sizeof(double));
    std::memcpy(b, B[which - 1].a.data(), B[which - 1].a.size() * sizeof(double));
  });
}
int port_set_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
}
int port_init(double dt, double dkx, double dkz, long nx, long ny, long nz, double alpha, double nu) {
  return guarded([&] { g_port.init(dt, dkx, dkz, nx, ny, nz, alpha, nu); });
}
int port_init_fields_builtin() {
  return guarded([&] { g_port.builtin_ic(); g_port.startup(); });
}
int port_set_velocity(const double *u, const double *v, const double *w) {
  return guarded([&] {
    copy_in(g_port.F.at("velx"), u); copy_in(g_port.F.at("vely"), v); copy_in(g_port.F.at("velz"), w);
    g_port.startup();
  });
}
int port_step(int n) {
  return guarded([&] { for (int i = 0; i < n; ++i) g_port.time_integration(); });
}
int port_call(const char *name) {
  return guarded([&] {
    std::string s(name);
    if (s == "get_vor_from_vel") g_port.get_vor_from_vel();
    else if (s == "solve_horizontal") g_port.solve_horizontal();
    else if (s == "Lamb_vec") g_port.lamb_vec();
    else if (s == "nonlinear_source") g_port.nonlinear_source();
    else if (s == "solve_friction_force") g_port.solve_friction_force();
    else if (s == "time_Integration") g_port.time_integration();
    else throw std::invalid_argument(s);
  });
}
int port_set_wall_velocity(const double *bottom, const double *top) {
  return guarded([&] {
    const size_t n = (size_t)g_port.NZ * g_port.NXH;
    if (!bottom || !top) { g_port.vw_bot.clear(); g_port.vw_top.clear(); return; }
    g_port.vw_bot.assign(reinterpret_cast<const cplx *>(bottom), reinterpret_cast<const cplx *>(bottom) + n);
    g_port.vw_top.assign(reinterpret_cast<const cplx *>(top), reinterpret_cast<const cplx *>(top) + n);
  });
}
int port_get_field(const char *name, double *out) {
  return guarded([&] { copy_out(g_port.F.at(name), out); });
}
int port_set_field(const char *name, const double *in) {
  return guarded([&] { copy_in(g_port.F.at(name), in); });
}
int port_get_cvec(const char *name, double *out) {
  return guarded([&] { copy_out(g_port.V.at(name), out); });
}
int port_set_cvec(const char *name, const double *in) {
  return guarded([&] { copy_in(g_port.V.at(name), in); });
}
int port_get_rvec(const char *name, double *out) {
  return guarded([&] {
    std::string s(name);
    const std::vector<double> *v = nullptr;
    if (s == "y") v = &g_port.y;
    else if (s == "s") v = &g_port.s;
    else if (s == "kx_local") v = &g_port.kx;
    else if (s == "kz_local") v = &g_port.kz;
    else if (s.rfind("dyds", 0) == 0) v = &g_port.dyds[s[4] - '1'];
    else v = &g_port.cvec_r.at(s);
    std::memcpy(out, v->data(), v->size() * sizeof(double));
  });
}
int port_get_scalar(const char *name, double *out) {
  return guarded([&] {
    if (std::string(name) == "ds") *out = g_port.ds;
    else *out = g_port.S.at(name);
  });
}
int port_set_scalar(const char *name, double val) {
  return guarded([&] { g_port.S.at(name) = val; });
}
int port_get_dy(int which, double *out) {
  return guarded([&] {
    if (which < 1 || which > 4) throw std::invalid_argument("DY index");
    std::memcpy(out, g_port.DY[which - 1].a.data(), g_port.DY[which - 1].a.size() * sizeof(double));
  });
}
int port_fourier2physical(const double *in, double *out) {
  return guarded([&] { g_port.fourier2physical(reinterpret_cast<const cplx *>(in), out); });
}
int port_physical2fourier(const double *in, double *out) {
  return guarded([&] { g_port.physical2fourier(in, reinterpret_cast<cplx *>(out)); });
}
// Wall-clock seconds of the mode loop over every `stride`-th mode, `reps`
// times (a bounded sample of one step's dominant stage).
double port_time_modes(long stride, long reps) {
  auto t0 = std::chrono::steady_clock::now();
  for (long r = 0; r < reps; ++r) g_port.mode_loop(0, g_port.NZ * g_port.NXH, stride);
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}
// Wall-clock seconds of `nfields` inverse and nfields/2 forward transforms.
double port_time_transforms(long nfields) {
  const size_t np = (size_t)g_port.NZ2 * g_port.NX2 * g_port.NY;
  std::vector<double> p(np);
  auto t0 = std::chrono::steady_clock::now();
  for (long q = 0; q < nfields; ++q) g_port.fourier2physical(g_port.f("velx"), p.data());
  for (long q = 0; q < nfields / 2; ++q) g_port.physical2fourier(p.data(), g_port.f("lmbx"));
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}
}

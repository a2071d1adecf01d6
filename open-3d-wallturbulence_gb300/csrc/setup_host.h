// Host-side setup of the wall-normal discretisation for the GPU time step.
//
// Everything here is computed once per handle on the host in FP64 and then
// uploaded: the stretched grid and metric (reference src/solver.cpp:57-106),
// the compact finite-difference stencils (src/compdiff.hpp:11-357, as coded),
// and the banded "augmented" forms of the two per-mode implicit systems.
//
// Augmented systems.  The reference solves, for every Fourier mode, the dense
// systems Av v = r and Ag g = r (src/solver.cpp:577-603) whose matrices are
// built from DYn = sum_m diag(c_nm) A_m^-1 B_m.  The same equations are banded
// when the compact derivatives d_m = A_m^-1 B_m v are kept as unknowns:
//
//   v-system, unknowns (v, d1, d2, d3) per node and d4 at nodes 0, 1, N-2,
//   N-1 only.  With G = (a c21 - nu c41, a c22 - nu c42, -nu c43, -nu c44)
//   (a, b as in solver.cpp:577) the interior equation of node m (2..N-3)
//     G1 d1 + G2 d2 + G3 d3 + G4 d4 - b v = r
//   gives d4_m = (r_m + b v_m - G1 d1_m - G2 d2_m - G3 d3_m) / G4_m, which is
//   substituted into the fourth-derivative rows, so d4 leaves the interior:
//     A_m d_m - B_m v = 0                                  (m = 1..3, all rows)
//     sum_m A4[j,m] d4_m - B_4 v = 0 with d4_m substituted where it can be
//                            (right-hand side -sum_m A4[j,m] r_m / G4_m)
//     v_0 = 0, c11_0 d1_0 = 0, c11_N-1 d1_N-1 = 0, v_N-1 = 0   (solver.cpp:581-596)
//   4N + 4 unknowns instead of 5N, and less fill after pivoting.
//
//   omega_y-system, reduced to 2 unknowns per node (d1, d2): with
//   g_j = (r_j + nu c21_j d1_j + nu c22_j d2_j) / cg on interior nodes and
//   g = 0 at the walls (solver.cpp:578, 588-599), cg = nu k^2 + gamma0/dt,
//     A_m d_m - B_m g(d) = 0    (m = 1, 2)   i.e.   A_m d_m - (1/cg) B_m G d = (1/cg) B_m r
//
// The mean-mode solve of solve_mean (src/solver.cpp:448-485) is the
// omega_y-system at k = 0, so it reuses that factorization.
//
// Scaling.  The unknown d_t (t-th derivative) is solved for as h^t d_t, and
// every row is divided by its largest coefficient when a mode's matrix is
// assembled (the inverse scales of rows carrying a right-hand side are kept).
// Partial pivoting then compares like with like; without it the stencil rows
// (coefficients ~1) are satisfied only to the round-off of the ~1e8-sized
// E rows, and DY1 v recomputed from the solved v disagrees with the solved
// d1 at the 1e-10 level instead of 1e-15.
//
// Equations are ordered by the midpoint of their column span (unknowns
// interleaved by node); the resulting band widths are structural constants
// (v-system kl = 15, ku = 16 (kVKL, kVKU); omega_y-system kl = ku = 6) that the CUDA kernels
// take as template parameters.  Band matrices are stored in LAPACK's
// factorization layout (2kl+ku+1 rows, fill rows first) so that a partial-
// pivoting band LU (the algorithm of LAPACK dgbtf2/dgbtrs) runs in place.
#pragma once
#ifndef __CUDACC__
#ifndef __host__
#define __host__
#define __device__
#endif
#endif
#include <cstdint>
#include <string>
#include <vector>

namespace owt {

struct Grid {
  int N = 0;
  double ds = 0;
  std::vector<double> s, y, dyds1, dyds2, dyds3, dyds4;
  std::vector<double> c11, c21, c22, c31, c32, c33, c41, c42, c43, c44;
};

// Dense N x N row-major matrices of the stencils A_n, B_n (n = 1..4).
struct Stencils {
  int N = 0;
  std::vector<double> A[4], B[4];
  double a(int n, int i, int j) const { return A[n][(size_t)i * N + j]; }
  double b(int n, int i, int j) const { return B[n][(size_t)i * N + j]; }
};

// rhs_node tags of the v-system rows: a combination of interior r values
// (kRhsTable), zero (kRhsNone), and the two rows v_0 = v_w(bottom),
// v_N-1 = v_w(top), zero (no-slip, src/solver.cpp:593-596) unless wall
// blowing/suction is set.
constexpr int kRhsTable = 0, kRhsNone = -1, kRhsWallBottom = -2, kRhsWallTop = -3;

// Column of unknown type t at node j in the v-system (types 0..3 = v, h d1,
// h^2 d2, h^3 d3 at every node; type 4 = h^4 d4 only at nodes 0, 1, N-2,
// N-1).  The four nodes at the walls hold their unknowns in type order; the
// interior nodes in reverse (h^3 d3, h^2 d2, h d1, v): with the equations
// sorted by the midpoint of their column spans, partial pivoting then fills
// 78 entries of L and U per interior node instead of 105 (the union over the
// mask derivation's sweep), for band widths 15 below and 16 above the
// diagonal instead of 15 and 13.
constexpr int kVKL = 15, kVKU = 16;
__host__ __device__ inline int vcol(int t, int j, int N) {
  return j < 2 ? 5 * j + t : j < N - 2 ? 10 + 4 * (j - 2) + (3 - t) : 4 * N - 6 + 5 * (j - (N - 2)) + t;
}
__host__ __device__ inline void vcol_split(int c, int N, int &t, int &j) {
  if (c < 10) {
    j = c / 5; t = c - 5 * j;
  } else if (c < 4 * N - 6) {
    const int q = c - 10;
    j = 2 + (q >> 2); t = 3 - (q & 3);
  } else {
    const int q = c - (4 * N - 6);
    j = N - 2 + q / 5; t = q - 5 * (q / 5);
  }
}

// One equation: coefficients on unknown columns, split as
// value(k) = t0 + s1(k) * t1 + s2(k) * t2 with per-mode scalars s1, s2.
struct Entry {
  int col;
  double t0, t1, t2;
};

// A banded system in template form, ordered and ready to be factored per mode.
struct BandTemplate {
  int n = 0;   // unknowns
  int kl = 0, ku = 0;
  int per_node = 0;
  // [(kl+ku+1) x n]: entry (i, j) of the ordered matrix at row ku + i - j.
  std::vector<double> t0, t1, t2;
  // v-system: what feeds the rhs of each row position: kRhsTable (the rbv
  // table below), kRhsNone (zero), kRhsWallBottom / kRhsWallTop (the
  // wall-velocity rows v_0 and v_N-1).
  std::vector<int> rhs_node;
  // v-system: rhs of a kRhsTable row p = sum_e rbv_val[p][e] * r[rbv_col[p][e]]
  std::vector<int> rbv_col;     // [n x 4]
  std::vector<double> rbv_val;  // [n x 4]
  // omega_y-system: rhs of row p = (1/cg) sum_e rb_val[p][e] * r[rb_col[p][e]].
  std::vector<int> rb_col;     // [n x 5]
  std::vector<double> rb_val;  // [n x 5]
};

Grid make_grid(int N, double alpha);
// Compact-FD stencils; order 8 (the reference's interior schemes) or 6
// (sixth-order tridiagonal interior schemes for D1-D3, same boundary rows).
Stencils make_stencils(int N, double h, int order = 8);
BandTemplate build_v_system(const Grid &g, const Stencils &st, double nu);
BandTemplate build_g_system(const Grid &g, const Stencils &st, double nu);
// Band LU (no per-mode scalars) of A_1, shared by every mode for DY1 f; the
// band is at least (min_kl, min_ku) wide (zero diagonals pad narrower stencils).
BandTemplate build_plain_band(const Stencils &st, int which, int min_kl = 2, int min_ku = 2);

// Widen a band template to at least (kl, ku) with zero diagonals, so that a
// narrower stencil set runs in the kernels specialised for the wider band.
void pad_band(BandTemplate &bt, int kl, int ku);

// Twiddle table exp(-2 pi i k / L), k in [0, L), interleaved (re, im).
std::vector<double> twiddles(int L);
// Radix schedule for an FFT of length L = 2^a 3^b (4s first, then 2, then 3s).
bool fft_radices(int L, std::vector<int> &radices);

}  // namespace owt

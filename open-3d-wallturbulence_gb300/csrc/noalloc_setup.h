// The DY1 operator of owt_dy1_noalloc, built in place inside its static
// device array: grid metric c11, the B1 rows and the A1 band, then the band
// LU.  Written as host/device functions so that a host program can build the
// same tables and compare them with setup_host.cpp's make_grid and
// make_stencils (the handle's DY1), which restate src/compdiff.hpp:11-69 and
// src/solver.cpp:77,94.
#pragma once
#include <math.h>
#include <stdint.h>

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#define __device__
#endif
#endif

namespace owt {

// Largest NY the tables are laid out for (the entry point's OWT_NOALLOC_MAX_NY).
constexpr int kNoallocMaxNY = 1025;
constexpr int kNoallocKL = 2, kNoallocKU = 2, kNoallocKV = kNoallocKL + kNoallocKU;
constexpr int kNoallocBandRows = 2 * kNoallocKL + kNoallocKU + 1;

struct NoallocSetup {
  double *ab;    // kNoallocBandRows x NY band, LAPACK factorization layout (row KV = diagonal)
  double *c11;   // NY
  double *bval;  // NY x 5: B1 row entries, zero-padded
  int *bcol;     // NY x 5: their columns
  uint8_t *piv;  // NY: row interchange offset of each column
};

// Fixed offsets for the largest NY, so the layout does not depend on the call.
__host__ __device__ inline NoallocSetup noalloc_layout(unsigned char *base) {
  NoallocSetup s;
  const int nmax = kNoallocMaxNY;
  s.ab = reinterpret_cast<double *>(base);
  s.c11 = s.ab + kNoallocBandRows * nmax;
  s.bval = s.c11 + nmax;
  s.bcol = reinterpret_cast<int *>(s.bval + 5 * nmax);
  s.piv = reinterpret_cast<uint8_t *>(s.bcol + 5 * nmax);
  return s;
}
// Bytes the layout spans.
constexpr size_t noalloc_setup_bytes() {
  return (size_t)kNoallocMaxNY * (kNoallocBandRows + 1 + 5) * sizeof(double) +
         (size_t)kNoallocMaxNY * 5 * sizeof(int) + (size_t)kNoallocMaxNY;
}

// c11 = 1/(dy/ds) on y = tanh(alpha s)/tanh(alpha), the B1 rows and the
// unfactored A1 band (eighth-order interior, fourth-order rows 1 and NY-2,
// third-order closures at the walls).  Everything the derivative kernel reads
// is written, fill rows cleared, so nothing depends on an earlier call.
__host__ __device__ inline void noalloc_assemble(NoallocSetup s, int NY, double alpha) {
  const double h = 2.0 / (NY - 1.0);
  const double coth_ap = 1.0 / tanh(alpha);
  for (int i = 0; i < NY; ++i) {
    const double si = 2 * i / (NY - 1.0) - 1.0;
    const double sech = 1.0 / cosh(alpha * si);
    s.c11[i] = 1.0 / (alpha * coth_ap * sech * sech);
  }
  for (int e = 0; e < 5 * NY; ++e) {
    s.bcol[e] = 0;
    s.bval[e] = 0.0;
  }
  // entries of each row in increasing column order (the handle's B1 row order)
  auto put = [&](int row, int k, int col, double v) {
    s.bcol[row * 5 + k] = col;
    s.bval[row * 5 + k] = v;
  };
  const double a = 40.0 / 27.0, b = 25.0 / 54.0;
  for (int i = 2; i < NY - 2; ++i) {
    put(i, 0, i - 2, -b / (4 * h));
    put(i, 1, i - 1, -a / (2 * h));
    put(i, 2, i + 1, a / (2 * h));
    put(i, 3, i + 2, b / (4 * h));
  }
  for (int q = 0; q < 2; ++q) {
    const int i = q == 0 ? 1 : NY - 2;
    put(i, 0, i - 1, -1.5 / (2 * h));
    put(i, 1, i + 1, 1.5 / (2 * h));
  }
  const double a0 = -17.0 / 6.0, b0 = 1.5, c0 = 1.5, d0 = -1.0 / 6.0;
  put(0, 0, 0, a0 / h);
  put(0, 1, 1, b0 / h);
  put(0, 2, 2, c0 / h);
  put(0, 3, 3, d0 / h);
  put(NY - 1, 0, NY - 4, -d0 / h);
  put(NY - 1, 1, NY - 3, -c0 / h);
  put(NY - 1, 2, NY - 2, -b0 / h);
  put(NY - 1, 3, NY - 1, -a0 / h);
  // A1 band: entry (i, j) at row KV + i - j of column j
  for (int e = 0; e < kNoallocBandRows * NY; ++e) s.ab[e] = 0.0;
  auto A = [&](int i, int j) -> double & { return s.ab[(kNoallocKV + i - j) * NY + j]; };
  for (int i = 2; i < NY - 2; ++i) {
    A(i, i - 2) = 1.0 / 36.0;
    A(i, i - 1) = 4.0 / 9.0;
    A(i, i) = 1.0;
    A(i, i + 1) = 4.0 / 9.0;
    A(i, i + 2) = 1.0 / 36.0;
  }
  for (int q = 0; q < 2; ++q) {
    const int i = q == 0 ? 1 : NY - 2;
    A(i, i - 1) = 0.25;
    A(i, i) = 1.0;
    A(i, i + 1) = 0.25;
  }
  A(0, 0) = 1.0;
  A(0, 1) = 3.0;
  A(NY - 1, NY - 1) = 1.0;
  A(NY - 1, NY - 2) = 3.0;
}

// Band LU with partial pivoting in place, the algorithm of LAPACK dgbtf2 (the
// handle's factorization order); the diagonal row then holds 1/U_jj.
__host__ __device__ inline void noalloc_factor(NoallocSetup s, int NY) {
  constexpr int KL = kNoallocKL, KU = kNoallocKU, KV = kNoallocKV;
  auto AB = [&](int r, int c) -> double & { return s.ab[r * NY + c]; };
  int ju = 0;
  for (int j = 0; j < NY; ++j) {
    const int km = KL < NY - 1 - j ? KL : NY - 1 - j;
    int jp = 0;
    double best = fabs(AB(KV, j));
    for (int i = 1; i <= km; ++i) {
      const double v = fabs(AB(KV + i, j));
      if (v > best) {
        best = v;
        jp = i;
      }
    }
    s.piv[j] = (uint8_t)jp;
    const int reach = j + KU + jp < NY - 1 ? j + KU + jp : NY - 1;
    ju = ju > reach ? ju : reach;
    if (jp != 0)
      for (int c = j; c <= ju; ++c) {
        const double t = AB(KV + jp - (c - j), c);
        AB(KV + jp - (c - j), c) = AB(KV - (c - j), c);
        AB(KV - (c - j), c) = t;
      }
    const double rp = 1.0 / AB(KV, j);
    for (int i = 1; i <= km; ++i) AB(KV + i, j) *= rp;
    for (int c = j + 1; c <= ju; ++c) {
      const double t = AB(KV - (c - j), c);
      if (t != 0.0)
        for (int i = 1; i <= km; ++i) AB(KV + i - (c - j), c) -= AB(KV + i, j) * t;
    }
  }
  for (int j = 0; j < NY; ++j) AB(KV, j) = 1.0 / AB(KV, j);
}

}  // namespace owt

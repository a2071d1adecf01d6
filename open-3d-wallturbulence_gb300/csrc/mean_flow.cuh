// Mixed precision: the interaction of the mean flow with the fluctuations,
// formed mode by mode beside the FP32 transforms (k_mean_lamb) and added to
// the Lamb vector by the z forward kernels.
//
// With the mean split on, the z backward leaves mode (0, 0) of every field
// out of the FP32 transforms, so the product the transforms form is the
// fluctuations' u' x om'.  The rest of u x om (src/solver.cpp:284-286) is
//   Ubar x om' + u' x Obar   at every mode,   Ubar x Obar   at (0, 0),
// with Ubar, Obar the (0, 0) modes of row j (real parts).  A product with a
// function of y alone is a product mode by mode, so these terms need no
// transform: each is a few FP32 products of one mode's values, with an
// error relative to that mode's own value rather than to the largest value
// of the plane, as a transform's would be.  The kx = 0 column enters through
// its Hermitian part (u_k + conj u_-k) / 2, as the real-part extraction of
// the x transform makes it enter the physical product; the Nyquist row
// (kz index NZH) never reaches physical space and gets nothing.
#pragma once
#include <cuda_runtime.h>

#include "owt_device.cuh"
#include "solve_kernels.h"

namespace owt {

// Field q of the step (0..2 velocity, 3..5 vorticity), row j.
__device__ __forceinline__ const double2 *xform_field_row(const XformArgs &a, int q, int j) {
  const double2 *base = a.in[q];
  if (a.ring_mask & (1 << q)) base += (size_t)ring_head(*a.step) * a.fs;
  return base + (size_t)j * a.d.NZ * a.d.NXH;
}

// One thread per mode m of row j (the grid's y; 256-thread blocks along the
// modes), all three components.  Every value is read once and converted by
// d2f_bits (this kernel runs beside the FP32 z backward, whose hardware
// conversions occupy the FP64 pipe); products and sums are explicit FP32
// roundings, so the batched and one-channel kernels give the same bits.
__device__ __forceinline__ void mean_lamb_body(const XformArgs &a, const int bx, const int j) {
  const XformDims d = a.d;
  const int M = d.NZ * d.NXH;
  const int m = bx * 256 + threadIdx.x;
  if (m >= M) return;
  const int kz = m / d.NXH, kx = m - kz * d.NXH;
  const size_t e = (size_t)j * M + m;
  if (kz == d.NZH) {
#pragma unroll
    for (int f = 0; f < 3; ++f) a.lm[f][e] = make_float2(0.f, 0.f);
    return;
  }
  const double2 *row[6];
#pragma unroll
  for (int q = 0; q < 6; ++q) row[q] = xform_field_row(a, q, j);
  float Ub[3], Ob[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    Ub[q] = d2f_bits(row[q][0].x);
    Ob[q] = d2f_bits(row[3 + q][0].x);
  }
  if (m == 0) {
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      const int f1 = (f + 1) % 3, f2 = (f + 2) % 3;
      a.lm[f][e] = make_float2(__fsub_rn(__fmul_rn(Ub[f1], Ob[f2]), __fmul_rn(Ub[f2], Ob[f1])), 0.f);
    }
    return;
  }
  float2 F[6];
  const int mirror = (kz == 0 ? 0 : d.NZ - kz) * d.NXH;
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    const double2 x = row[q][m];
    if (kx != 0) {
      F[q] = make_float2(d2f_bits(x.x), d2f_bits(x.y));
    } else {
      const double2 y = row[q][mirror];
      F[q] = make_float2(__fmul_rn(0.5f, __fadd_rn(d2f_bits(x.x), d2f_bits(y.x))),
                         __fmul_rn(0.5f, __fsub_rn(d2f_bits(x.y), d2f_bits(y.y))));
    }
  }
  // (a x b)_f = a_f1 b_f2 - a_f2 b_f1, linear part in the fluctuations:
  // Ubar_f1 om_f2 - Ubar_f2 om_f1 + u_f1 Obar_f2 - u_f2 Obar_f1
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    const int f1 = (f + 1) % 3, f2 = (f + 2) % 3;
    float2 acc;
    acc.x = __fmul_rn(Ub[f1], F[3 + f2].x);
    acc.y = __fmul_rn(Ub[f1], F[3 + f2].y);
    acc.x = __fmaf_rn(-Ub[f2], F[3 + f1].x, acc.x);
    acc.y = __fmaf_rn(-Ub[f2], F[3 + f1].y, acc.y);
    acc.x = __fmaf_rn(Ob[f2], F[f1].x, acc.x);
    acc.y = __fmaf_rn(Ob[f2], F[f1].y, acc.y);
    acc.x = __fmaf_rn(-Ob[f1], F[f2].x, acc.x);
    acc.y = __fmaf_rn(-Ob[f1], F[f2].y, acc.y);
    a.lm[f][e] = acc;
  }
}

}  // namespace owt

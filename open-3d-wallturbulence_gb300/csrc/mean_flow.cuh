// Mixed precision: the interaction of the mean flow with the fluctuations,
// added to the Lamb vector by the FP32 z forward kernels element by element.
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

// The mean profiles component f of row j needs: with f1 = f + 1, f2 = f + 2
// (mod 3), Ubar_f1, Ubar_f2, Obar_f1, Obar_f2 in FP32.
struct MeanRow {
  int f1, f2;
  float u1, u2, o1, o2;
};

__device__ __forceinline__ MeanRow mean_row(const XformArgs &a, int j, int f) {
  MeanRow r;
  r.f1 = f == 2 ? 0 : f + 1;
  r.f2 = f == 0 ? 2 : f - 1;
  r.u1 = d2f_bits(xform_field_row(a, r.f1, j)[0].x);
  r.u2 = d2f_bits(xform_field_row(a, r.f2, j)[0].x);
  r.o1 = d2f_bits(xform_field_row(a, 3 + r.f1, j)[0].x);
  r.o2 = d2f_bits(xform_field_row(a, 3 + r.f2, j)[0].x);
  return r;
}

// Component f (that of mean_row) of the mean-flow terms at mode (kz, kx) of
// row j.  A term whose mean-profile factor is zero (Vbar and Obar_y always
// are when they start zero, and every profile on a wall row) is skipped with
// its load.
__device__ __forceinline__ float2 mean_term(const XformArgs &a, const MeanRow &r, int j, int kz, int kx) {
  const XformDims d = a.d;
  if (kz == d.NZH) return make_float2(0.f, 0.f);
  if (kz == 0 && kx == 0) return make_float2(__fsub_rn(__fmul_rn(r.u1, r.o2), __fmul_rn(r.u2, r.o1)), 0.f);
  const size_t at = (size_t)kz * d.NXH + kx;
  const size_t mirror = (size_t)(kz == 0 ? 0 : d.NZ - kz) * d.NXH;
  auto F = [&](int q) -> float2 {
    const double2 *row = xform_field_row(a, q, j);
    const double2 x = row[at];
    if (kx != 0) return make_float2(d2f_bits(x.x), d2f_bits(x.y));
    const double2 y = row[mirror];
    return make_float2(__fmul_rn(0.5f, __fadd_rn(d2f_bits(x.x), d2f_bits(y.x))),
                       __fmul_rn(0.5f, __fsub_rn(d2f_bits(x.y), d2f_bits(y.y))));
  };
  // (a x b)_f = a_f1 b_f2 - a_f2 b_f1, linear part in the fluctuations:
  // Ubar_f1 om_f2 - Ubar_f2 om_f1 + u_f1 Obar_f2 - u_f2 Obar_f1
  float2 acc = make_float2(0.f, 0.f);
  auto add = [&](float c, int q) {
    if (c == 0.f) return;
    const float2 v = F(q);
    acc.x = __fmaf_rn(c, v.x, acc.x);
    acc.y = __fmaf_rn(c, v.y, acc.y);
  };
  add(r.u1, 3 + r.f2);
  add(-r.u2, 3 + r.f1);
  add(r.o2, r.f1);
  add(-r.o1, r.f2);
  return acc;
}

}  // namespace owt

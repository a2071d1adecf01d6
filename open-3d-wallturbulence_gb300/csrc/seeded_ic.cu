// Seeded initial condition generated on the device: laminar Poiseuille flow
// plus a random divergence-free perturbation, built as follows, so that a
// batch of many channels needs no host work to start:
//
//  * per Fourier mode (kx, kz) != (0, 0): complex Gaussian coefficients a_p,
//    b_p (p = 0..5) of Chebyshev series, scaled by the energy spectrum
//    amp = (kmin / k)^2 (k = |(kx, kz)|, kmin the smaller fundamental);
//  * v = amp (1 - y^2)^2 sum a_p T_p(y), omega_y = amp (1 - y^2) sum b_p T_p(y),
//    so v, dv/dy and omega_y vanish at both walls;
//  * u, w from continuity and the definition of omega_y with the formulas of
//    the reference's solve_horizontal (src/solver.cpp:532-533):
//    u = i kx/k^2 DY1 v - i kz/k^2 g, w = i kx/k^2 g + i kz/k^2 DY1 v;
//  * the kx = 0 column Hermitian in kz (mode -kz the conjugate of +kz), the
//    Nyquist kz row zero, so the physical field is real;
//  * the perturbation scaled to an RMS of `rms` (Parseval over the modes, kx > 0
//    counted twice, trapezoidal weights in y), then the mean mode set to the
//    laminar profile 1.5 (1 - y^2) (src/solver.cpp:338-341).
//
// Random numbers: the counter-based generator Philox4x32-10 (Salmon, Moraes,
// Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC 2011), keyed by
// the seed and counted by (mode, p, series), two 53-bit uniforms per draw and
// one Box-Muller pair per complex coefficient.  Every value depends only on
// the seed and the mode, so the field is the same for any launch shape, and the
// RMS sum is reduced in a fixed order, so a seed gives the same bits each time.
#include <cuda_runtime.h>
#include <stdint.h>

#include "solve_kernels.h"

namespace owt {

namespace {

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}

// uniform in (0, 1) from 53 bits of two 32-bit words
__device__ __forceinline__ double unit53(uint32_t hi, uint32_t lo) {
  const uint64_t m = ((uint64_t)hi << 21) | (uint64_t)(lo >> 11);
  return ((double)m + 0.5) * 0x1.0p-53;
}

// complex standard Gaussian (variance 1 per part) for counter (mode, p, series)
__device__ __forceinline__ double2 gauss(uint64_t seed, int mode, int p, int series) {
  const uint4 r = philox4x32_10(make_uint4((uint32_t)mode, (uint32_t)p, (uint32_t)series, 0u),
                                make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
  const double u1 = unit53(r.x, r.y), u2 = unit53(r.z, r.w);
  const double rad = sqrt(-2.0 * log(u1));
  double s, c;
  sincos(6.283185307179586 * u2, &s, &c);
  return make_double2(rad * c, rad * s);
}

}  // namespace

// Coefficients [m][series][p] of every mode, Hermitian in the kx = 0 column.
__global__ void k_ic_coef(SeedArgs a) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= a.M) return;
  const int k = m / a.NXH, i = m - k * a.NXH;
  const int np = a.degree + 1;
  double2 *out = a.coef + (size_t)m * 2 * np;
  const bool mirror = i == 0 && k > a.NZH;  // mode -kz of the kx = 0 column
  const int src = mirror ? (a.NZ - k) * a.NXH : m;
  const bool zero = m == 0 || k == a.NZH;
  for (int s = 0; s < 2; ++s)
    for (int p = 0; p < np; ++p) {
      double2 z = make_double2(0.0, 0.0);
      if (!zero) {
        z = gauss(a.seed, src, p, s);
        if (mirror) z.y = -z.y;
      }
      out[s * np + p] = z;
    }
}

// v (into v) and omega_y (into g), [y][mode]
__global__ void k_ic_fields(SeedArgs a, double2 *v, double2 *g) {
  const size_t n = (size_t)a.NY * a.M;
  const int np = a.degree + 1;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / a.M), m = (int)(e - (size_t)j * a.M);
    const int k = m / a.NXH, i = m - k * a.NXH;
    const double kx = a.kx[i], kz = a.kz[k];
    const double k2 = kx * kx + kz * kz;
    const double amp = k2 > 0.0 ? a.kmin * a.kmin / k2 : 0.0;
    const double y = a.y[j], s1 = 1.0 - y * y;
    const double2 *cf = a.coef + (size_t)m * 2 * np;
    double2 sv = make_double2(0.0, 0.0), sg = make_double2(0.0, 0.0);
    double tp = 1.0, tq = y;  // T_p, T_(p+1)
    for (int p = 0; p < np; ++p) {
      sv.x += cf[p].x * tp; sv.y += cf[p].y * tp;
      sg.x += cf[np + p].x * tp; sg.y += cf[np + p].y * tp;
      const double tn = 2.0 * y * tq - tp;  // T_(p+2) = 2 y T_(p+1) - T_p
      tp = tq;
      tq = tn;
    }
    const double fv = amp * s1 * s1, fg = amp * s1;
    v[e] = make_double2(sv.x * fv, sv.y * fv);
    g[e] = make_double2(sg.x * fg, sg.y * fg);
  }
}

// u, w from DY1 v (raw compact derivative, metric c11 applied here) and g
__global__ void k_ic_uw(SeedArgs a, const double2 *d1v_raw, const double2 *g, double2 *u, double2 *w) {
  const size_t n = (size_t)a.NY * a.M;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / a.M), m = (int)(e - (size_t)j * a.M);
    const int k = m / a.NXH, i = m - k * a.NXH;
    const double kx = a.kx[i], kz = a.kz[k];
    const double k2 = kx * kx + kz * kz;
    if (m == 0 || !(k2 > 0.0)) {
      u[e] = make_double2(0.0, 0.0);
      w[e] = make_double2(0.0, 0.0);
      continue;
    }
    const double c = a.c11[j];
    const double2 dv = make_double2(c * d1v_raw[e].x, c * d1v_raw[e].y), gg = g[e];
    const double ax = kx / k2, az = kz / k2;
    // i a z = (-a z.y, a z.x)
    u[e] = make_double2(-ax * dv.y + az * gg.y, ax * dv.x - az * gg.x);
    w[e] = make_double2(-ax * gg.y - az * dv.y, ax * gg.x + az * dv.x);
  }
}

// Weighted energy sum of u, v, w in a fixed order: block b of kIcBlocks sums
// elements b*256 + t + q*stride, then a tree in shared memory.
constexpr int kIcBlocks = 1024;
__global__ void __launch_bounds__(256) k_ic_energy(SeedArgs a, const double2 *u, const double2 *v, const double2 *w,
                                                   double *partial) {
  __shared__ double sh[256];
  const size_t n = (size_t)a.NY * a.M;
  double acc = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / a.M), m = (int)(e - (size_t)j * a.M);
    const int i = m % a.NXH;
    const double wt = (i == 0 ? 1.0 : 2.0) * a.wy[j];
    const double2 x = u[e], y = v[e], z = w[e];
    acc += wt * (x.x * x.x + x.y * x.y + y.x * y.x + y.y * y.y + z.x * z.x + z.y * z.y);
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// partial[kIcBlocks] := rms / sqrt(sum / 3) (0 when the sum is 0), one thread
__global__ void k_ic_scale_factor(double *partial, double rms) {
  double sum = 0.0;
  for (int b = 0; b < kIcBlocks; ++b) sum += partial[b];
  const double cur = sqrt(sum / 3.0);
  partial[kIcBlocks] = cur > 0.0 ? rms / cur : 0.0;
}

// u, v, w *= s; the mean mode of u := the laminar profile
__global__ void k_ic_apply(SeedArgs a, const double *partial, double2 *u, double2 *v, double2 *w) {
  const size_t n = (size_t)a.NY * a.M;
  const double s = partial[kIcBlocks];
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / a.M), m = (int)(e - (size_t)j * a.M);
    double2 x = u[e], y = v[e], z = w[e];
    x = make_double2(x.x * s, x.y * s);
    if (m == 0) {
      const double yy = a.y[j];
      x = make_double2(1.5 * (1.0 - yy * yy), 0.0);
    }
    u[e] = x;
    v[e] = make_double2(y.x * s, y.y * s);
    w[e] = make_double2(z.x * s, z.y * s);
  }
}

size_t ic_coef_values(int M, int degree) { return (size_t)M * 2 * (degree + 1); }
size_t ic_partial_values() { return kIcBlocks + 1; }

int launch_ic_fields(const SeedArgs &a, double2 *v, double2 *g, cudaStream_t st) {
  k_ic_coef<<<(a.M + 127) / 128, 128, 0, st>>>(a);
  k_ic_fields<<<1024, 256, 0, st>>>(a, v, g);
  return 2;
}
int launch_ic_velocity(const SeedArgs &a, const double2 *d1v_raw, const double2 *g, double2 *u, double2 *v,
                       double2 *w, double *partial, double rms, cudaStream_t st) {
  k_ic_uw<<<1024, 256, 0, st>>>(a, d1v_raw, g, u, w);
  k_ic_energy<<<kIcBlocks, 256, 0, st>>>(a, u, v, w, partial);
  k_ic_scale_factor<<<1, 1, 0, st>>>(partial, rms);
  k_ic_apply<<<1024, 256, 0, st>>>(a, partial, u, v, w);
  return 4;
}

}  // namespace owt

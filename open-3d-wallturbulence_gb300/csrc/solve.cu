// Per-mode wall-normal kernels of the time step (FP64 throughout).
//
// Device layout of a spectral field: [y][kz][kx] complex128, element
// (j, k, i) at j*M + k*NXH + i with M = NZ*NXH, so the mode index m = k*NXH + i
// is fastest and one thread per mode reads and writes coalesced rows.
//
// History levels (vely_0..2, vory_0..2, Hv_0..2, Hg_0..2 and the mean-mode
// vectors, src/setup.hpp:64-79) live in three-slot rings; the reference's
// deep-copy rotation (src/solver.cpp:612-626) becomes a step counter kept in
// device memory: at counter s, level l is slot (2s + l) mod 3.  The counter
// advances right after the mode kernel, so the new values written there
// become level 0 and every later kernel of the step sees them as current.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <random>
#include <vector>

#include "owt_device.cuh"
#include "solve_kernels.h"
#include "modes_kernel.cuh"

namespace owt {

// ---------------------------------------------------------------------------
// Assemble and factor one banded system per unique mode (thread per mode).
// value = t0 + s1[u] t1 + s2[u] t2; then LU with partial pivoting in the
// order of LAPACK dgbtf2 (pivot: first entry of maximal magnitude within KL
// rows; interchange across the current fill extent ju; scale; rank-1 update),
// pivot offsets kept as bytes, and the diagonal replaced by its reciprocal.
// ---------------------------------------------------------------------------
template <int KL, int KU>
__global__ void k_band_factor(double *__restrict__ ab, uint8_t *__restrict__ piv, int n, int U,
                              const double *__restrict__ t0, const double *__restrict__ t1,
                              const double *__restrict__ t2, const double *__restrict__ s1,
                              const double *__restrict__ s2, double *__restrict__ rscale, int *__restrict__ info) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= U) return;
  constexpr int KV = KL + KU;
  constexpr int NB = 2 * KL + KU + 1;
  const size_t sn = (size_t)n * U;
  auto AB = [&](int b, int c) -> double & { return ab[(size_t)b * sn + (size_t)c * U + u]; };
  const double a1 = s1 ? s1[u] : 0.0, a2 = s2 ? s2[u] : 0.0;
  for (int c = 0; c < n; ++c)
    for (int b = 0; b < NB; ++b) {
      double v = 0.0;
      if (b >= KL) {
        const size_t at = (size_t)(b - KL) * n + c;
        v = __fma_rn(a2, t2[at], __fma_rn(a1, t1[at], t0[at]));
      }
      AB(b, c) = v;
    }
  // row equilibration: row p holds A(p, c) at band row KV + p - c
  if (rscale) {
    for (int p = 0; p < n; ++p) {
      const int c0 = max(0, p - KL), c1 = min(n - 1, p + KU);
      double mx = 0.0;
      for (int c = c0; c <= c1; ++c) mx = fmax(mx, fabs(AB(KV + p - c, c)));
      const double inv = mx > 0.0 ? 1.0 / mx : 1.0;
      for (int c = c0; c <= c1; ++c) AB(KV + p - c, c) *= inv;
      rscale[(size_t)p * U + u] = inv;
    }
  }
  int ju = 0;
  for (int j = 0; j < n; ++j) {
    const int km = min(KL, n - 1 - j);
    int jp = 0;
    double best = fabs(AB(KV, j));
    for (int i = 1; i <= km; ++i) {
      const double v = fabs(AB(KV + i, j));
      if (v > best) { best = v; jp = i; }
    }
    piv[(size_t)j * U + u] = (uint8_t)jp;
    if (AB(KV + jp, j) == 0.0) {
      atomicMax(info, 1);
      continue;
    }
    ju = max(ju, min(j + KU + jp, n - 1));
    if (jp != 0)
      for (int c = j; c <= ju; ++c) {
        double &x = AB(KV + jp - (c - j), c);
        double &y = AB(KV - (c - j), c);
        const double t = x; x = y; y = t;
      }
    const double rp = 1.0 / AB(KV, j);
    for (int i = 1; i <= km; ++i) AB(KV + i, j) *= rp;
    for (int c = j + 1; c <= ju; ++c) {
      const double t = AB(KV - (c - j), c);
      if (t != 0.0)
        for (int i = 1; i <= km; ++i) {
          double &x = AB(KV + i - (c - j), c);
          x = __fma_rn(-AB(KV + i, j), t, x);
        }
    }
  }
  for (int j = 0; j < n; ++j) AB(KV, j) = 1.0 / AB(KV, j);
}

// Warp-cooperative form of k_band_factor for systems with few modes (a
// thread-per-mode LU is latency-bound when a channel has only hundreds of
// modes): one warp per unique mode, the active columns [j, j + KV] of its band
// in a shared-memory window (column c in slot c mod (KV + 1)); pivot search,
// interchange, scaling and the rank-1 update spread over the lanes.  Every
// element sees the same operations in the same order as in k_band_factor, so
// the factors are bitwise the same.  Rows are equilibrated as they enter the
// window: row p is first touched by the step of column p - KL, and its entries
// span columns p - KL .. p + KU, all in the window then and still unmodified.
template <int KL, int KU, int WARPS>
__global__ void __launch_bounds__(32 * WARPS)
    k_band_factor_warp(double *__restrict__ ab, uint8_t *__restrict__ piv, int n, int U, const double *__restrict__ t0,
                       const double *__restrict__ t1, const double *__restrict__ t2, const double *__restrict__ s1,
                       const double *__restrict__ s2, double *__restrict__ rscale, int *__restrict__ info) {
  constexpr int KV = KL + KU, NB = 2 * KL + KU + 1, WC = KV + 1;
  constexpr unsigned FULL = 0xffffffffu;
  __shared__ double win[WARPS][WC * NB];
  const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
  const int u = blockIdx.x * WARPS + wq;
  if (u >= U) return;  // the whole warp
  double *w = win[wq];
  const size_t sn = (size_t)n * U;
  auto W = [&](int b, int c) -> double & { return w[(c % WC) * NB + b]; };
  const double a1 = s1 ? s1[u] : 0.0, a2 = s2 ? s2[u] : 0.0;
  auto load_col = [&](int c) {
    for (int b = lane; b < NB; b += 32) {
      double v = 0.0;
      if (b >= KL) {
        const size_t at = (size_t)(b - KL) * n + c;
        v = __fma_rn(a2, t2[at], __fma_rn(a1, t1[at], t0[at]));
      }
      W(b, c) = v;
    }
  };
  auto equilibrate = [&](int p) {  // row p holds A(p, c) at band row KV + p - c
    const int c0 = max(0, p - KL), c1 = min(n - 1, p + KU);
    double mx = 0.0;
    for (int c = c0 + lane; c <= c1; c += 32) mx = fmax(mx, fabs(W(KV + p - c, c)));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(FULL, mx, o));
    const double inv = mx > 0.0 ? 1.0 / mx : 1.0;
    for (int c = c0 + lane; c <= c1; c += 32) W(KV + p - c, c) *= inv;
    if (lane == 0) rscale[(size_t)p * U + u] = inv;
  };
  for (int c = 0; c <= min(n - 1, KV); ++c) load_col(c);
  __syncwarp();
  if (rscale)
    for (int p = 0; p <= min(n - 1, KL); ++p) equilibrate(p);
  __syncwarp();
  int ju = 0;
  for (int j = 0; j < n; ++j) {
    const int km = min(KL, n - 1 - j);
    // pivot: the first entry of maximal magnitude among rows j .. j + km
    unsigned long long key = 0ull;
    int jp = 0x7fffffff;
    if (lane <= km) {
      const double v = fabs(W(KV + lane, j));
      key = v == v ? (unsigned long long)__double_as_longlong(v) : 0ull;  // non-negative: bits order as values
      jp = lane;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ok = __shfl_xor_sync(FULL, key, o);
      const int oj = __shfl_xor_sync(FULL, jp, o);
      if (ok > key || (ok == key && oj < jp)) {
        key = ok;
        jp = oj;
      }
    }
    if (lane == 0) piv[(size_t)j * U + u] = (uint8_t)jp;
    if (W(KV + jp, j) == 0.0) {
      if (lane == 0) atomicMax(info, 1);
    } else {
      ju = max(ju, min(j + KU + jp, n - 1));
      if (jp != 0)
        for (int c = j + lane; c <= ju; c += 32) {
          double &x = W(KV + jp - (c - j), c);
          double &y = W(KV - (c - j), c);
          const double t = x;
          x = y;
          y = t;
        }
      __syncwarp();
      const double rp = 1.0 / W(KV, j);
      for (int i = 1 + lane; i <= km; i += 32) W(KV + i, j) *= rp;
      __syncwarp();
      const int total = (ju - j) * km;
      for (int q = lane; q < total; q += 32) {
        const int cc = q / km, i = q - cc * km + 1, c = j + 1 + cc;
        const double t = W(KV - (c - j), c);  // row j: not written in this step
        if (t != 0.0) {
          double &x = W(KV + i - (c - j), c);
          x = __fma_rn(-W(KV + i, j), t, x);
        }
      }
    }
    __syncwarp();
    // column j is final: out to the factors, the diagonal as its reciprocal
    for (int b = lane; b < NB; b += 32) {
      double v = W(b, j);
      if (b == KV) v = 1.0 / v;
      ab[(size_t)b * sn + (size_t)j * U + u] = v;
    }
    __syncwarp();
    if (j + WC < n) load_col(j + WC);  // into column j's slot
    __syncwarp();
    if (rscale && j + 1 + KL < n) equilibrate(j + 1 + KL);
    __syncwarp();
  }
}

// kernel: 1 thread per mode, 2 warp per mode, 0 by the number of modes (the
// warp form when the thread form would leave the GPU mostly idle)
template <int KL, int KU>
static void factor_t(int kernel, double *ab, uint8_t *piv, int n, int U, const double *t0, const double *t1,
                     const double *t2, const double *s1, const double *s2, double *rscale, int *info,
                     cudaStream_t st) {
  if (kernel == 0) kernel = U < kBandFactorWarpBelow ? 2 : 1;
  if (kernel == 2) {
    constexpr int WARPS = 4;
    k_band_factor_warp<KL, KU, WARPS><<<(U + WARPS - 1) / WARPS, 32 * WARPS, 0, st>>>(ab, piv, n, U, t0, t1, t2, s1,
                                                                                      s2, rscale, info);
  } else {
    const int bs = 64, gs = (U + bs - 1) / bs;
    k_band_factor<KL, KU><<<gs, bs, 0, st>>>(ab, piv, n, U, t0, t1, t2, s1, s2, rscale, info);
  }
}
void launch_band_factor(int kl, int ku, double *ab, uint8_t *piv, int n, int U, const double *t0,
                        const double *t1, const double *t2, const double *s1, const double *s2, double *rscale,
                        int *info, cudaStream_t st, int kernel) {
  if (kl == kVKL && ku == kVKU) factor_t<kVKL, kVKU>(kernel, ab, piv, n, U, t0, t1, t2, s1, s2, rscale, info, st);
  else if (kl == 6 && ku == 6) factor_t<6, 6>(kernel, ab, piv, n, U, t0, t1, t2, s1, s2, rscale, info, st);
  else if (kl == 2 && ku == 2) factor_t<2, 2>(kernel, ab, piv, n, U, t0, t1, t2, s1, s2, rscale, info, st);
}

// Both factorization kernels on the same random systems: bitwise comparison
// of factors, pivots and row scales, and the time of each (testing aid).
int band_factor_selftest(int kl, int ku, int n, int U, uint64_t seed, long long *mismatches, float *ms_thread,
                         float *ms_warp) {
  const int rows = kl + ku + 1, nb = 2 * kl + ku + 1;
  std::mt19937_64 gen(seed);
  std::normal_distribution<double> nd(0.0, 1.0);
  std::vector<double> t[3], s[2];
  for (auto &v : t) { v.resize((size_t)rows * n); for (double &x : v) x = nd(gen); }
  for (auto &v : s) { v.resize(U); for (double &x : v) x = nd(gen); }
  const size_t nab = (size_t)nb * n * U, np = (size_t)n * U;
  double *d_t[3] = {}, *d_s[2] = {}, *ab[2] = {}, *rs[2] = {};
  uint8_t *pv[2] = {};
  int *info = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t err = cudaSuccess;
  auto chk = [&](cudaError_t e) { if (err == cudaSuccess) err = e; };
  for (int q = 0; q < 3; ++q) {
    chk(cudaMalloc(&d_t[q], t[q].size() * sizeof(double)));
    if (err == cudaSuccess) chk(cudaMemcpy(d_t[q], t[q].data(), t[q].size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  for (int q = 0; q < 2; ++q) {
    chk(cudaMalloc(&d_s[q], (size_t)U * sizeof(double)));
    if (err == cudaSuccess) chk(cudaMemcpy(d_s[q], s[q].data(), (size_t)U * sizeof(double), cudaMemcpyHostToDevice));
    chk(cudaMalloc(&ab[q], nab * sizeof(double)));
    chk(cudaMalloc(&rs[q], np * sizeof(double)));
    chk(cudaMalloc(&pv[q], np));
  }
  chk(cudaMalloc(&info, sizeof(int)));
  chk(cudaEventCreate(&e0));
  chk(cudaEventCreate(&e1));
  float ms[2] = {0.f, 0.f};
  if (err == cudaSuccess) {
    for (int q = 0; q < 2; ++q) {
      launch_band_factor(kl, ku, ab[q], pv[q], n, U, d_t[0], d_t[1], d_t[2], d_s[0], d_s[1], rs[q], info, 0, q + 1);
      chk(cudaEventRecord(e0, 0));
      launch_band_factor(kl, ku, ab[q], pv[q], n, U, d_t[0], d_t[1], d_t[2], d_s[0], d_s[1], rs[q], info, 0, q + 1);
      chk(cudaEventRecord(e1, 0));
      chk(cudaEventSynchronize(e1));
      chk(cudaGetLastError());
      if (err == cudaSuccess) chk(cudaEventElapsedTime(&ms[q], e0, e1));
    }
  }
  long long bad = 0;
  if (err == cudaSuccess) {
    std::vector<double> a(nab), b(nab), ra(np), rb(np);
    std::vector<uint8_t> pa(np), pb(np);
    chk(cudaMemcpy(a.data(), ab[0], nab * sizeof(double), cudaMemcpyDeviceToHost));
    chk(cudaMemcpy(b.data(), ab[1], nab * sizeof(double), cudaMemcpyDeviceToHost));
    chk(cudaMemcpy(ra.data(), rs[0], np * sizeof(double), cudaMemcpyDeviceToHost));
    chk(cudaMemcpy(rb.data(), rs[1], np * sizeof(double), cudaMemcpyDeviceToHost));
    chk(cudaMemcpy(pa.data(), pv[0], np, cudaMemcpyDeviceToHost));
    chk(cudaMemcpy(pb.data(), pv[1], np, cudaMemcpyDeviceToHost));
    for (size_t q = 0; q < nab; ++q) bad += std::memcmp(&a[q], &b[q], sizeof(double)) != 0;
    for (size_t q = 0; q < np; ++q) bad += (std::memcmp(&ra[q], &rb[q], sizeof(double)) != 0) + (pa[q] != pb[q]);
  }
  for (int q = 0; q < 3; ++q) cudaFree(d_t[q]);
  for (int q = 0; q < 2; ++q) { cudaFree(d_s[q]); cudaFree(ab[q]); cudaFree(rs[q]); cudaFree(pv[q]); }
  cudaFree(info);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (err != cudaSuccess) return -1;
  *mismatches = bad;
  *ms_thread = ms[0];
  *ms_warp = ms[1];
  return 0;
}

bool band_supported(int kl, int ku) {
  return (kl == kVKL && ku == kVKU) || (kl == 6 && ku == 6) || (kl == 2 && ku == 2);
}

// Mode-kernel variants live in modes_pair.cu and modes_quad.cu (separate
// translation units so they compile in parallel); this dispatches by index.
// Variants: the pair mapping's, then the quad mapping's, then those for
// single-channel launches only (modes_split.cu; batches choose among the
// first two families).
int modes_variant_count() { return modes_pair_count() + modes_quad_count() + modes_split_count(); }
int modes_batch_variant_count() { return modes_pair_count() + modes_quad_count(); }
bool modes_variant_is_quad(int v) {
  if (v < modes_pair_count()) return false;
  v -= modes_pair_count();
  return v < modes_quad_count() || modes_split_is_quad(v - modes_quad_count());
}
const char *modes_variant_name(int v) {
  if (v < modes_pair_count()) return modes_pair_name(v);
  v -= modes_pair_count();
  if (v < modes_quad_count()) return modes_quad_name(v);
  return modes_split_name(v - modes_quad_count());
}
void launch_modes(const ModeArgs &a, int klv, int kuv, int klg, int kug, bool sparse, int variant, cudaStream_t st) {
  if (!(klv == kVKL && kuv == kVKU && klg == 6 && kug == 6)) return;
  if (!sparse) { modes_dense_launch(a, st); return; }
  if (variant < modes_pair_count()) { modes_pair_launch(variant, a, st); return; }
  variant -= modes_pair_count();
  if (variant < modes_quad_count()) modes_quad_launch(variant, a, st);
  else modes_split_launch(variant - modes_quad_count(), a, st);
}

// Batched mode kernel: variant -1 is the full-band solve.
ModeBatchShape modes_batch_shape(int variant) {
  if (variant < 0) return modes_dense_batch_shape();
  if (variant < modes_pair_count()) return modes_pair_batch_shape(variant);
  return modes_quad_batch_shape(variant - modes_pair_count());
}
void launch_modes_batch(const BatchTable<ModeArgs> &t, int variant, int *work, int grid, cudaStream_t st) {
  if (variant < 0) modes_dense_batch_launch(t, work, grid, st);
  else if (variant < modes_pair_count()) modes_pair_batch_launch(variant, t, work, grid, st);
  else modes_quad_batch_launch(variant - modes_pair_count(), t, work, grid, st);
}

// Every factored system must keep its interior fill inside the masks of its
// masked solve: count the modes whose L or U has a nonzero outside the masks
// in columns [Masks::lo, n - Masks::hi).
template <int KL, int KU, int NT, int OFF, class Masks>
__global__ void k_check_pattern(const double *__restrict__ ab, const uint8_t *__restrict__ piv, int n, int U,
                                int *__restrict__ bad) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= U) return;
  constexpr int KV = KL + KU;
  const size_t sn = (size_t)n * U;
  int nbad = 0;
  for (int c = Masks::lo; c < n - Masks::hi; ++c) {
    const int ty = (c + OFF) % NT;
    const double *col = ab + (size_t)c * U + u;
    for (int t = 1; t <= KL; ++t)
      if (!((Masks::l(ty) >> t) & 1ull) && col[(size_t)(KV + t) * sn] != 0.0) ++nbad;
    for (int t = 1; t <= KV; ++t)
      if (!((Masks::u(ty) >> t) & 1ull) && col[(size_t)(KV - t) * sn] != 0.0) ++nbad;
    const int off = piv[(size_t)c * U + u];
    if (off != 0 && !((Masks::p(ty) >> off) & 1ull)) ++nbad;
  }
  if (nbad) atomicAdd(bad, 1);
}

// which: 0 the v-system, 1 the omega_y-system
// which: 0 the v-system against the eighth-order masks, 1 the omega_y-system,
// 2 the v-system against the sixth-order masks
void launch_check_pattern(int which, const double *ab, const uint8_t *piv, int n, int U, int *bad,
                          cudaStream_t st) {
  if (which == 0)
    k_check_pattern<kVKL, kVKU, 4, 2, VMasks><<<(U + 127) / 128, 128, 0, st>>>(ab, piv, n, U, bad);
  else if (which == 2)
    k_check_pattern<kVKL, kVKU, 4, 2, VMasks6><<<(U + 127) / 128, 128, 0, st>>>(ab, piv, n, U, bad);
  else
    k_check_pattern<6, 6, 2, 0, GMasks><<<(U + 127) / 128, 128, 0, st>>>(ab, piv, n, U, bad);
}
void launch_modes_sixth(const ModeArgs &a, cudaStream_t st) { modes_sixth_launch(a, st); }

// dst[p U + u] = scale[u] src[p U + u] (setup: per-mode factors folded into
// a [row][unique mode] table)
__global__ void k_scale_by_mode(double *dst, const double *src, const double *scale, int n, int U) {
  const size_t total = (size_t)n * U;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
    dst[e] = scale[e % U] * src[e];
}
void launch_scale_by_mode(double *dst, const double *src, const double *scale, int n, int U, cudaStream_t st) {
  const size_t total = (size_t)n * U;
  const unsigned blocks = (unsigned)std::min<size_t>((total + 255) / 256, 4096);
  k_scale_by_mode<<<blocks, 256, 0, st>>>(dst, src, scale, n, U);
}

__global__ void k_advance(long long *step) { *step += 1; }
void launch_advance(long long *step, cudaStream_t st) { k_advance<<<1, 1, 0, st>>>(step); }
__global__ void k_advance_batch(const __grid_constant__ StepCounters c) {
  if ((int)threadIdx.x < c.n) *c.p[threadIdx.x] += 1;
}
void launch_advance_batch(const StepCounters &c, cudaStream_t st) { k_advance_batch<<<1, kBatchChannels, 0, st>>>(c); }

// ---------------------------------------------------------------------------
// Mean mode (solve_mean + solve_friction_force, src/solver.cpp:306-327,
// 428-514) for the step whose counter value after advancing is s: old level l
// is slot (h+1+l) mod 3 and the new values go to slot h = ring_head(s).  It
// touches only mode (0, 0) of the fields and the mean histories, so in a step
// it runs concurrently with the mode kernel (pre_advance: s = counter + 1).  Thread 0 solves for the mean streamwise
// velocity U, thread 1 for W, each with the omega_y-system of mode (0, 0)
// (the same matrix as solve_mean's A).
// ---------------------------------------------------------------------------
template <bool SMEM>
__device__ __forceinline__ void mean_body(const MeanArgs &a) {
  const int t = threadIdx.x;
  const int NY = a.NY, n = a.n_g;
  const int h = ring_head(*a.step + (a.pre_advance ? 1 : 0));
  const int o0 = (h + 1) % 3, o1 = (h + 2) % 3, o2 = h;
  // The factors of mode (0, 0) are strided by the number of unique modes in
  // global memory; a sequential solve on them is latency-bound, so the block
  // first gathers them (and the scratch vectors) into shared memory.
  extern __shared__ __align__(16) unsigned char smraw[];
  constexpr int NB = 2 * 6 + 6 + 1;
  const double *ab = a.ab_g;
  const uint8_t *piv = a.piv_g;
  const double *rs = a.rs_g;
  int stride = a.U;
  double2 *scr = a.scratch;
  const int *rbc = a.rb_col;
  const double *rbv = a.rb_val, *c11 = a.c11, *c21 = a.c21, *c22 = a.c22;
  if (SMEM) {
    double2 *ssc = reinterpret_cast<double2 *>(smraw);             // 2 NY + 2 n
    double *sab = reinterpret_cast<double *>(ssc + 2 * NY + 2 * n);  // NB n
    double *srs = sab + (size_t)NB * n;                             // n
    double *srbv = srs + n;                                         // 5 n
    double *sc = srbv + 5 * (size_t)n;                              // 3 NY
    int *srbc = reinterpret_cast<int *>(sc + 3 * (size_t)NY);       // 5 n
    uint8_t *spv = reinterpret_cast<uint8_t *>(srbc + 5 * (size_t)n);  // n
    for (int e = t; e < NB * n; e += blockDim.x) sab[e] = a.ab_g[(size_t)e * a.U];
    for (int e = t; e < n; e += blockDim.x) {
      srs[e] = a.rs_g[(size_t)e * a.U];
      spv[e] = a.piv_g[(size_t)e * a.U];
    }
    for (int e = t; e < 5 * n; e += blockDim.x) { srbv[e] = a.rb_val[e]; srbc[e] = a.rb_col[e]; }
    for (int e = t; e < NY; e += blockDim.x) { sc[e] = a.c11[e]; sc[NY + e] = a.c21[e]; sc[2 * NY + e] = a.c22[e]; }
    ab = sab; piv = spv; rs = srs; stride = 1; scr = ssc;
    rbc = srbc; rbv = srbv; c11 = sc; c21 = sc + NY; c22 = sc + 2 * NY;
  }
  // right-hand sides of the U and W solves, all threads (solver.cpp:452-457)
  {
    const double al0 = 3.0, al1 = -1.5, al2 = 1.0 / 3.0, be0 = 3.0, be1 = -3.0, be2 = 1.0;
    for (int e = t; e < 2 * NY; e += blockDim.x) {
      const int q = e / NY, j = e - q * NY;
      const double2 *U = q == 0 ? a.U_ring : a.W_ring;
      const double2 *L = q == 0 ? a.lx_ring : a.lz_ring;
      const double *F = q == 0 ? a.fx_ring : a.fz_ring;
      double2 r = make_double2(0.0, 0.0);
      if (j != 0 && j != NY - 1) {
        const double f0 = F[o0], f1 = F[o1], f2 = F[o2];
        const double2 l0 = L[o0 * NY + j], l1 = L[o1 * NY + j], l2 = L[o2 * NY + j];
        const double2 u0 = U[o0 * NY + j], u1 = U[o1 * NY + j], u2 = U[o2 * NY + j];
        r.x = be0 * (l0.x + f0) + be1 * (l1.x + f1) + be2 * (l2.x + f2) +
              (al0 * u0.x + al1 * u1.x + al2 * u2.x) * a.inv_dt;
        r.y = be0 * l0.y + be1 * l1.y + be2 * l2.y + (al0 * u0.y + al1 * u1.y + al2 * u2.y) * a.inv_dt;
      }
      scr[(size_t)q * NY + j] = r;
    }
  }
  __syncthreads();
  // one lane per real component of each profile: lanes 0, 1 U (Re, Im),
  // lanes 2, 3 W; the factors are real, so each component is its own solve
  // with the operations the complex solve applies to it
  if (t < 4) {
    const int q = t >> 1, comp = t & 1;
    double *U = reinterpret_cast<double *>(q == 0 ? a.U_ring : a.W_ring) + comp;
    const double *sg = reinterpret_cast<const double *>(scr + (size_t)q * NY) + comp;
    double *yy = reinterpret_cast<double *>(scr + 2 * (size_t)NY + (size_t)q * n) + comp;
    double *dd = reinterpret_cast<double *>(a.dy1 + (size_t)q * NY) + comp;
    const double icg = a.inv_cg0;
    double d2 = 0.0;
    double *Un = U + 2 * (size_t)h * NY;
    auto rhs = [&](int p) -> double {
      double acc = 0.0;
      for (int e = 0; e < 5; ++e) acc += rbv[p * 5 + e] * sg[2 * rbc[p * 5 + e]];
      const double sc = icg * rs[(size_t)p * stride];
      return acc * sc;
    };
    auto ys = [&](int p, double y) { yy[2 * p] = y; };
    auto yl = [&](int p) -> double { return yy[2 * p]; };
    auto out = [&](int c, double x) {
      const int jn = c >> 1;
      if (c & 1) {
        d2 = x * a.inv_h2;
      } else {
        x = x * a.inv_h;
        double g = 0.0;
        if (jn != 0 && jn != NY - 1) {
          const double r = sg[2 * jn];
          const double w1 = a.nu * c21[jn], w2 = a.nu * c22[jn];
          g = (r + w1 * x + w2 * d2) * icg;
        }
        Un[2 * jn] = g;
        dd[2 * jn] = c11[jn] * x;
      }
    };
    band_solve<6, 6>(ab, piv, n, stride, 0, rhs, ys, yl, out);
  }
  __syncthreads();
  const double2 *dU = a.dy1, *dW = a.dy1 + NY;
  if (t == 0) {
    const double fx = -a.nu / a.Ly * (dU[NY - 1].x - dU[0].x);
    const double fz = -a.nu / a.Ly * (dW[NY - 1].x - dW[0].x);
    a.fx_ring[h] = fx;
    a.fz_ring[h] = fz;
    if (!isfinite(fx) || !isfinite(fz)) atomicMax(a.err, 2);
  }
  const double2 *Un = a.U_ring + (size_t)h * NY, *Wn = a.W_ring + (size_t)h * NY;
  for (int j = t; j < NY; j += blockDim.x) {
    const size_t at = (size_t)j * a.M;  // mode 0
    a.u_field[at] = Un[j];
    a.w_field[at] = Wn[j];
    a.ox_field[at] = dW[j];
    a.oz_field[at] = make_double2(-dU[j].x, -dU[j].y);
  }
}

template <bool SMEM>
__global__ void k_mean(const __grid_constant__ MeanArgs a) { mean_body<SMEM>(a); }

// every channel of a batch: block c runs channel c's mean mode
template <bool SMEM>
__global__ void k_mean_batch(const __grid_constant__ BatchTable<MeanArgs> t) { mean_body<SMEM>(t.a[blockIdx.x]); }

size_t mean_smem_bytes(int NY, int n_g) {
  return (2 * (size_t)NY + 2 * (size_t)n_g) * sizeof(double2) + 19 * (size_t)n_g * sizeof(double) +
         (size_t)n_g * sizeof(double) + 5 * (size_t)n_g * (sizeof(double) + sizeof(int)) +
         3 * (size_t)NY * sizeof(double) + (size_t)n_g + 16;
}

// Opt in to the shared memory of the staged mean-mode solve when it fits.
bool mean_prepare(int NY, int n_g) {
  const size_t b = mean_smem_bytes(NY, n_g);
  if (b > 200 * 1024) return false;
  return raise_smem_limit(k_mean<true>, b) == cudaSuccess;
}

void launch_mean(const MeanArgs &a, bool smem, cudaStream_t st) {
  if (smem) k_mean<true><<<1, 256, mean_smem_bytes(a.NY, a.n_g), st>>>(a);
  else k_mean<false><<<1, 128, 0, st>>>(a);
}

// shared memory of the batched launch: the largest channel's
cudaError_t mean_batch_prepare(size_t smem_bytes) { return raise_smem_limit(k_mean_batch<true>, smem_bytes); }
void launch_mean_batch(const BatchTable<MeanArgs> &t, bool smem, size_t smem_bytes, cudaStream_t st) {
  if (smem) k_mean_batch<true><<<t.n, 256, smem_bytes, st>>>(t);
  else k_mean_batch<false><<<t.n, 128, 0, st>>>(t);
}

// ---------------------------------------------------------------------------
// nonlinear_source (src/solver.cpp:240-260), one thread per real component of
// a mode (lanes 2m, 2m+1 are Re, Im of mode m; A1 and B1 are real):
//   Hg = i kz lx - i kx lz,   Hv = -k^2 ly - c11 A1^-1 B1 (i kx lx + i kz lz)
// written to the level-0 slot.  Pass 1 forms this lane's component of
// f = i kx lx + i kz lz once per row (scratch) and Hg; pass 2 applies B1 (at
// most four taps per row, checked at setup) inside the right-hand side of the
// A1 band solve and writes Hv from its output.  Component c of i z is
// (2c - 1) times the other component of z.  The lane of component 0 of mode
// (0, 0) also records the new mean Lamb vector (src/solver.cpp:296-302).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void nl_body(const NLArgs &a, const int tid) {
  const int m = tid >> 1, comp = tid & 1;
  if (m >= a.M) return;
  const int M = a.M, NY = a.NY;
  const int k = m / a.NXH, i = m - k * a.NXH;
  const double sgn = comp ? 1.0 : -1.0;
  const double kx = a.kx[i], kz = a.kz[k];
  const double skx = sgn * kx, skz = sgn * kz;
  const double k2 = kx * kx + kz * kz;
  const int h = ring_head(*a.step);
  const size_t fs = (size_t)NY * M;
  const double *lx = reinterpret_cast<const double *>(a.lx), *ly = reinterpret_cast<const double *>(a.ly);
  const double *lz = reinterpret_cast<const double *>(a.lz);
  double *hv = reinterpret_cast<double *>(a.hv_ring + (size_t)h * fs) + comp;
  double *hg = reinterpret_cast<double *>(a.hg_ring + (size_t)h * fs) + comp;
  double *f = reinterpret_cast<double *>(a.fscr) + comp;
  double *y = reinterpret_cast<double *>(a.yscr) + comp;
  auto E = [&](int j) { return 2 * ((size_t)j * M + m); };
  const int oc = 1 - comp;
  for (int j = 0; j < NY; ++j) {
    const size_t e = E(j);
    const double x = lx[e + oc], z = lz[e + oc];
    f[e] = skx * x + skz * z;
    hg[e] = skz * x - skx * z;
  }
  auto rhs = [&](int p) -> double {
    double acc = 0.0;
#pragma unroll
    for (int q = 0; q < 4; ++q) acc += a.b1_val[p * 5 + q] * f[E(a.b1_col[p * 5 + q])];
    return acc;
  };
  auto ys = [&](int p, double v) { y[E(p)] = v; };
  auto yl = [&](int p) -> double { return y[E(p)]; };
  auto out = [&](int c, double d) {
    const size_t e = E(c);
    hv[e] = -k2 * ly[e + comp] - a.c11[c] * d;
  };
  band_solve<2, 2>(a.ab1, a.piv1, NY, 1, 0, rhs, ys, yl, out);
  if (m == 0 && comp == 0 && a.lx_mean) {
    for (int j = 0; j < NY; ++j) {
      a.lx_mean[(size_t)h * NY + j] = a.lx[(size_t)j * M];
      a.lz_mean[(size_t)h * NY + j] = a.lz[(size_t)j * M];
    }
  }
}

__global__ void __launch_bounds__(128) k_nl(const __grid_constant__ NLArgs a) {
  nl_body(a, blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void __launch_bounds__(128) k_nl_batch(const __grid_constant__ BatchTable<NLArgs> t) {
  const int c = batch_channel(t.start, t.n, blockIdx.x);
  nl_body(t.a[c], (blockIdx.x - t.start[c]) * 128 + threadIdx.x);
}

void launch_nl(const NLArgs &a, cudaStream_t st) {
  const int bs = 128, gs = (2 * a.M + bs - 1) / bs;
  k_nl<<<gs, bs, 0, st>>>(a);
}
int nl_batch_blocks(const NLArgs &a) { return (2 * a.M + 127) / 128; }
void launch_nl_batch(const BatchTable<NLArgs> &t, cudaStream_t st) { k_nl_batch<<<t.start[t.n], 128, 0, st>>>(t); }

// ---------------------------------------------------------------------------
// d = A_n^-1 B_n f along y for every mode (raw compact derivative on the
// uniform s-grid; callers apply the metric).  Used at start-up and by the
// DYn entry point, not in the step.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_dapply(DApplyArgs a) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= a.M) return;
  const int M = a.M, NY = a.NY;
  for (int j = 0; j < NY; ++j) {
    double2 acc = make_double2(0.0, 0.0);
#pragma unroll
    for (int e = 0; e < 5; ++e) {
      const double b = a.b_val[j * 5 + e];
      if (b != 0.0) {
        const double2 f = a.in[(size_t)a.b_col[j * 5 + e] * M + m];
        acc.x += b * f.x;
        acc.y += b * f.y;
      }
    }
    a.bf[(size_t)j * M + m] = acc;
  }
  auto rhs = [&](int p) -> double2 { return a.bf[(size_t)p * M + m]; };
  auto ys = [&](int p, double2 y) { a.yscr[(size_t)p * M + m] = y; };
  auto yl = [&](int p) -> double2 { return a.yscr[(size_t)p * M + m]; };
  auto out = [&](int c, double2 d) { a.out[(size_t)c * M + m] = d; };
  band_solve<2, 2>(a.ab, a.piv, NY, 1, 0, rhs, ys, yl, out);
}

void launch_dapply(const DApplyArgs &a, cudaStream_t st) {
  const int bs = 128, gs = (a.M + bs - 1) / bs;
  k_dapply<<<gs, bs, 0, st>>>(a);
}

// ---------------------------------------------------------------------------
// DY2 f = c21 A1^-1 B1 f + c22 A2^-1 B2 f along y for every mode of up to
// three fields (the DY2 v history after v levels were replaced), in one
// launch: one thread per field (blockIdx.y), mode and real component (the
// band systems are real), two band solves per thread with the B stencils
// applied inside the right-hand sides.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_dy2(DY2Args a) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if ((tid >> 1) >= a.mcount) return;
  const int m = a.m0 + (tid >> 1), comp = tid & 1, f = blockIdx.y;
  const int M = a.M, NY = a.NY;
  auto E = [&](int j) { return 2 * ((size_t)j * M + m) + comp; };
  const double *in = reinterpret_cast<const double *>(a.in[f]);
  double *out = reinterpret_cast<double *>(a.out[f]);
  double *scr = reinterpret_cast<double *>(a.scr[f]);
  auto ys = [&](int p, double y) { scr[E(p)] = y; };
  auto yl = [&](int p) -> double { return scr[E(p)]; };
  auto stencil = [&](const int *bc, const double *bv, int p) -> double {
    double acc = 0.0;
#pragma unroll
    for (int e = 0; e < 5; ++e) {
      const double b = bv[p * 5 + e];
      if (b != 0.0) acc += b * in[E(bc[p * 5 + e])];
    }
    return acc;
  };
  auto rhs1 = [&](int p) -> double { return stencil(a.b1_col, a.b1_val, p); };
  auto out1 = [&](int c, double d) { out[E(c)] = a.c21[c] * d; };
  band_solve<2, 2>(a.ab1, a.piv1, NY, 1, 0, rhs1, ys, yl, out1);
  auto rhs2 = [&](int p) -> double { return stencil(a.b2_col, a.b2_val, p); };
  auto out2 = [&](int c, double d) { out[E(c)] += a.c22[c] * d; };
  band_solve<2, 2>(a.ab2, a.piv2, NY, 1, 0, rhs2, ys, yl, out2);
}

void launch_dy2(const DY2Args &a, cudaStream_t st) {
  k_dy2<<<dim3((unsigned)((2 * (long long)a.mcount + 127) / 128), a.nf), 128, 0, st>>>(a);
}

// Elementwise helpers --------------------------------------------------------

// out = sa * A + sb * B with per-y real coefficients (either may be null).
__global__ void k_combine_y(double2 *out, const double2 *A, const double *ca, const double2 *B, const double *cb,
                            int NY, int M) {
  const size_t n = (size_t)NY * M;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / M);
    double2 r = make_double2(0.0, 0.0);
    if (A) { r.x += ca[j] * A[e].x; r.y += ca[j] * A[e].y; }
    if (B) { r.x += cb[j] * B[e].x; r.y += cb[j] * B[e].y; }
    out[e] = r;
  }
}
void launch_combine_y(double2 *out, const double2 *A, const double *ca, const double2 *B, const double *cb, int NY,
                      int M, cudaStream_t st) {
  k_combine_y<<<1024, 256, 0, st>>>(out, A, ca, B, cb, NY, M);
}

// get_vor_from_vel (src/solver.cpp:227-237) given D1 u and D1 w:
//   vorx = c11 D1w - i kz v ; vory = i kz u - i kx w ; vorz = i kx v - c11 D1u
__global__ void k_vor(VorArgs a) {
  const size_t n = (size_t)a.NY * a.M;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / a.M);
    const int m = (int)(e - (size_t)j * a.M);
    const int k = m / a.NXH, i = m - k * a.NXH;
    const double kx = a.kx[i], kz = a.kz[k], c11 = a.c11[j];
    const double2 u = a.u[e], v = a.v[e], w = a.w[e], du = a.d1u[e], dw = a.d1w[e];
    a.ox[e] = make_double2(c11 * dw.x + kz * v.y, c11 * dw.y - kz * v.x);
    a.oy[e] = make_double2(-kz * u.y + kx * w.y, kz * u.x - kx * w.x);
    a.oz[e] = make_double2(-kx * v.y - c11 * du.x, kx * v.x - c11 * du.y);
  }
}
void launch_vor(const VorArgs &a, cudaStream_t st) { k_vor<<<1024, 256, 0, st>>>(a); }

// solve_friction_force (src/solver.cpp:306-327) from D1 u and D1 w of mode 0;
// shift = 1 moves the history by explicit copies (stand-alone call), shift = 0
// writes level 0 in place (start-up fills all levels afterwards).
__global__ void k_friction(const double2 *d1u, const double2 *d1w, const double *c11, int NY, int M, double nu,
                           double Ly, double *fx_ring, double *fz_ring, const long long *step, int shift, int *err) {
  const int h = ring_head(*step);
  const double dub = c11[0] * d1u[0].x, dut = c11[NY - 1] * d1u[(size_t)(NY - 1) * M].x;
  const double dwb = c11[0] * d1w[0].x, dwt = c11[NY - 1] * d1w[(size_t)(NY - 1) * M].x;
  const double fx = -nu / Ly * (dut - dub), fz = -nu / Ly * (dwt - dwb);
  if (shift) {
    const int l0 = h, l1 = (h + 1) % 3, l2 = (h + 2) % 3;
    fx_ring[l2] = fx_ring[l1]; fx_ring[l1] = fx_ring[l0];
    fz_ring[l2] = fz_ring[l1]; fz_ring[l1] = fz_ring[l0];
  }
  fx_ring[h] = fx;
  fz_ring[h] = fz;
  if (!isfinite(fx) || !isfinite(fz)) atomicMax(err, 2);
}
void launch_friction(const double2 *d1u, const double2 *d1w, const double *c11, int NY, int M, double nu, double Ly,
                     double *fx_ring, double *fz_ring, const long long *step, int shift, int *err, cudaStream_t st) {
  k_friction<<<1, 1, 0, st>>>(d1u, d1w, c11, NY, M, nu, Ly, fx_ring, fz_ring, step, shift, err);
}

// Mean Lamb history shift by copies, as Lamb_vec does it (src/solver.cpp:296-302).
__global__ void k_lamb_mean_shift(double2 *lx_ring, double2 *lz_ring, const double2 *lx, const double2 *lz, int NY,
                                  int M, const long long *step) {
  const int h = ring_head(*step), l1 = (h + 1) % 3, l2 = (h + 2) % 3;
  for (int j = threadIdx.x; j < NY; j += blockDim.x) {
    lx_ring[l2 * NY + j] = lx_ring[l1 * NY + j];
    lx_ring[l1 * NY + j] = lx_ring[h * NY + j];
    lx_ring[h * NY + j] = lx[(size_t)j * M];
    lz_ring[l2 * NY + j] = lz_ring[l1 * NY + j];
    lz_ring[l1 * NY + j] = lz_ring[h * NY + j];
    lz_ring[h * NY + j] = lz[(size_t)j * M];
  }
}
void launch_lamb_mean_shift(double2 *lx_ring, double2 *lz_ring, const double2 *lx, const double2 *lz, int NY, int M,
                            const long long *step, cudaStream_t st) {
  k_lamb_mean_shift<<<1, 256, 0, st>>>(lx_ring, lz_ring, lx, lz, NY, M, step);
}

// Wall-normal statistics by Parseval, one block per y plane, fixed reduction
// order (deterministic).  Physical field f = sum_{kx>0} 2 Re(f_k e^{..}) +
// Re(sum_kz f(0,kz) e^{..}) with the Nyquist kz row dropped, so the x-z mean of
// f g is sum_{kx>0} 2 Re(f conj g) + sum_kz Re(Hf conj Hg) over the kx = 0
// column's Hermitian parts Hf(kz) = (f(kz) + conj f(-kz))/2.
__global__ void k_stats(const double2 *u, const double2 *v, const double2 *w, int NY, int NZ, int NXH, double *out) {
  const int j = blockIdx.x;
  const int M = NZ * NXH, NZH = NZ / 2;
  const double2 *pu = u + (size_t)j * M, *pv = v + (size_t)j * M, *pw = w + (size_t)j * M;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};  // uu, vv, ww, uv
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    const int k = m / NXH, i = m - k * NXH;
    if (k == NZH) continue;
    double2 a = pu[m], b = pv[m], c = pw[m];
    double wgt = 2.0;
    if (i == 0) {
      const int kp = (k == 0) ? 0 : NZ - k;
      const double2 ap = pu[(size_t)kp * NXH], bp = pv[(size_t)kp * NXH], cp = pw[(size_t)kp * NXH];
      a = make_double2(0.5 * (a.x + ap.x), 0.5 * (a.y - ap.y));
      b = make_double2(0.5 * (b.x + bp.x), 0.5 * (b.y - bp.y));
      c = make_double2(0.5 * (c.x + cp.x), 0.5 * (c.y - cp.y));
      wgt = 1.0;
    }
    acc[0] += wgt * (a.x * a.x + a.y * a.y);
    acc[1] += wgt * (b.x * b.x + b.y * b.y);
    acc[2] += wgt * (c.x * c.x + c.y * c.y);
    acc[3] += wgt * (a.x * b.x + a.y * b.y);
  }
  __shared__ double red[4][256];
  for (int q = 0; q < 4; ++q) red[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int q = 0; q < 4; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double U = pu[0].x, V = pv[0].x, W = pw[0].x;
    out[0 * NY + j] = U;
    out[1 * NY + j] = V;
    out[2 * NY + j] = W;
    out[3 * NY + j] = sqrt(fmax(red[0][0] - U * U, 0.0));
    out[4 * NY + j] = sqrt(fmax(red[1][0] - V * V, 0.0));
    out[5 * NY + j] = sqrt(fmax(red[2][0] - W * W, 0.0));
    out[6 * NY + j] = red[3][0] - U * V;
  }
}
void launch_stats(const double2 *u, const double2 *v, const double2 *w, int NY, int NZ, int NXH, double *out,
                  cudaStream_t st) {
  k_stats<<<NY, 256, 0, st>>>(u, v, w, NY, NZ, NXH, out);
}

// Reference layout [z][x][y] <-> device layout [y][z][x]: a transpose of an
// M x NY matrix of complex128 through 32 x 32 shared-memory tiles.
__global__ void k_transpose(const double2 *__restrict__ in, double2 *__restrict__ out, int rows, int cols) {
  __shared__ double2 tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int row = by + r, col = bx + threadIdx.x;
    if (row < rows && col < cols) tile[r][threadIdx.x] = in[(size_t)row * cols + col];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int orow = bx + r, ocol = by + threadIdx.x;
    if (orow < cols && ocol < rows) out[(size_t)orow * rows + ocol] = tile[threadIdx.x][r];
  }
}
void launch_transpose(const double2 *in, double2 *out, int rows, int cols, cudaStream_t st) {
  dim3 b(32, 8), g((cols + 31) / 32, (rows + 31) / 32);
  k_transpose<<<g, b, 0, st>>>(in, out, rows, cols);
}
// A block of rows of the reference layout into the device layout: rows r of
// in ([rows][cols]) become columns r of out, whose rows are ldo values apart.
__global__ void k_transpose_ld(const double2 *__restrict__ in, double2 *__restrict__ out, int rows, int cols,
                               int ldo) {
  __shared__ double2 tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int row = by + r, col = bx + threadIdx.x;
    if (row < rows && col < cols) tile[r][threadIdx.x] = in[(size_t)row * cols + col];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int orow = bx + r, ocol = by + threadIdx.x;
    if (orow < cols && ocol < rows) out[(size_t)orow * ldo + ocol] = tile[threadIdx.x][r];
  }
}
void launch_transpose_ld(const double2 *in, double2 *out, int rows, int cols, int ldo, cudaStream_t st) {
  dim3 b(32, 8), g((cols + 31) / 32, (rows + 31) / 32);
  k_transpose_ld<<<g, b, 0, st>>>(in, out, rows, cols, ldo);
}
// Host -> device copy by the SMs: 16-byte loads of device-addressable host
// memory (pinned, or any host memory on a system with coherent host access)
// over the host link, grid-strided over one block per SM.
__global__ void k_host_load(const float4 *__restrict__ src, float4 *__restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}
void launch_host_load(const void *src, void *dst, size_t bytes, cudaStream_t st) {
  if (bytes == 0) return;
  k_host_load<<<152, 256, 0, st>>>(static_cast<const float4 *>(src), static_cast<float4 *>(dst), bytes / 16);
}
// Physical fields: [y][z][x] (device) <-> [z][x][y] (the reference's
// Field<double> layout), a rows x cols transpose of doubles.
__global__ void k_transpose_real(const double *__restrict__ in, double *__restrict__ out, int rows, int cols) {
  __shared__ double tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int row = by + r, col = bx + threadIdx.x;
    if (row < rows && col < cols) tile[r][threadIdx.x] = in[(size_t)row * cols + col];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int orow = bx + r, ocol = by + threadIdx.x;
    if (orow < cols && ocol < rows) out[(size_t)orow * rows + ocol] = tile[threadIdx.x][r];
  }
}
void launch_transpose_real(const double *in, double *out, int rows, int cols, cudaStream_t st) {
  dim3 b(32, 8), g((cols + 31) / 32, (rows + 31) / 32);
  k_transpose_real<<<g, b, 0, st>>>(in, out, rows, cols);
}

}  // namespace owt

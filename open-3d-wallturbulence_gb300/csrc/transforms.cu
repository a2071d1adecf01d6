// Dealiased transforms and the Lamb vector (src/solver.cpp:262-304,
// src/FFT.cpp:49-194) as three kernels that never write a padded 3/2-grid
// physical field to memory:
//
//  k_zback : per (y, kx tile, field) -- gather kz into the padded z line
//            (k < NZH -> slot k, k > NZH -> slot k + NZH, the Nyquist row
//            k = NZH dropped, FFT.cpp:78-87), backward FFT of length NZ2.
//  k_xlamb : per (y, z) line pair -- Hermitian extension in x (slot i = u_i,
//            slot NX + i = conj(u_{NXH-i}), FFT.cpp:109-119) with two real
//            fields packed into one complex backward FFT of length NX2 (the
//            real part of the reference's c2c output is exactly such a c2r,
//            with Im u_0 ignored), the cross product u x omega in physical
//            space (solver.cpp:284-286, no fused multiply-add), two real
//            products packed into one forward FFT, keep kx < NXH, / NX2
//            (FFT.cpp:153-162).
//  k_zfwd  : per (y, kx tile, field) -- forward FFT of length NZ2, keep slots
//            k < NZH and NZ + k (k < NZH) -> kz index k + NZH, / NZ2
//            (FFT.cpp:177-188).  The Nyquist row is kept on this path.
//            FP32 (mixed precision): plus the mean-flow terms.
//  k_mean_lamb (mixed precision only): the mean-flow terms that the FP32
//            transforms leave out, mode by mode in FP32 (mean_flow.cuh).
//
// Between kernels the z-padded, x-truncated planes live in HBM as
// [field][y][z][kx] complex<T>.  T = double (FP64 step) or float (mixed).
#include <cuda_runtime.h>

#include "mean_flow.cuh"
#include "owt_device.cuh"
#include "solve_kernels.h"

namespace owt {

template <typename T> struct XCfg;
// TX lines per z block, P (y, z) lines per x block (3P FFT lines).  Blocks
// have as many threads as the line length (NZ2 or NX2, at most 1024).
// XREG caps the x-pass registers: 56 keeps two 576-thread FP32 blocks (whose
// shared memory allows two) resident per SM; 64 is the bound of a 1024-thread
// block.
template <> struct XCfg<double> { static constexpr int TX = 6; static constexpr int P = 4; static constexpr int XREG = 64; };
template <> struct XCfg<float> { static constexpr int TX = 12; static constexpr int P = 4; static constexpr int XREG = 56; };

__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }

// Each kernel's body takes its block coordinates explicitly: the one-channel
// kernels pass blockIdx, the batched kernels the coordinates of the block
// within its channel's grid.
template <typename T, bool R5>
__device__ __forceinline__ void zback_body(const XformArgs &a, const int bx, const int j, const int f) {
  constexpr int TX = XCfg<T>::TX;
  extern __shared__ __align__(16) unsigned char smraw[];
  const XformDims d = a.d;
  const int ls = line_stride<T>(d.NZ2);
  cpx<T> *bufa = reinterpret_cast<cpx<T> *>(smraw);
  cpx<T> *bufb = bufa + TX * ls;
  const int i0 = bx * TX;
  const int M = d.NZ * d.NXH;
  const double2 *base = a.in[f];
  if (a.ring_mask & (1 << f)) base += (size_t)ring_head(*a.step) * a.fs;
  const double2 *src = base + (size_t)j * M;
  for (int idx = threadIdx.x; idx < TX * ls; idx += blockDim.x) bufa[idx] = mk<T>((T)0, (T)0);
  __syncthreads();
  for (int idx = threadIdx.x; idx < d.NZ * TX; idx += blockDim.x) {
    const int kz = idx / TX, c = idx - kz * TX;
    if (i0 + c < d.NXH && kz != d.NZH && !(a.mean_split && kz == 0 && i0 + c == 0)) {
      const int slot = kz < d.NZH ? kz : kz + d.NZH;
      bufa[c * ls + sw<T>(slot)] = from_d<T>(src[(size_t)kz * d.NXH + i0 + c]);
    }
  }
  __syncthreads();
  const cpx<T> *r = fft_lines<T, true, R5>(bufa, bufb, TX, ls, a.pz, reinterpret_cast<const cpx<T> *>(a.twz));
  cpx<T> *dst = reinterpret_cast<cpx<T> *>(a.zbuf) + ((size_t)f * d.NY + j) * d.NZ2 * d.NXH;
  for (int idx = threadIdx.x; idx < d.NZ2 * TX; idx += blockDim.x) {
    const int z = idx / TX, c = idx - z * TX;
    if (i0 + c < d.NXH) dst[(size_t)z * d.NXH + i0 + c] = r[c * ls + sw<T>(z)];
  }
}

template <typename T, int P, bool R5>
__device__ __forceinline__ void xlamb_body(const XformArgs &a, const int bx) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const XformDims d = a.d;
  const int ls = line_stride<T>(d.NX2);
  cpx<T> *bufa = reinterpret_cast<cpx<T> *>(smraw);
  cpx<T> *bufb = bufa + 3 * P * ls;
  const size_t nlines = (size_t)d.NY * d.NZ2;
  const size_t line0 = (size_t)bx * P;
  const size_t fstride = nlines * d.NXH;
  const cpx<T> *zb = reinterpret_cast<const cpx<T> *>(a.zbuf);
  // 1. pack field pairs (u,v), (w,ox), (oy,oz) into complex spectra; the
  // block has NX2 threads, thread mm owns point mm of every line
  const int mm = threadIdx.x;
#pragma unroll
  for (int q = 0; q < 3 * P; ++q) {
    const int pair = q / P, l = q - pair * P;
    const size_t line = line0 + l;
    cpx<T> z = mk<T>((T)0, (T)0);
    if (line < nlines) {
      const cpx<T> *A = zb + (size_t)(2 * pair) * fstride + line * d.NXH;
      z = hermitian_pair<T>(A, A + fstride, mm, d.NXH, d.NX2);
    }
    bufa[q * ls + sw<T>(mm)] = z;
  }
  __syncthreads();
  const cpx<T> *tw = reinterpret_cast<const cpx<T> *>(a.twx);
  cpx<T> *r = fft_lines<T, true, R5>(bufa, bufb, 3 * P, ls, a.px, tw);
  cpx<T> *o = (r == bufa) ? bufb : bufa;
  // 2. lamb = u x omega, packed as (lx + i ly) per line and (lz_l + i lz_l+1)
#pragma unroll
  for (int l = 0; l < P; ++l) {
    const int x = sw<T>(mm);
    const cpx<T> uv = r[(0 * P + l) * ls + x], wox = r[(1 * P + l) * ls + x], oyz = r[(2 * P + l) * ls + x];
    const T u = uv.x, v = uv.y, w = wox.x, ox = wox.y, oy = oyz.x, oz = oyz.y;
    const T lx = mul_rn(v, oz) - mul_rn(w, oy);
    const T ly = mul_rn(w, ox) - mul_rn(u, oz);
    const T lz = mul_rn(u, oy) - mul_rn(v, ox);
    o[l * ls + x] = mk<T>(lx, ly);
    if (l & 1) o[(P + l / 2) * ls + x].y = lz;
    else o[(P + l / 2) * ls + x].x = lz;
  }
  __syncthreads();
  cpx<T> *fo = fft_lines<T, false, R5>(o, r, P + P / 2, ls, a.px, tw);
  // 3. unpack the real-pair spectra, keep kx < NXH, scale by 1/NX2
  cpx<T> *lb = reinterpret_cast<cpx<T> *>(a.lbuf);
  const T half = (T)(0.5 * a.inv_nx2);
  for (int idx = threadIdx.x; idx < P * d.NXH; idx += blockDim.x) {
    const int l = idx / d.NXH, km = idx - l * d.NXH;
    const size_t line = line0 + l;
    if (line >= nlines) continue;
    const int mc = (km == 0) ? 0 : d.NX2 - km;
    {
      const cpx<T> zm = fo[l * ls + sw<T>(km)], zc = fo[l * ls + sw<T>(mc)];
      // Xa = (Z[m] + conj Z[-m]) / 2 ; Xb = (Z[m] - conj Z[-m]) / (2i)
      lb[line * d.NXH + km] = mk<T>((zm.x + zc.x) * half, (zm.y - zc.y) * half);
      lb[fstride + line * d.NXH + km] = mk<T>((zm.y + zc.y) * half, (zc.x - zm.x) * half);
    }
    {
      const cpx<T> zm = fo[(P + l / 2) * ls + sw<T>(km)], zc = fo[(P + l / 2) * ls + sw<T>(mc)];
      const cpx<T> val = (l & 1) ? mk<T>((zm.y + zc.y) * half, (zc.x - zm.x) * half)
                                 : mk<T>((zm.x + zc.x) * half, (zm.y - zc.y) * half);
      lb[2 * fstride + line * d.NXH + km] = val;
    }
  }
}

template <typename T, bool R5>
__device__ __forceinline__ void zfwd_body(const XformArgs &a, const int bx, const int j, const int f) {
  constexpr int TX = XCfg<T>::TX;
  extern __shared__ __align__(16) unsigned char smraw[];
  const XformDims d = a.d;
  const int ls = line_stride<T>(d.NZ2);
  cpx<T> *bufa = reinterpret_cast<cpx<T> *>(smraw);
  cpx<T> *bufb = bufa + TX * ls;
  const int i0 = bx * TX;
  const cpx<T> *src = reinterpret_cast<const cpx<T> *>(a.lbuf) + ((size_t)f * d.NY + j) * d.NZ2 * d.NXH;
  for (int idx = threadIdx.x; idx < d.NZ2 * TX; idx += blockDim.x) {
    const int z = idx / TX, c = idx - z * TX;
    bufa[c * ls + sw<T>(z)] = (i0 + c < d.NXH) ? src[(size_t)z * d.NXH + i0 + c] : mk<T>((T)0, (T)0);
  }
  __syncthreads();
  const cpx<T> *r = fft_lines<T, false, R5>(bufa, bufb, TX, ls, a.pz, reinterpret_cast<const cpx<T> *>(a.twz));
  double2 *dst = a.out[f] + (size_t)j * d.NZ * d.NXH;
  if constexpr (sizeof(T) == sizeof(float)) {
    // FP32 transforms: the 1/NZ2 normalisation and (mean split) the
    // mean-flow terms k_mean_lamb wrote, in FP32, then the exact widening
    const float sc = (float)a.inv_nz2;
    const float2 *lm = a.mean_split ? a.lm[f] + (size_t)j * d.NZ * d.NXH : nullptr;
    for (int idx = threadIdx.x; idx < d.NZ * TX; idx += blockDim.x) {
      const int kz = idx / TX, c = idx - kz * TX;
      if (i0 + c < d.NXH) {
        const int slot = kz < d.NZH ? kz : kz + d.NZH;
        const float2 v = r[c * ls + sw<T>(slot)];
        const size_t at = (size_t)kz * d.NXH + i0 + c;
        float2 o = make_float2(__fmul_rn(v.x, sc), __fmul_rn(v.y, sc));
        if (lm) {
          const float2 l = lm[at];
          o.x = __fadd_rn(o.x, l.x);
          o.y = __fadd_rn(o.y, l.y);
        }
        dst[at] = to_d(o);
      }
    }
  } else {
    const double sc = a.inv_nz2;
    for (int idx = threadIdx.x; idx < d.NZ * TX; idx += blockDim.x) {
      const int kz = idx / TX, c = idx - kz * TX;
      if (i0 + c < d.NXH) {
        const int slot = kz < d.NZH ? kz : kz + d.NZH;
        const double2 v = r[c * ls + sw<T>(slot)];
        // explicit roundings: the batched and the one-channel kernels must
        // give the same bits whatever each compilation contracts
        dst[(size_t)kz * d.NXH + i0 + c] = make_double2(__dmul_rn(v.x, sc), __dmul_rn(v.y, sc));
      }
    }
  }
}

// Kernels.  R5: the lines the kernel transforms have a radix-5 stage (3NZ/2,
// 3NX/2 divisible by 5).  The radix-5 butterfly is compiled only into those
// instances, so the others keep their register budget (and occupancy).
template <typename T, bool R5>
__global__ void __launch_bounds__(1024) k_zback(const __grid_constant__ XformArgs a) {
  zback_body<T, R5>(a, blockIdx.x, blockIdx.y, blockIdx.z);
}
template <typename T, int P, bool R5>
__global__ void __maxnreg__(XCfg<T>::XREG) k_xlamb(const __grid_constant__ XformArgs a) {
  xlamb_body<T, P, R5>(a, blockIdx.x);
}
template <typename T, bool R5>
__global__ void __launch_bounds__(1024) k_zfwd(const __grid_constant__ XformArgs a) {
  zfwd_body<T, R5>(a, blockIdx.x, blockIdx.y, blockIdx.z);
}
__global__ void __launch_bounds__(256) k_mean_lamb(const __grid_constant__ XformArgs a) {
  mean_lamb_body(a, blockIdx.x, blockIdx.y);
}

// Stand-alone dealiased transforms of one field in FP64 (the reference's
// Fourier2Physical_dealiased / Physical2Fourier_dealiased, src/FFT.cpp:49-194):
// the z passes are the step's (field 0 of zbuf / lbuf); these x kernels write
// or read physical lines instead of forming products.  A block transforms
// 2 kPhysQ (y, z) lines, two real lines per complex FFT; physical lines are
// [y][z][x] with x fastest.
constexpr int kPhysQ = 4;
template <bool R5>
__global__ void __launch_bounds__(1024) k_xback_phys(const __grid_constant__ XformArgs a, double *phys) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const XformDims d = a.d;
  const int ls = line_stride<double>(d.NX2);
  double2 *bufa = reinterpret_cast<double2 *>(smraw);
  double2 *bufb = bufa + kPhysQ * ls;
  const size_t nlines = (size_t)d.NY * d.NZ2;
  const size_t line0 = (size_t)blockIdx.x * 2 * kPhysQ;
  const double2 *zb = reinterpret_cast<const double2 *>(a.zbuf);
  const int mm = threadIdx.x;
  for (int q = 0; q < kPhysQ; ++q) {
    const size_t la = line0 + 2 * q, lb = la + 1;
    double2 z = make_double2(0.0, 0.0);
    if (la < nlines)
      z = hermitian_pair<double, true>(zb + la * d.NXH, lb < nlines ? zb + lb * d.NXH : nullptr, mm, d.NXH, d.NX2);
    bufa[q * ls + mm] = z;
  }
  __syncthreads();
  const double2 *r = fft_lines<double, true, R5>(bufa, bufb, kPhysQ, ls, a.px, reinterpret_cast<const double2 *>(a.twx));
  for (int q = 0; q < kPhysQ; ++q) {
    const size_t la = line0 + 2 * q, lb = la + 1;
    const double2 v = r[q * ls + mm];
    if (la < nlines) phys[la * d.NX2 + mm] = v.x;
    if (lb < nlines) phys[lb * d.NX2 + mm] = v.y;
  }
}
template <bool R5>
__global__ void __launch_bounds__(1024) k_xfwd_phys(const __grid_constant__ XformArgs a, const double *phys) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const XformDims d = a.d;
  const int ls = line_stride<double>(d.NX2);
  double2 *bufa = reinterpret_cast<double2 *>(smraw);
  double2 *bufb = bufa + kPhysQ * ls;
  const size_t nlines = (size_t)d.NY * d.NZ2;
  const size_t line0 = (size_t)blockIdx.x * 2 * kPhysQ;
  const int mm = threadIdx.x;
  for (int q = 0; q < kPhysQ; ++q) {
    const size_t la = line0 + 2 * q, lb = la + 1;
    bufa[q * ls + mm] = make_double2(la < nlines ? phys[la * d.NX2 + mm] : 0.0, lb < nlines ? phys[lb * d.NX2 + mm] : 0.0);
  }
  __syncthreads();
  const double2 *fo = fft_lines<double, false, R5>(bufa, bufb, kPhysQ, ls, a.px, reinterpret_cast<const double2 *>(a.twx));
  // keep kx < NXH, / NX2 (FFT.cpp:153-162): Xa = (Z[m] + conj Z[-m]) / 2, Xb = (Z[m] - conj Z[-m]) / (2i)
  double2 *lb_out = reinterpret_cast<double2 *>(a.lbuf);
  const double half = 0.5 * a.inv_nx2;
  for (int idx = threadIdx.x; idx < kPhysQ * d.NXH; idx += blockDim.x) {
    const int q = idx / d.NXH, km = idx - q * d.NXH;
    const size_t la = line0 + 2 * q, lb = la + 1;
    const int mc = (km == 0) ? 0 : d.NX2 - km;
    const double2 zm = fo[q * ls + km], zc = fo[q * ls + mc];
    if (la < nlines) lb_out[la * d.NXH + km] = make_double2((zm.x + zc.x) * half, (zm.y - zc.y) * half);
    if (lb < nlines) lb_out[lb * d.NXH + km] = make_double2((zm.y + zc.y) * half, (zc.x - zm.x) * half);
  }
}

// Batched: one launch over every channel of a table whose channels share the
// precision and the length of the lines a block spans (NZ2 for the z passes,
// NX2 for the x pass); blocks are numbered channel by channel, each channel's
// grid flattened x fastest.
template <typename T, bool R5>
__global__ void __launch_bounds__(1024) k_zback_batch(const __grid_constant__ BatchTable<XformArgs> t) {
  const int c = batch_channel(t.start, t.n, blockIdx.x);
  const XformArgs &a = t.a[c];
  const int gx = (a.d.NXH + XCfg<T>::TX - 1) / XCfg<T>::TX, lb = blockIdx.x - t.start[c], r = lb / gx;
  zback_body<T, R5>(a, lb - r * gx, r % a.d.NY, r / a.d.NY);
}
template <typename T, int P, bool R5>
__global__ void __maxnreg__(XCfg<T>::XREG) k_xlamb_batch(const __grid_constant__ BatchTable<XformArgs> t) {
  const int c = batch_channel(t.start, t.n, blockIdx.x);
  xlamb_body<T, P, R5>(t.a[c], blockIdx.x - t.start[c]);
}
template <typename T, bool R5>
__global__ void __launch_bounds__(1024) k_zfwd_batch(const __grid_constant__ BatchTable<XformArgs> t) {
  const int c = batch_channel(t.start, t.n, blockIdx.x);
  const XformArgs &a = t.a[c];
  const int gx = (a.d.NXH + XCfg<T>::TX - 1) / XCfg<T>::TX, lb = blockIdx.x - t.start[c], r = lb / gx;
  zfwd_body<T, R5>(a, lb - r * gx, r % a.d.NY, r / a.d.NY);
}
__global__ void __launch_bounds__(256) k_mean_lamb_batch(const __grid_constant__ BatchTable<XformArgs> t) {
  const int c = batch_channel(t.start, t.n, blockIdx.x);
  const XformArgs &a = t.a[c];
  const int gx = (a.d.NZ * a.d.NXH + 255) / 256, lb = blockIdx.x - t.start[c], r = lb / gx;
  mean_lamb_body(a, lb - r * gx, r);
}

static void launch_mean_lamb(const XformArgs &a, cudaStream_t st) {
  const int M = a.d.NZ * a.d.NXH;
  k_mean_lamb<<<dim3((M + 255) / 256, a.d.NY), 256, 0, st>>>(a);
}

template <typename T>
static size_t smem_z(const XformDims &d) { return 2 * (size_t)XCfg<T>::TX * line_stride<T>(d.NZ2) * sizeof(cpx<T>); }
template <typename T>
static size_t smem_x(const XformDims &d, int P) { return 2 * 3 * (size_t)P * line_stride<T>(d.NX2) * sizeof(cpx<T>); }
// (y, z) lines per x block: XCfg<T>::P where its shared memory fits, else 2
// (FP64 lines longer than 604 points)
template <typename T>
static int x_lines(const XformDims &d) {
  return smem_x<T>(d, XCfg<T>::P) <= 227 * 1024 ? XCfg<T>::P : 2;
}

// The instances a channel's transforms use: by precision, x lines per block
// and radix-5 stages of the z and x lines.
// FP32 lines with a two-pass factorisation (transforms_reg.cu) use the
// register-transform kernels unless `stockham` is set; they keep TX = 12
// columns per z block, and P (y, z) lines per x block of their own.
template <typename T>
struct XformKernels {
  int P;
  void (*zback)(XformArgs), (*xlamb)(XformArgs), (*zfwd)(XformArgs);
  void (*zback_b)(BatchTable<XformArgs>), (*xlamb_b)(BatchTable<XformArgs>), (*zfwd_b)(BatchTable<XformArgs>);
  int zthreads, xthreads;
  size_t zsmem, xsmem;
  int xgrid;  // x-pass blocks at most (0: one block per group of P lines)
};
template <typename T>
static XformKernels<T> kernels(const XformDims &d, bool stockham = false) {
  constexpr int PP = XCfg<T>::P;
  const bool z5 = d.NZ2 % 5 == 0, x5 = d.NX2 % 5 == 0;
  XformKernels<T> k;
  k.P = x_lines<T>(d);
  k.zthreads = d.NZ2;
  k.xthreads = d.NX2;
  k.zsmem = smem_z<T>(d);
  k.xsmem = smem_x<T>(d, k.P);
  k.xgrid = 0;
  k.zback = z5 ? k_zback<T, true> : k_zback<T, false>;
  k.zfwd = z5 ? k_zfwd<T, true> : k_zfwd<T, false>;
  k.zback_b = z5 ? k_zback_batch<T, true> : k_zback_batch<T, false>;
  k.zfwd_b = z5 ? k_zfwd_batch<T, true> : k_zfwd_batch<T, false>;
  if (k.P == PP) {
    k.xlamb = x5 ? k_xlamb<T, PP, true> : k_xlamb<T, PP, false>;
    k.xlamb_b = x5 ? k_xlamb_batch<T, PP, true> : k_xlamb_batch<T, PP, false>;
  } else {
    k.xlamb = x5 ? k_xlamb<T, 2, true> : k_xlamb<T, 2, false>;
    k.xlamb_b = x5 ? k_xlamb_batch<T, 2, true> : k_xlamb_batch<T, 2, false>;
  }
  if (sizeof(T) == sizeof(float) && !stockham) {
    static_assert(XCfg<float>::TX == 12, "register z kernels assume the FP32 z block shape");
    const RegXformKernels rz = reg_xform_kernels(d.NZ2), rx = reg_xform_kernels(d.NX2);
    if (rz.ok) {
      k.zback = rz.zback; k.zfwd = rz.zfwd; k.zback_b = rz.zback_b; k.zfwd_b = rz.zfwd_b;
      k.zthreads = rz.zthreads;
      k.zsmem = rz.zsmem;
    }
    if (rx.ok) {
      k.xlamb = rx.xlamb; k.xlamb_b = rx.xlamb_b;
      k.xthreads = rx.xthreads;
      k.xsmem = rx.xsmem;
      k.P = rx.xlines;
      k.xgrid = rx.xgrid;
    }
  }
  return k;
}

// One of the kernels (0: z backward, 1: x pass, 2: z forward, 3: the
// mean-flow terms of the mixed-precision Lamb vector).
template <typename T>
static void lamb_part_t(const XformArgs &a, int part, cudaStream_t st) {
  const XformDims &d = a.d;
  const XformKernels<T> k = kernels<T>(d, a.stockham != 0);
  constexpr int TX = XCfg<T>::TX;
  if (part == 0) {
    k.zback<<<dim3((d.NXH + TX - 1) / TX, d.NY, 6), k.zthreads, k.zsmem, st>>>(a);
  } else if (part == 1) {
    const size_t nl = (size_t)d.NY * d.NZ2;
    size_t grid = (nl + k.P - 1) / k.P;
    if (k.xgrid > 0 && grid > (size_t)k.xgrid) grid = k.xgrid;
    k.xlamb<<<(unsigned)grid, k.xthreads, k.xsmem, st>>>(a);
  } else if (part == 2) {
    k.zfwd<<<dim3((d.NXH + TX - 1) / TX, d.NY, 3), k.zthreads, k.zsmem, st>>>(a);
  } else if (a.mean_split) {
    launch_mean_lamb(a, st);
  }
}

// On one stream: the mean-flow terms (mixed precision) first, as the z
// forward adds them.
template <typename T>
static int lamb_t(const XformArgs &a, cudaStream_t st) {
  if (a.mean_split) lamb_part_t<T>(a, 3, st);
  for (int part = 0; part < 3; ++part) lamb_part_t<T>(a, part, st);
  return a.mean_split ? 4 : 3;
}

// Opt the channel's transform kernels (single and batched) in to the dynamic
// shared memory they need, before any launch or graph capture.
template <typename T>
static cudaError_t prepare_t(const XformDims &d) {
  cudaError_t e = cudaSuccess;
  for (int stockham = 0; stockham < 2 && e == cudaSuccess; ++stockham) {
    const XformKernels<T> k = kernels<T>(d, stockham != 0);
    e = raise_smem_limit(k.zback, k.zsmem);
    if (e == cudaSuccess) e = raise_smem_limit(k.zfwd, k.zsmem);
    if (e == cudaSuccess) e = raise_smem_limit(k.xlamb, k.xsmem);
    if (e == cudaSuccess) e = raise_smem_limit(k.zback_b, k.zsmem);
    if (e == cudaSuccess) e = raise_smem_limit(k.zfwd_b, k.zsmem);
    if (e == cudaSuccess) e = raise_smem_limit(k.xlamb_b, k.xsmem);
  }
  return e;
}

cudaError_t lamb_prepare(const XformDims &d) {
  cudaError_t e = prepare_t<double>(d);
  return e == cudaSuccess ? prepare_t<float>(d) : e;
}

int launch_lamb(const XformArgs &a, int precision, cudaStream_t st) {
  return precision == 0 ? lamb_t<double>(a, st) : lamb_t<float>(a, st);
}

void launch_lamb_part(const XformArgs &a, int precision, int part, cudaStream_t st) {
  if (precision == 0) lamb_part_t<double>(a, part, st);
  else lamb_part_t<float>(a, part, st);
}

// Blocks of one channel in part 0 (z backward), 1 (x pass), 2 (z forward) or
// 3 (mean-flow terms); the grids of the one-channel launches, flattened.
template <typename T>
static int lamb_blocks_t(const XformDims &d, int part, bool stockham) {
  const int gx = (d.NXH + XCfg<T>::TX - 1) / XCfg<T>::TX;
  if (part == 0) return gx * d.NY * 6;
  if (part == 2) return gx * d.NY * 3;
  if (part == 1) {
    const int P = kernels<T>(d, stockham).P;
    return (int)(((size_t)d.NY * d.NZ2 + P - 1) / P);
  }
  return ((d.NZ * d.NXH + 255) / 256) * d.NY;
}
int lamb_batch_blocks(const XformDims &d, int precision, int part, bool stockham) {
  return precision == 0 ? lamb_blocks_t<double>(d, part, stockham) : lamb_blocks_t<float>(d, part, stockham);
}

cudaError_t lamb_batch_prepare(const XformDims &d, int precision) {
  return precision == 0 ? prepare_t<double>(d) : prepare_t<float>(d);
}

template <typename T>
static void lamb_batch_t(const BatchTable<XformArgs> &t, int part, cudaStream_t st) {
  const XformDims &d = t.a[0].d;
  const XformKernels<T> k = kernels<T>(d, t.a[0].stockham != 0);
  const unsigned blocks = (unsigned)t.start[t.n];
  if (part == 0) k.zback_b<<<blocks, k.zthreads, k.zsmem, st>>>(t);
  else if (part == 1) k.xlamb_b<<<k.xgrid > 0 && blocks > (unsigned)k.xgrid ? (unsigned)k.xgrid : blocks, k.xthreads,
                                  k.xsmem, st>>>(t);
  else if (part == 2) k.zfwd_b<<<blocks, k.zthreads, k.zsmem, st>>>(t);
  else k_mean_lamb_batch<<<blocks, 256, 0, st>>>(t);
}
void launch_lamb_batch(const BatchTable<XformArgs> &t, int precision, int part, cudaStream_t st) {
  if (precision == 0) lamb_batch_t<double>(t, part, st);
  else lamb_batch_t<float>(t, part, st);
}

static size_t smem_phys(const XformDims &d) { return 2 * (size_t)kPhysQ * line_stride<double>(d.NX2) * sizeof(double2); }

cudaError_t phys_prepare(const XformDims &d) {
  const size_t sx = smem_phys(d);
  cudaError_t e = raise_smem_limit(k_xback_phys<true>, sx);
  if (e == cudaSuccess) e = raise_smem_limit(k_xback_phys<false>, sx);
  if (e == cudaSuccess) e = raise_smem_limit(k_xfwd_phys<true>, sx);
  if (e == cudaSuccess) e = raise_smem_limit(k_xfwd_phys<false>, sx);
  return e;
}

// a.in[0] (spectral [y][kz][kx], FP64 tables) -> phys [y][z][x]; zbuf field 0 in between.
void launch_fourier2physical(const XformArgs &a, double *phys, cudaStream_t st) {
  const XformDims &d = a.d;
  const XformKernels<double> k = kernels<double>(d);
  constexpr int TX = XCfg<double>::TX;
  k.zback<<<dim3((d.NXH + TX - 1) / TX, d.NY, 1), d.NZ2, smem_z<double>(d), st>>>(a);
  const size_t nl = (size_t)d.NY * d.NZ2;
  const unsigned blocks = (unsigned)((nl + 2 * kPhysQ - 1) / (2 * kPhysQ));
  if (d.NX2 % 5 == 0) k_xback_phys<true><<<blocks, d.NX2, smem_phys(d), st>>>(a, phys);
  else k_xback_phys<false><<<blocks, d.NX2, smem_phys(d), st>>>(a, phys);
}
// phys [y][z][x] -> a.out[0] (spectral); lbuf field 0 in between.
void launch_physical2fourier(const XformArgs &a, const double *phys, cudaStream_t st) {
  const XformDims &d = a.d;
  const XformKernels<double> k = kernels<double>(d);
  constexpr int TX = XCfg<double>::TX;
  const size_t nl = (size_t)d.NY * d.NZ2;
  const unsigned blocks = (unsigned)((nl + 2 * kPhysQ - 1) / (2 * kPhysQ));
  if (d.NX2 % 5 == 0) k_xfwd_phys<true><<<blocks, d.NX2, smem_phys(d), st>>>(a, phys);
  else k_xfwd_phys<false><<<blocks, d.NX2, smem_phys(d), st>>>(a, phys);
  k.zfwd<<<dim3((d.NXH + TX - 1) / TX, d.NY, 1), d.NZ2, smem_z<double>(d), st>>>(a);
}

size_t lamb_zbuf_bytes(const XformDims &d, int precision) {
  return 6 * (size_t)d.NY * d.NZ2 * d.NXH * (precision == 0 ? sizeof(double2) : sizeof(float2));
}
size_t lamb_lbuf_bytes(const XformDims &d, int precision) {
  return 3 * (size_t)d.NY * d.NZ2 * d.NXH * (precision == 0 ? sizeof(double2) : sizeof(float2));
}

// ---------------------------------------------------------------------------
// Check of d2f_bits against the hardware conversion.  Sample i is one of the
// edge values below (i < kConvEdges) or a splitmix64 bit pattern with an
// exponent across the FP32 range and a little beyond.  counts: [0] results
// equal to __double2float_rn, [1] ties (the dropped bits exactly half an
// ulp) rounded away from zero where the hardware rounds to even, [2]
// subnormal results flushed to zero, [3] results outside these three.
// ---------------------------------------------------------------------------
constexpr int kConvEdges = 16;
__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ bool f_is_nan(float f) { return (__float_as_uint(f) & 0x7fffffffu) > 0x7f800000u; }

__global__ void k_convert_check(long long n, uint64_t seed, unsigned long long *counts) {
  unsigned long long c[4] = {0, 0, 0, 0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const uint64_t r = splitmix64(seed ^ (uint64_t)i * 0x2545f4914f6cdd1dull), r2 = splitmix64(r);
    double x;
    if (i < kConvEdges) {
      // 0, -0, inf, -inf, NaN, ties with an even and an odd kept bit, the
      // largest float, 2^128 (overflow), just below the rounding-to-2^128
      // boundary, the smallest normal, half of it, 1, -1, 1/3, 1e30
      const uint64_t e[kConvEdges] = {0x0000000000000000ull, 0x8000000000000000ull, 0x7ff0000000000000ull,
                                      0xfff0000000000000ull, 0x7ff8000000000001ull, 0x3ff0000010000000ull,
                                      0x3ff0000030000000ull, 0x47efffffe0000000ull, 0x47f0000000000000ull,
                                      0x47efffffefffffffull, 0x3810000000000000ull, 0x3800000000000000ull,
                                      0x3ff0000000000000ull, 0xbff0000000000000ull, 0x3fd5555555555555ull,
                                      0x46293e5939a08ceaull};
      x = __longlong_as_double((long long)e[i]);
    } else {
      // exponent 1023 + [-140, 140), random sign and fraction
      const uint64_t ex = (uint64_t)(1023 - 140 + (int)(r2 % 280));
      x = __longlong_as_double((long long)((r & 0x800fffffffffffffull) | (ex << 52)));
    }
    const float got = d2f_bits(x), want = __double2float_rn(x);
    const unsigned ug = __float_as_uint(got), uw = __float_as_uint(want);
    const unsigned lo = (unsigned)__double2loint(x), ah = (unsigned)__double2hiint(x) & 0x7fffffffu;
    const bool tie = (lo & 0x1fffffffu) == 0x10000000u && ah >= (897u << 20) && ah < (1151u << 20);
    if (ug == uw || (f_is_nan(got) && f_is_nan(want))) ++c[0];
    else if (tie && (ug & 0x7fffffffu) == (uw & 0x7fffffffu) + 1u && (ug >> 31) == (uw >> 31)) ++c[1];
    else if ((ug & 0x7fffffffu) == 0u && (uw & 0x7fffffffu) <= 0x00800000u && (ug >> 31) == (uw >> 31)) ++c[2];
    else ++c[3];
  }
  for (int k = 0; k < 4; ++k)
    if (c[k]) atomicAdd(counts + k, c[k]);
}

int convert_selftest(long long n, uint64_t seed, long long counts[4]) {
  unsigned long long *d = nullptr;
  cudaError_t e = cudaMalloc(&d, 4 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(d, 0, 4 * sizeof(unsigned long long));
  if (e == cudaSuccess) {
    k_convert_check<<<1024, 256>>>(n, seed, d);
    e = cudaGetLastError();
  }
  unsigned long long h[4] = {};
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
  if (d) cudaFree(d);
  for (int k = 0; k < 4; ++k) counts[k] = (long long)h[k];
  return e == cudaSuccess ? 0 : 1;
}

}  // namespace owt

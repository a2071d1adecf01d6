// FP32 transform kernels of the mixed-precision step with register-resident
// line transforms (fft_reg.cuh), for line lengths L = A B with a two-pass
// factorisation (reg_fft_a): the same three kernels, data layouts and
// dealiasing as transforms.cu (src/FFT.cpp:49-194, src/solver.cpp:262-304),
// but each line is transformed by A-point and B-point transforms held in
// registers with one shared-memory transpose between them, instead of one
// shared-memory pass per radix-2/3/4 stage.
//
// A line of length L is held by T = max(A, B) threads.  Pass 1: thread b < B
// transforms the points b + B a (a < A), multiplies output a' by w_L^(b a')
// and stores it at row a', column b of the line's transpose (rows padded to
// B + 1 values).  Pass 2: thread a < A reads row a and transforms it; its
// output b' is point a + A b' of the line's transform.
//
//  k_zback_r : block (kx tile of TX columns, y, field); thread (t, c) with the
//              column c fastest, so that global loads and stores along kx
//              coalesce; the padded z line is gathered straight into pass-1
//              registers (the Nyquist row and the padding are zeros).
//  k_xlamb_r : persistent; per group of P (y, z) lines: 3P packed backward
//              lines (field pairs), products u x omega in shared memory, 3P/2
//              packed forward lines, the real-pair unpack; thread (q, t), t
//              fastest; the next group's input lines arrive by cp.async.
//  k_zfwd_r  : as k_zback_r, forward, keeping kz < NZ/2 and the upper slots,
//              / NZ2, plus the mixed precision's mean-flow terms.
#include <cuda_runtime.h>

#include "batch.cuh"
#include "fft_reg.cuh"
#include "owt_device.cuh"
#include "solve_kernels.h"

namespace owt {

constexpr int kRegTX = 12;  // kx columns per z block (as the FP32 Stockham z kernels)

template <int A, int B>
struct Line2 {
  static constexpr int L = A * B;
  static constexpr int T = A > B ? A : B;
  static constexpr int RS = B + 1;      // row stride of the transpose
  static constexpr int TS = A * RS;     // values of one transpose
  static constexpr int LS = TS > L ? TS : L;  // shared-memory values per line
};

// x[a'] *= w_L^(b a') (forward) or its conjugate (backward), a' >= 1; the
// table (in shared memory) holds exp(-2 pi i k / L) for k < L, and b a' < L.
template <int A, bool BACKWARD>
__device__ __forceinline__ void twiddle_row(float2 *x, int b, const float2 *tw) {
#pragma unroll
  for (int a = 1; a < A; ++a) {
    float2 w = tw[b * a];
    if (BACKWARD) w.y = -w.y;
    x[a] = cmul(x[a], w);
  }
}

// The twiddle table of a line length into shared memory (then a barrier).
__device__ __forceinline__ void load_twiddles(float2 *dst, const float2 *__restrict__ src, int L) {
  for (int k = threadIdx.x; k < L; k += blockDim.x) dst[k] = src[k];
  __syncthreads();
}

// ---------------------------------------------------------------------------
// z backward
// ---------------------------------------------------------------------------
template <int A, int B>
__device__ __forceinline__ void zback_r_body(const XformArgs &a, const int bx, const int j, const int f) {
  using G = Line2<A, B>;
  extern __shared__ __align__(16) unsigned char smraw[];
  float2 *S = reinterpret_cast<float2 *>(smraw);
  const XformDims d = a.d;
  const int c = threadIdx.x % kRegTX, t = threadIdx.x / kRegTX;
  const int i = bx * kRegTX + c;
  const bool col = i < d.NXH;
  const int M = d.NZ * d.NXH;
  const double2 *base = a.in[f];
  if (a.ring_mask & (1 << f)) base += (size_t)ring_head(*a.step) * a.fs;
  const double2 *src = base + (size_t)j * M + i;
  float2 *tw = S + kRegTX * G::LS;
  load_twiddles(tw, reinterpret_cast<const float2 *>(a.twz), G::L);
  float2 *T0 = S + c * G::LS;
  if (t < B) {
    float2 x[A];
#pragma unroll
    for (int q = 0; q < A; ++q) {
      const int s = t + B * q;  // slot of the padded line: k < NZH -> k, k > NZH -> k + NZH
      int kz = -1;
      if (s < d.NZH) kz = s;
      else if (s > d.NZ) kz = s - d.NZH;
      float2 v = make_float2(0.f, 0.f);
      if (col && kz >= 0 && !(a.mean_split && kz == 0 && i == 0)) v = from_d<float>(src[(size_t)kz * d.NXH]);
      x[q] = v;
    }
    dft<A, true, float>(x);
    twiddle_row<A, true>(x, t, tw);
#pragma unroll
    for (int q = 0; q < A; ++q) T0[q * G::RS + t] = x[q];
  }
  __syncthreads();
  if (t < A && col) {
    float2 y[B];
#pragma unroll
    for (int q = 0; q < B; ++q) y[q] = T0[t * G::RS + q];
    dft<B, true, float>(y);
    float2 *dst = reinterpret_cast<float2 *>(a.zbuf) + ((size_t)f * d.NY + j) * d.NZ2 * d.NXH + i;
#pragma unroll
    for (int q = 0; q < B; ++q) dst[(size_t)(t + A * q) * d.NXH] = y[q];
  }
}

// ---------------------------------------------------------------------------
// z forward (+ the mean-flow terms of the mixed precision)
// ---------------------------------------------------------------------------
template <int A, int B>
__device__ __forceinline__ void zfwd_r_body(const XformArgs &a, const int bx, const int j, const int f) {
  using G = Line2<A, B>;
  extern __shared__ __align__(16) unsigned char smraw[];
  float2 *S = reinterpret_cast<float2 *>(smraw);
  const XformDims d = a.d;
  const int c = threadIdx.x % kRegTX, t = threadIdx.x / kRegTX;
  const int i = bx * kRegTX + c;
  const bool col = i < d.NXH;
  const float2 *src = reinterpret_cast<const float2 *>(a.lbuf) + ((size_t)f * d.NY + j) * d.NZ2 * d.NXH + i;
  float2 *tw = S + kRegTX * G::LS;
  load_twiddles(tw, reinterpret_cast<const float2 *>(a.twz), G::L);
  float2 *T0 = S + c * G::LS;
  if (t < B) {
    float2 x[A];
#pragma unroll
    for (int q = 0; q < A; ++q) x[q] = col ? src[(size_t)(t + B * q) * d.NXH] : make_float2(0.f, 0.f);
    dft<A, false, float>(x);
    twiddle_row<A, false>(x, t, tw);
#pragma unroll
    for (int q = 0; q < A; ++q) T0[q * G::RS + t] = x[q];
  }
  __syncthreads();
  if (t < A && col) {
    float2 y[B];
#pragma unroll
    for (int q = 0; q < B; ++q) y[q] = T0[t * G::RS + q];
    dft<B, false, float>(y);
    double2 *dst = a.out[f] + (size_t)j * d.NZ * d.NXH + i;
    const float2 *lm = a.mean_split ? a.lm[f] + (size_t)j * d.NZ * d.NXH + i : nullptr;
    // the 1/NZ2 normalisation and the mean-flow terms k_mean_lamb wrote, in
    // FP32, then the exact widening
    const float sc = (float)a.inv_nz2;
#pragma unroll
    for (int q = 0; q < B; ++q) {
      const int s = t + A * q;  // keep slots k < NZH (kz k) and NZ + k (kz k + NZH)
      int kz = -1;
      if (s < d.NZH) kz = s;
      else if (s >= d.NZ) kz = s - d.NZ + d.NZH;
      if (kz >= 0) {
        float2 o = make_float2(__fmul_rn(y[q].x, sc), __fmul_rn(y[q].y, sc));
        if (lm) {
          const float2 l = lm[(size_t)kz * d.NXH];
          o.x = __fadd_rn(o.x, l.x);
          o.y = __fadd_rn(o.y, l.y);
        }
        dst[(size_t)kz * d.NXH] = to_d(o);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// x pass: Hermitian extension, backward transforms of the field pairs,
// u x omega, forward transforms of the product pairs, kx < NXH, / NX2.
// Persistent: each resident block takes groups of P (y, z) lines g, g + grid,
// ...; while it transforms one group, the six input fields' lines of its next
// group arrive in the other half of a double buffer by cp.async (16-byte
// copies that bypass the registers; wait_group is a hardware wait).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, int src_bytes) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Start the copies of the six fields' lines line0 .. line0 + P - 1 (the P
// lines of a field are consecutive in memory) into buf: field f, line l at
// (f P + l) NXH.  Lines past the last are zero-filled without a read.
template <int P>
__device__ __forceinline__ void xlamb_stage(const XformArgs &a, size_t line0, float2 *buf) {
  const XformDims d = a.d;
  const size_t nlines = (size_t)d.NY * d.NZ2, fstride = nlines * d.NXH;
  const int nl = nlines - line0 < (size_t)P ? (int)(nlines - line0) : P;
  const int per4 = P * d.NXH / 2, have4 = nl * d.NXH / 2;  // 16-byte chunks per field (NXH even)
  const float4 *zb = reinterpret_cast<const float4 *>(a.zbuf);
  for (int idx = threadIdx.x; idx < 6 * per4; idx += blockDim.x) {
    const int f = idx / per4, o = idx - f * per4;
    const bool have = o < have4;
    const float4 *src = zb + ((size_t)f * fstride + line0 * d.NXH) / 2 + (have ? o : 0);
    cp_async16(reinterpret_cast<float4 *>(buf) + idx, src, have ? 16 : 0);
  }
}

// One group of P (y, z) lines in R (3P lines of shared memory).  Lines, in
// turn: the 3P backward transposes; the 3P physical lines (field pairs); in
// place, the 3P/2 product pairs in lines 0 .. 3P/2 - 1; their forward
// transposes in lines 3P/2 .. 3P - 1; their spectra in lines 0 .. 3P/2 - 1.
// after_input() runs once every thread has read Rin (the next group's input
// may then start arriving there).
template <int A, int B, int P, class AfterInput>
__device__ __forceinline__ void xlamb_r_group(const XformArgs &a, const size_t line0, const float2 *Rin, float2 *R,
                                              const float2 *tw, AfterInput after_input) {
  using G = Line2<A, B>;
  static_assert(P % 2 == 0, "lz lines pack two (y, z) lines each");
  constexpr int NF = P + P / 2, L = G::L;
  const XformDims d = a.d;
  const int q = threadIdx.x / G::T, t = threadIdx.x - q * G::T;
  const size_t nlines = (size_t)d.NY * d.NZ2;
  const size_t fstride = nlines * d.NXH;
  // 1. backward pass 1: packed line q = pair * P + l holds fields (2 pair, 2 pair + 1)
  if (t < B) {
    const int pair = q / P, l = q - pair * P;
    float2 x[A];
    const float2 *Af = Rin + (2 * pair * P + l) * d.NXH;
#pragma unroll
    for (int r = 0; r < A; ++r) x[r] = hermitian_pair<float>(Af, Af + P * d.NXH, t + B * r, d.NXH, d.NX2);
    dft<A, true, float>(x);
    twiddle_row<A, true>(x, t, tw);
#pragma unroll
    for (int r = 0; r < A; ++r) R[q * G::LS + r * G::RS + t] = x[r];
  }
  __syncthreads();
  after_input();
  // 2. backward pass 2: point t + A r of each packed line (a + i b = the two fields)
  float2 y[B];
  if (t < A) {
#pragma unroll
    for (int r = 0; r < B; ++r) y[r] = R[q * G::LS + t * G::RS + r];
    dft<B, true, float>(y);
  }
  __syncthreads();
  if (t < A) {
#pragma unroll
    for (int r = 0; r < B; ++r) R[q * G::LS + t + A * r] = y[r];
  }
  __syncthreads();
  // 3. lamb = u x omega (no fused multiply-add, as the reference's separate
  // products), packed as (lx + i ly) in line l and (lz_l + i lz_l+1) in line
  // P + l/2, in place: one thread owns point xx of every line, reading all
  // its values before writing any
  for (int xx = threadIdx.x; xx < L; xx += blockDim.x) {
    float2 uv[P], wox[P], oyz[P];
#pragma unroll
    for (int l = 0; l < P; ++l) {
      uv[l] = R[(0 * P + l) * G::LS + xx];
      wox[l] = R[(1 * P + l) * G::LS + xx];
      oyz[l] = R[(2 * P + l) * G::LS + xx];
    }
#pragma unroll
    for (int l = 0; l < P; l += 2) {
      float lz[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float u = uv[l + h].x, v = uv[l + h].y, w = wox[l + h].x, ox = wox[l + h].y, oy = oyz[l + h].x,
                    oz = oyz[l + h].y;
        const float lx = __fmul_rn(v, oz) - __fmul_rn(w, oy);
        const float ly = __fmul_rn(w, ox) - __fmul_rn(u, oz);
        lz[h] = __fmul_rn(u, oy) - __fmul_rn(v, ox);
        R[(l + h) * G::LS + xx] = make_float2(lx, ly);
      }
      R[(P + l / 2) * G::LS + xx] = make_float2(lz[0], lz[1]);
    }
  }
  __syncthreads();
  // 4. forward pass 1 of the NF product pairs, transposes into lines NF + q
  if (q < NF && t < B) {
    float2 x[A];
#pragma unroll
    for (int r = 0; r < A; ++r) x[r] = R[q * G::LS + t + B * r];
    dft<A, false, float>(x);
    twiddle_row<A, false>(x, t, tw);
#pragma unroll
    for (int r = 0; r < A; ++r) R[(NF + q) * G::LS + r * G::RS + t] = x[r];
  }
  __syncthreads();
  // 5. forward pass 2: spectrum slot t + A r, into line q
  if (q < NF && t < A) {
#pragma unroll
    for (int r = 0; r < B; ++r) y[r] = R[(NF + q) * G::LS + t * G::RS + r];
    dft<B, false, float>(y);
#pragma unroll
    for (int r = 0; r < B; ++r) R[q * G::LS + t + A * r] = y[r];
  }
  __syncthreads();
  // 6. unpack the real-pair spectra, keep kx < NXH, scale by 1/NX2
  float2 *lb = reinterpret_cast<float2 *>(a.lbuf);
  const float half = (float)(0.5 * a.inv_nx2);
  for (int idx = threadIdx.x; idx < P * d.NXH; idx += blockDim.x) {
    const int l = idx / d.NXH, km = idx - l * d.NXH;
    const size_t line = line0 + l;
    if (line >= nlines) continue;
    const int mc = (km == 0) ? 0 : d.NX2 - km;
    {
      const float2 zm = R[l * G::LS + km], zc = R[l * G::LS + mc];
      // Xa = (Z[m] + conj Z[-m]) / 2 ; Xb = (Z[m] - conj Z[-m]) / (2i)
      lb[line * d.NXH + km] = make_float2((zm.x + zc.x) * half, (zm.y - zc.y) * half);
      lb[fstride + line * d.NXH + km] = make_float2((zm.y + zc.y) * half, (zc.x - zm.x) * half);
    }
    {
      const float2 zm = R[(P + l / 2) * G::LS + km], zc = R[(P + l / 2) * G::LS + mc];
      const float2 val = (l & 1) ? make_float2((zm.y + zc.y) * half, (zc.x - zm.x) * half)
                                 : make_float2((zm.x + zc.x) * half, (zm.y - zc.y) * half);
      lb[2 * fstride + line * d.NXH + km] = val;
    }
  }
}

// Resident x blocks asked of the register allocator: four 144-thread blocks
// for the 24 x 24 factorisation (at most 113 registers a thread), else one.
template <int A, int B, int P> struct XMinBlocks { static constexpr int value = (A == 24 && B == 24) ? 4 : 1; };

template <int A, int B>
__global__ void __launch_bounds__(kRegTX * Line2<A, B>::T) k_zback_r(const __grid_constant__ XformArgs a) {
  zback_r_body<A, B>(a, blockIdx.x, blockIdx.y, blockIdx.z);
}
template <int A, int B>
__global__ void __launch_bounds__(kRegTX * Line2<A, B>::T) k_zfwd_r(const __grid_constant__ XformArgs a) {
  zfwd_r_body<A, B>(a, blockIdx.x, blockIdx.y, blockIdx.z);
}
// Shared memory of the persistent x pass: R (3P lines: transposes, physical
// lines, product pairs, their transposes and spectra), the input of one
// group (6 P NXH values), the twiddle table.
template <int A, int B, int P>
struct XSmem {
  using G = Line2<A, B>;
  static constexpr int R = 0, IN = 3 * P * G::LS, INSZ = 6 * P * (G::L / 3), TW = IN + INSZ, TOTAL = TW + G::L;
};

// The groups g0, g0 + step, ... < ngroups; `args(g)` gives the arguments and
// first line of group g (several channels in the batch).  The input of the
// next group is copied (cp.async) into the one input buffer as soon as
// every thread has read the current one, so it arrives while the current
// group is transformed.
template <int A, int B, int P, class Args>
__device__ __forceinline__ void xlamb_r_run(int g0, int step, int ngroups, const float2 *twsrc, Args args) {
  using S = XSmem<A, B, P>;
  static_assert((Line2<A, B>::L / 3) % 2 == 0, "16-byte staging needs NXH even");
  extern __shared__ __align__(16) unsigned char smraw[];
  float2 *sm = reinterpret_cast<float2 *>(smraw);
  float2 *tw = sm + S::TW;
  for (int k = threadIdx.x; k < Line2<A, B>::L; k += blockDim.x) tw[k] = twsrc[k];
  if (g0 < ngroups) {
    size_t line0;
    const XformArgs &a0 = args(g0, line0);
    xlamb_stage<P>(a0, line0, sm + S::IN);
  }
  cp_async_commit();
  for (int g = g0; g < ngroups; g += step) {
    cp_async_wait<0>();
    __syncthreads();
    size_t line0;
    const XformArgs &ag = args(g, line0);
    const int gn = g + step;
    xlamb_r_group<A, B, P>(ag, line0, sm + S::IN, sm + S::R, tw, [&] {
      if (gn < ngroups) {
        size_t nline0;
        const XformArgs &an = args(gn, nline0);
        xlamb_stage<P>(an, nline0, sm + S::IN);
      }
      cp_async_commit();
    });
  }
  cp_async_wait<0>();
}

template <int A, int B, int P>
__global__ void __launch_bounds__(3 * P * Line2<A, B>::T, XMinBlocks<A, B, P>::value) k_xlamb_r(const __grid_constant__ XformArgs a) {
  const int ngroups = (int)(((size_t)a.d.NY * a.d.NZ2 + P - 1) / P);
  const XformArgs *pa = &a;  // the kernel parameter itself (grid constant), not a copy
  xlamb_r_run<A, B, P>(blockIdx.x, gridDim.x, ngroups, reinterpret_cast<const float2 *>(a.twx),
                       [pa](int g, size_t &line0) -> const XformArgs & {
                         line0 = (size_t)g * P;
                         return *pa;
                       });
}
template <int A, int B>
__global__ void __launch_bounds__(kRegTX * Line2<A, B>::T) k_zback_r_batch(const __grid_constant__ BatchTable<XformArgs> t) {
  const int c = batch_channel(t.start, t.n, blockIdx.x);
  const XformArgs &a = t.a[c];
  const int gx = (a.d.NXH + kRegTX - 1) / kRegTX, lb = blockIdx.x - t.start[c], r = lb / gx;
  zback_r_body<A, B>(a, lb - r * gx, r % a.d.NY, r / a.d.NY);
}
template <int A, int B>
__global__ void __launch_bounds__(kRegTX * Line2<A, B>::T) k_zfwd_r_batch(const __grid_constant__ BatchTable<XformArgs> t) {
  const int c = batch_channel(t.start, t.n, blockIdx.x);
  const XformArgs &a = t.a[c];
  const int gx = (a.d.NXH + kRegTX - 1) / kRegTX, lb = blockIdx.x - t.start[c], r = lb / gx;
  zfwd_r_body<A, B>(a, lb - r * gx, r % a.d.NY, r / a.d.NY);
}
// Batched: the groups of every channel of the table (all with the same NX2),
// numbered channel by channel as the table's block offsets.
template <int A, int B, int P>
__global__ void __launch_bounds__(3 * P * Line2<A, B>::T, XMinBlocks<A, B, P>::value) k_xlamb_r_batch(const __grid_constant__ BatchTable<XformArgs> t) {
  xlamb_r_run<A, B, P>(blockIdx.x, gridDim.x, t.start[t.n], reinterpret_cast<const float2 *>(t.a[0].twx),
                       [&](int g, size_t &line0) -> const XformArgs & {
                         const int c = batch_channel(t.start, t.n, g);
                         line0 = (size_t)(g - t.start[c]) * P;
                         return t.a[c];
                       });
}

// Kernels, block sizes and shared memory of one line length.  P (y, z)
// lines per x block: 2 for the 24 x 24 factorisation, whose transforms keep
// ~130 registers per thread (three 144-thread blocks per SM), else 4.
template <int A, int B, int P>
static RegXformKernels reg_kernels_ab() {
  using G = Line2<A, B>;
  RegXformKernels k;
  k.zback = k_zback_r<A, B>;
  k.zfwd = k_zfwd_r<A, B>;
  k.xlamb = k_xlamb_r<A, B, P>;
  k.zback_b = k_zback_r_batch<A, B>;
  k.zfwd_b = k_zfwd_r_batch<A, B>;
  k.xlamb_b = k_xlamb_r_batch<A, B, P>;
  k.zthreads = kRegTX * G::T;
  k.xthreads = 3 * P * G::T;
  k.xlines = P;
  k.zsmem = ((size_t)kRegTX * G::LS + G::L) * sizeof(float2);
  k.xsmem = (size_t)XSmem<A, B, P>::TOTAL * sizeof(float2);
  // the persistent x pass runs exactly the resident blocks (found once)
  static int resident = 0;
  if (!resident) {
    int dev = 0, sms = 0, per = 0;
    if (raise_smem_limit(k.xlamb, k.xsmem) == cudaSuccess && raise_smem_limit(k.xlamb_b, k.xsmem) == cudaSuccess &&
        cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k.xlamb, k.xthreads, k.xsmem) == cudaSuccess && per > 0)
      resident = per * sms;
  }
  k.xgrid = resident > 0 ? resident : 1024;
  k.ok = true;
  return k;
}

RegXformKernels reg_xform_kernels(int L) {
  switch (L) {
    case 576: return reg_kernels_ab<24, 24, 2>();
    case 192: return reg_kernels_ab<16, 12, 4>();
    case 96: return reg_kernels_ab<12, 8, 4>();
    case 72: return reg_kernels_ab<9, 8, 4>();
    case 48: return reg_kernels_ab<8, 6, 4>();
    default: return RegXformKernels{};
  }
}

}  // namespace owt

// Device building blocks shared by the transform and solve kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "setup_host.h"  // kVKL, kVKU

namespace owt {

// Ring slot of history level 0 at step counter s (level l is (head + l) mod 3).
__device__ __forceinline__ int ring_head(long long s) { return (int)((2 * (s % 3)) % 3); }

// ---------------------------------------------------------------------------
// Complex values: double2 / float2 with the arithmetic the kernels need.
// ---------------------------------------------------------------------------
template <typename T> struct cpx_t;
template <> struct cpx_t<double> { using type = double2; };
template <> struct cpx_t<float> { using type = float2; };
template <typename T> using cpx = typename cpx_t<T>::type;

template <typename T> __host__ __device__ __forceinline__ cpx<T> mk(T x, T y) { cpx<T> r; r.x = x; r.y = y; return r; }
template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
// a * b
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
  C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
// a * conj(b)
template <typename C> __host__ __device__ __forceinline__ C cmulc(C a, C b) {
  C r; r.x = a.x * b.x + a.y * b.y; r.y = a.y * b.x - a.x * b.y; return r;
}


// ---------------------------------------------------------------------------
// FP64 -> FP32 conversion in integer instructions, for kernels that convert
// many values beside other kernels' hardware conversions: those run on the
// FP64 pipe, which on this part executes about two operations a clock per
// SM.  Ten integer operations or fewer, from the IEEE-754 bit layouts
// (binary64: sign, 11-bit exponent biased by 1023, 52-bit fraction; binary32:
// sign, 8-bit exponent biased by 127, 23-bit fraction): round to nearest,
// ties away from zero (the hardware's round-to-nearest-even differs only
// when the 29 dropped fraction bits are exactly 1 followed by zeros);
// magnitudes below 2^-126 (the smallest FP32 normal) become a signed zero;
// magnitudes at or above 2^128, and those that round up to it, become
// infinity; NaN stays NaN.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float d2f_bits(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned ah = hi & 0x7fffffffu;
  // exponent rebias 1023 -> 127 is 896 << 20 in the high word; the top 3
  // fraction bits of the low word complete the 23-bit fraction
  unsigned m = __funnelshift_l(lo, ah - (896u << 20), 3);
  m += (lo >> 28) & 1u;  // the first dropped bit: round half away from zero
  if (ah < (897u << 20)) m = 0u;
  if (ah >= (1151u << 20)) m = (ah > 0x7ff00000u || (ah == 0x7ff00000u && lo)) ? 0x7fc00000u : 0x7f800000u;
  return __uint_as_float(m | (hi & 0x80000000u));
}

// Complex values between the FP64 state and the FP32 transforms.
__device__ __forceinline__ double2 to_d(double2 a) { return a; }
__device__ __forceinline__ double2 to_d(float2 a) { return make_double2(a.x, a.y); }
template <typename T> __device__ __forceinline__ cpx<T> from_d(double2 a);
template <> __device__ __forceinline__ double2 from_d<double>(double2 a) { return a; }
template <> __device__ __forceinline__ float2 from_d<float>(double2 a) { return make_float2((float)a.x, (float)a.y); }

// ---------------------------------------------------------------------------
// FFT of many lines held in shared memory: self-sorting (Stockham) mixed-radix
// schedule with radices 4, 2, 3, 5.  At a stage of radix R after ns points have
// been combined, butterfly j (of L/R) reads x[j + r L/R], multiplies by
// w^(k r) with k = j mod ns and w = exp(sign 2 pi i / (ns R)), transforms, and
// writes y[(j / ns) ns R + k + r ns].  Twiddles come from one table of
// exp(-2 pi i m / L); the backward transform (sign +1) uses its conjugate.
// Unnormalised in both directions, like FFTW.
// ---------------------------------------------------------------------------
// A plan holds, per stage, the sizes the stage loop would otherwise divide out
// (nr = L/R butterflies, ns points combined before it, twiddle stride
// step = L/(ns R)) and multipliers ceil(2^32/d) for exact division by nr and
// ns with a multiply-high (exact for n d < 2^32; 0 marks d = 1).  Lines of at
// most 1024 points have at most 6 stages.
constexpr int kFftMaxStages = 8;
struct FftPlan {
  int L;
  int nst;
  int8_t R[kFftMaxStages];
  uint16_t nr[kFftMaxStages], ns[kFftMaxStages], step[kFftMaxStages];
  uint32_t mnr[kFftMaxStages], mns[kFftMaxStages];
};

// quotient n / d with the plan's multiplier m for d (m = 0: d = 1)
__device__ __forceinline__ int fft_div(int n, uint32_t m) { return m ? (int)__umulhi((unsigned)n, m) : n; }

inline uint32_t fft_magic(int d) { return d > 1 ? (uint32_t)((((uint64_t)1 << 32) + (uint64_t)d - 1) / (uint64_t)d) : 0u; }
// The plan for length L with the given stage radices (false if too many).
inline bool make_fft_plan(int L, const int *radices, int nst, FftPlan &p) {
  if (nst < 1 || nst > kFftMaxStages) return false;
  p = FftPlan{};
  p.L = L;
  p.nst = nst;
  int ns = 1;
  for (int s = 0; s < nst; ++s) {
    const int R = radices[s];
    p.R[s] = (int8_t)R;
    p.nr[s] = (uint16_t)(L / R);
    p.ns[s] = (uint16_t)ns;
    p.step[s] = (uint16_t)(L / (ns * R));
    p.mnr[s] = fft_magic(L / R);
    p.mns[s] = fft_magic(ns);
    ns *= R;
  }
  return ns == L;
}

// Position of point i of a line in shared memory.  FP32 lines (8-byte
// values, 16 per 128-byte wavefront) permute each aligned block of 16 by
// i ^ 5 ((i >> 4) & 3): the stride-R stores of the first two radix-4 stages
// then hit 16 different bank pairs per half-warp instead of 4, and runs of
// consecutive points stay conflict-free.  A line occupies whole blocks
// (line_stride).  FP64 lines are stored as they are: the same permutation
// over blocks of 8 (i ^ (g | (g & 2) << 1)) removes their conflicts too but
// measured slower, the FP64 kernels being FP64-pipe-bound.
template <typename T>
__device__ __forceinline__ int sw(int i) {
  if (sizeof(T) == sizeof(float)) return i ^ (5 * ((i >> 4) & 3));
  return i;
}
template <typename T>
__host__ __device__ __forceinline__ int line_stride(int L) {
  return (sizeof(T) == sizeof(float) ? (L + 15) / 16 * 16 : L) + 1;
}

template <typename T, bool BACKWARD>
__device__ __forceinline__ cpx<T> twiddle(const cpx<T> *__restrict__ tw, int idx) {
  cpx<T> w = tw[idx];
  if (BACKWARD) w.y = -w.y;
  return w;
}

template <typename T, bool BACKWARD, bool R5>
__device__ __forceinline__ void butterfly(const cpx<T> *src, cpx<T> *dst, int R, int j, int nr, int ns, int base,
                                          cpx<T> w1, cpx<T> w2, cpx<T> w3, cpx<T> w4, bool twid) {
  if (R == 4) {
    cpx<T> x0 = src[sw<T>(j)], x1 = src[sw<T>(j + nr)], x2 = src[sw<T>(j + 2 * nr)], x3 = src[sw<T>(j + 3 * nr)];
    if (twid) { x1 = cmul(x1, w1); x2 = cmul(x2, w2); x3 = cmul(x3, w3); }
    const cpx<T> t0 = cadd(x0, x2), t1 = csub(x0, x2), t2 = cadd(x1, x3);
    const cpx<T> d = csub(x1, x3);
    // t3 = d * (sign i): forward multiplies by -i, backward by +i
    const cpx<T> t3 = BACKWARD ? mk<T>(-d.y, d.x) : mk<T>(d.y, -d.x);
    dst[sw<T>(base)] = cadd(t0, t2);
    dst[sw<T>(base + ns)] = cadd(t1, t3);
    dst[sw<T>(base + 2 * ns)] = csub(t0, t2);
    dst[sw<T>(base + 3 * ns)] = csub(t1, t3);
  } else if (R == 2) {
    cpx<T> x0 = src[sw<T>(j)], x1 = src[sw<T>(j + nr)];
    if (twid) x1 = cmul(x1, w1);
    dst[sw<T>(base)] = cadd(x0, x1);
    dst[sw<T>(base + ns)] = csub(x0, x1);
  } else if (R5 && R == 5) {
    // DFT of length 5 from the sums and differences of the pairs (1, 4) and
    // (2, 3): y1,4 = a1 -+ sign i b1 and y2,3 = a2 -+ sign i b2 with
    // a1 = x0 + c1 t1 + c2 t2, a2 = x0 + c2 t1 + c1 t2,
    // b1 = s1 d1 + s2 d2, b2 = s2 d1 - s1 d2 (c_n, s_n = cos, sin 2 pi n / 5)
    cpx<T> x0 = src[sw<T>(j)], x1 = src[sw<T>(j + nr)], x2 = src[sw<T>(j + 2 * nr)], x3 = src[sw<T>(j + 3 * nr)],
           x4 = src[sw<T>(j + 4 * nr)];
    if (twid) { x1 = cmul(x1, w1); x2 = cmul(x2, w2); x3 = cmul(x3, w3); x4 = cmul(x4, w4); }
    const T c1 = (T)0.30901699437494742410229341718281906, c2 = (T)-0.80901699437494742410229341718281906;
    const T s1 = (T)0.95105651629515357211643933337938214, s2 = (T)0.58778525229247312916870595463907277;
    const cpx<T> t1 = cadd(x1, x4), t2 = cadd(x2, x3), d1 = csub(x1, x4), d2 = csub(x2, x3);
    const cpx<T> a1 = mk<T>(x0.x + c1 * t1.x + c2 * t2.x, x0.y + c1 * t1.y + c2 * t2.y);
    const cpx<T> a2 = mk<T>(x0.x + c2 * t1.x + c1 * t2.x, x0.y + c2 * t1.y + c1 * t2.y);
    const cpx<T> b1 = mk<T>(s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y);
    const cpx<T> b2 = mk<T>(s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y);
    // e = b * (-sign i): forward (-i) b = (b.y, -b.x), backward (+i) b = (-b.y, b.x)
    const cpx<T> e1 = BACKWARD ? mk<T>(-b1.y, b1.x) : mk<T>(b1.y, -b1.x);
    const cpx<T> e2 = BACKWARD ? mk<T>(-b2.y, b2.x) : mk<T>(b2.y, -b2.x);
    dst[sw<T>(base)] = cadd(x0, cadd(t1, t2));
    dst[sw<T>(base + ns)] = cadd(a1, e1);
    dst[sw<T>(base + 2 * ns)] = cadd(a2, e2);
    dst[sw<T>(base + 3 * ns)] = csub(a2, e2);
    dst[sw<T>(base + 4 * ns)] = csub(a1, e1);
  } else {  // R == 3
    cpx<T> x0 = src[sw<T>(j)], x1 = src[sw<T>(j + nr)], x2 = src[sw<T>(j + 2 * nr)];
    if (twid) { x1 = cmul(x1, w1); x2 = cmul(x2, w2); }
    const T s60 = (T)0.86602540378443864676372317075294;
    const cpx<T> t = cadd(x1, x2);
    const cpx<T> d = csub(x1, x2);
    const cpx<T> m = mk<T>(x0.x - (T)0.5 * t.x, x0.y - (T)0.5 * t.y);
    // u = d * (sign i sin60)
    const cpx<T> u = BACKWARD ? mk<T>(-s60 * d.y, s60 * d.x) : mk<T>(s60 * d.y, -s60 * d.x);
    dst[sw<T>(base)] = cadd(x0, t);
    dst[sw<T>(base + ns)] = cadd(m, u);
    dst[sw<T>(base + 2 * ns)] = csub(m, u);
  }
}

// nlines lines of length p.L, line q at a + q * lstride; result in the
// returned buffer (a or b).  Each thread owns one butterfly index j per stage
// and applies it to every (blockDim / (L/R))-th line, so index arithmetic and
// twiddle loads happen once per stage; a block of L threads keeps every thread
// busy for radix 2, 3 and 4 when nlines is a multiple of 12.
// R5 compiles in the radix-5 butterfly; a plan with a radix-5 stage needs it.
template <typename T, bool BACKWARD, bool R5>
__device__ cpx<T> *fft_lines(cpx<T> *a, cpx<T> *b, int nlines, int lstride, const FftPlan &p,
                             const cpx<T> *__restrict__ tw) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int s = 0; s < p.nst; ++s) {
    const int R = p.R[s], nr = p.nr[s], ns = p.ns[s], step = p.step[s];
    const uint32_t mnr = p.mnr[s], mns = p.mns[s];
    const int per = fft_div(nt, mnr);  // lines per pass
    if (per > 0) {
      if (tid < per * nr) {
        const int lo = fft_div(tid, mnr), j = tid - lo * nr;
        const int q = fft_div(j, mns), k = j - q * ns;
        const int base = q * ns * R + k;
        const bool twid = k != 0;
        cpx<T> w1 = mk<T>((T)1, (T)0), w2 = w1, w3 = w1, w4 = w1;
        if (twid) {
          w1 = twiddle<T, BACKWARD>(tw, k * step);
          if (R >= 3) w2 = twiddle<T, BACKWARD>(tw, 2 * k * step);
          if (R >= 4) w3 = twiddle<T, BACKWARD>(tw, 3 * k * step);
          if (R5 && R == 5) w4 = twiddle<T, BACKWARD>(tw, 4 * k * step);
        }
        for (int line = lo; line < nlines; line += per)
          butterfly<T, BACKWARD, R5>(a + line * lstride, b + line * lstride, R, j, nr, ns, base, w1, w2, w3, w4, twid);
      }
    } else {
      for (int idx = tid; idx < nlines * nr; idx += nt) {
        const int line = fft_div(idx, mnr), j = idx - line * nr;
        const int k = j - fft_div(j, mns) * ns;
        const bool twid = k != 0;
        cpx<T> w1 = mk<T>((T)1, (T)0), w2 = w1, w3 = w1, w4 = w1;
        if (twid) {
          w1 = twiddle<T, BACKWARD>(tw, k * step);
          if (R >= 3) w2 = twiddle<T, BACKWARD>(tw, 2 * k * step);
          if (R >= 4) w3 = twiddle<T, BACKWARD>(tw, 3 * k * step);
          if (R5 && R == 5) w4 = twiddle<T, BACKWARD>(tw, 4 * k * step);
        }
        butterfly<T, BACKWARD, R5>(a + line * lstride, b + line * lstride, R, j, nr, ns, (j - k) * R + k, w1, w2, w3, w4,
                               twid);
      }
    }
    __syncthreads();
    cpx<T> *tmp = a; a = b; b = tmp;
  }
  return a;
}

// Point mm of the complex line whose backward FFT is a + i b, for the
// spectra A, B (kx = 0 .. NXH-1) of two real lines: Hermitian extension in x
// (slot i = u_i, slot NX2 - i = conj u_i, FFT.cpp:109-119), the imaginary
// part of u_0 ignored (the real part of the reference's c2c output), slots
// NXH .. NX2-NXH zero (padding).  MAYBE_NO_B: B may be null (b = 0).
template <typename T, bool MAYBE_NO_B = false>
__device__ __forceinline__ cpx<T> hermitian_pair(const cpx<T> *A, const cpx<T> *B, int mm, int NXH, int NX2) {
  const cpx<T> zero = mk<T>((T)0, (T)0);
  const bool hb = !MAYBE_NO_B || B != nullptr;
  if (mm == 0) return mk<T>(A[0].x, hb ? B[0].x : (T)0);
  if (mm < NXH) {
    const cpx<T> x = A[mm], y = hb ? B[mm] : zero;
    return mk<T>(x.x - y.y, x.y + y.x);
  }
  if (mm > NX2 - NXH) {
    const int mp = NX2 - mm;
    const cpx<T> x = A[mp], y = hb ? B[mp] : zero;
    return mk<T>(x.x + y.y, y.x - x.y);
  }
  return zero;
}

// Value helpers so the band solves run on one real component (double) or a
// complex value (double2) per thread.
__host__ __device__ __forceinline__ void fms(double &w, double l, double y) { w -= l * y; }
__host__ __device__ __forceinline__ void fms(double2 &w, double l, double2 y) { w.x -= l * y.x; w.y -= l * y.y; }
__host__ __device__ __forceinline__ double scal(double w, double r) { return w * r; }
__host__ __device__ __forceinline__ double2 scal(double2 w, double r) { return make_double2(w.x * r, w.y * r); }
template <class V> __host__ __device__ __forceinline__ V vzero();
template <> __host__ __device__ __forceinline__ double vzero<double>() { return 0.0; }
template <> __host__ __device__ __forceinline__ double2 vzero<double2>() { return make_double2(0.0, 0.0); }

// ---------------------------------------------------------------------------
// Banded LU solve, the algorithm of LAPACK dgbtrs ('N') on factors produced by
// the dgbtf2 algorithm (see k_band_factor): forward sweep applying the row
// interchanges and unit-lower multipliers column by column, then the upper
// band back substitution.  Band storage AB[b][c][u] in LAPACK's factorization
// layout (kv = KL + KU: row kv holds the diagonal, rows kv - t the t-th super-
// diagonal of U, rows kv + t the multipliers of L), one system per unique
// mode u, unique mode fastest so that neighbouring threads read neighbouring
// words.  The diagonal row holds 1/U_jj (stored by the factorization).
//
// Each thread solves one complex right-hand side.  The active window of the
// right-hand side lives in registers as a ring whose slot for entry j + t is
// (s + t) mod W at unrolled step s, so all register indices are compile-time.
//   rhs(p)      : entry p of the right-hand side (complex)
//   ystore(p,v) : keep the forward-swept entry p (read back in reverse)
//   yload(p)    : read it back
//   out(c, x)   : solution entry for column c, produced for c = n-1 .. 0
// ---------------------------------------------------------------------------
template <int KL, int KU, class Rhs, class YStore, class YLoad, class Out>
__host__ __device__ __forceinline__ void band_solve(const double *__restrict__ ab, const uint8_t *__restrict__ piv, int n,
                                           int U, int u, Rhs rhs, YStore ystore, YLoad yload, Out out) {
  using V = decltype(rhs(0));
  constexpr int KV = KL + KU;
  constexpr int W = KL + 1;
  const size_t sn = (size_t)n * U;  // stride between band rows
  {
    V w[W];
#pragma unroll
    for (int t = 0; t < W; ++t) w[t] = (t < n) ? rhs(t) : vzero<V>();
    for (int j0 = 0; j0 < n; j0 += W) {
#pragma unroll
      for (int s = 0; s < W; ++s) {
        const int j = j0 + s;
        if (j < n) {
          const int off = piv[(size_t)j * U + u];
#pragma unroll
          for (int t = 1; t < W; ++t) {
            if (off == t) {
              const V tmp = w[s];
              w[s] = w[(s + t) % W];
              w[(s + t) % W] = tmp;
            }
          }
          const V yj = w[s];
          ystore(j, yj);
          const double *col = ab + (size_t)j * U + u;
#pragma unroll
          for (int t = 1; t < W; ++t) fms(w[(s + t) % W], col[(size_t)(KV + t) * sn], yj);
          w[s] = (j + W < n) ? rhs(j + W) : vzero<V>();
        }
      }
    }
  }
  {
    constexpr int WB = KV + 1;
    V w[WB];
#pragma unroll
    for (int t = 0; t < WB; ++t) w[t] = (n - 1 - t >= 0) ? yload(n - 1 - t) : vzero<V>();
    for (int jj = 0; jj < n; jj += WB) {
#pragma unroll
      for (int s = 0; s < WB; ++s) {
        const int j = n - 1 - (jj + s);
        if (j >= 0) {
          const double *col = ab + (size_t)j * U + u;
          const V x = scal(w[s], col[(size_t)KV * sn]);
          out(j, x);
#pragma unroll
          for (int t = 1; t < WB; ++t) fms(w[(s + t) % WB], col[(size_t)(KV - t) * sn], x);
          w[s] = (j - WB >= 0) ? yload(j - WB) : vzero<V>();
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// The same solve skipping the entries of L and U that are structurally zero in
// interior columns.  Unknowns are interleaved by node, NT per interior node
// (column c is unknown type (c + OFF) mod NT); after partial pivoting the
// nonzero offsets of an interior column depend only on its type.  The masks
// are the union over wavenumbers, grid sizes, time steps, viscosities and
// stretchings, found by factorising the band templates on the host over such
// a sweep; every factorization is checked against them
// (k_check_pattern) and the full-band solve is used if any mode falls
// outside.  The first Masks::lo and the last Masks::hi columns keep the
// boundary closures' own fill and are swept with the full band: the widths
// are those beyond which the sweep found every column inside its type's masks
// (v-system, both orders: columns up to 41 from the bottom and 30 from the
// top lie outside; the omega_y-system 11 and 9), rounded up.
// Register rings are padded to multiples of NT so that the unknown type
// of every unrolled step is a compile-time constant (n is a multiple of NT).
// Mask bit t set: L[c+t][c] may be nonzero (forward), U[c-t][c] (backward),
// row interchange with offset t may occur (pivots).
// ---------------------------------------------------------------------------
// v-system (d3, d2, d1, v per interior node, types 0..3 in that order):
// 21.5 entries per column instead of 46 (the reference's eighth-order
// operators; the sixth-order option has masks of its own, vmask6_* / VMasks6
// below, checked at setup by launch_check_pattern with type 2)
__host__ __device__ constexpr unsigned long long vmask_l(int ty) {
  return ty == 0 ? 0xcfeull : ty == 1 ? 0x6feull : ty == 2 ? 0x3feull : 0x19feull;
}
__host__ __device__ constexpr unsigned long long vmask_u(int ty) {
  return ty == 0 ? 0x1ffeull : ty == 1 ? 0x7feull : ty == 2 ? 0x1feull : 0xffffeull;
}
// pivot offsets that occur in interior columns (bit t: offset t; 0 is free)
__host__ __device__ constexpr unsigned long long vmask_p(int ty) {
  return ty == 0 ? 0x44ull : ty == 1 ? 0x26ull : ty == 2 ? 0x12ull : 0xaull;
}
// omega_y-system (d1, d2 per node): 9 entries per column instead of 18, and
// no row interchange in interior columns
__host__ __device__ constexpr unsigned long long gmask_l(int ty) { return ty == 0 ? 0x3eull : 0x1eull; }
__host__ __device__ constexpr unsigned long long gmask_u(int ty) { return ty == 0 ? 0x1eull : 0x3eull; }
struct VMasks {
  static constexpr int lo = 44, hi = 32;
  __host__ __device__ static constexpr unsigned long long l(int ty) { return vmask_l(ty); }
  __host__ __device__ static constexpr unsigned long long u(int ty) { return vmask_u(ty); }
  __host__ __device__ static constexpr unsigned long long p(int ty) { return vmask_p(ty); }
};
// The sixth-order option (fd_order = 6) fills differently; its masks come
// from the same derivation over the same sweep.
__host__ __device__ constexpr unsigned long long vmask6_l(int ty) {
  return ty == 0 ? 0xcfeull : ty == 1 ? 0x67eull : ty == 2 ? 0x33eull : 0x19feull;
}
__host__ __device__ constexpr unsigned long long vmask6_u(int ty) {
  return ty == 0 ? 0x1feull : ty == 1 ? 0x7eull : ty == 2 ? 0x3eull : 0xffffeull;
}
__host__ __device__ constexpr unsigned long long vmask6_p(int ty) {
  return ty == 0 ? 0x44ull : ty == 1 ? 0x4ull : ty == 2 ? 0x10ull : 0xcull;
}
struct VMasks6 {
  static constexpr int lo = 44, hi = 32;
  __host__ __device__ static constexpr unsigned long long l(int ty) { return vmask6_l(ty); }
  __host__ __device__ static constexpr unsigned long long u(int ty) { return vmask6_u(ty); }
  __host__ __device__ static constexpr unsigned long long p(int ty) { return vmask6_p(ty); }
};
struct GMasks {
  static constexpr int lo = 16, hi = 16;
  __host__ __device__ static constexpr unsigned long long l(int ty) { return gmask_l(ty); }
  __host__ __device__ static constexpr unsigned long long u(int ty) { return gmask_u(ty); }
  __host__ __device__ static constexpr unsigned long long p(int) { return 0ull; }
};

// The forward sweep (row interchanges and L) and the backward sweep (U) of
// band_solve_masked, which exchange the forward-swept values only through
// ystore / yload; a caller may run other work between them.
template <int KL, int KU, int NT, int OFF, int W, class Masks, class Rhs, class YStore>
__host__ __device__ __forceinline__ void band_forward_masked(const double *__restrict__ ab, const uint8_t *__restrict__ piv,
                                                    int n, int U, int u, Rhs rhs, YStore ystore) {
  static_assert(W >= KL + 1 && W % NT == 0, "ring size");
  using V = decltype(rhs(0));
  constexpr int KV = KL + KU;
  const size_t sn = (size_t)n * U;
  {
    V w[W];
#pragma unroll
    for (int t = 0; t < W; ++t) w[t] = (t < n) ? rhs(t) : vzero<V>();
    for (int j0 = 0; j0 < n; j0 += W) {
      const bool sparse = (j0 >= Masks::lo) && (j0 + W - 1 < n - Masks::hi);
#pragma unroll
      for (int s = 0; s < W; ++s) {
        const int j = j0 + s;
        if (j < n) {
          const int off = piv[(size_t)j * U + u];
          // only the offsets that occur in interior columns are tested there
#pragma unroll
          for (int t = 1; t <= KL; ++t) {
            if ((!sparse || ((Masks::p((s + OFF) % NT) >> t) & 1ull)) && off == t) {
              const V tmp = w[s];
              w[s] = w[(s + t) % W];
              w[(s + t) % W] = tmp;
            }
          }
          const V yj = w[s];
          ystore(j, yj);
          const double *col = ab + (size_t)j * U + u;
          if (sparse) {
#pragma unroll
            for (int t = 1; t <= KL; ++t)
              if ((Masks::l((s + OFF) % NT) >> t) & 1ull) fms(w[(s + t) % W], col[(size_t)(KV + t) * sn], yj);
          } else {
#pragma unroll
            for (int t = 1; t <= KL; ++t) fms(w[(s + t) % W], col[(size_t)(KV + t) * sn], yj);
          }
          w[s] = (j + W < n) ? rhs(j + W) : vzero<V>();
        }
      }
    }
  }
}
template <int KL, int KU, int NT, int OFF, int WB, class Masks, class V, class YLoad, class Out>
__host__ __device__ __forceinline__ void band_backward_masked(const double *__restrict__ ab, int n, int U, int u, YLoad yload,
                                                     Out out) {
  static_assert(WB >= KL + KU + 1 && WB % NT == 0, "ring size");
  constexpr int KV = KL + KU;
  const size_t sn = (size_t)n * U;
  {
    V w[WB];
#pragma unroll
    for (int t = 0; t < WB; ++t) w[t] = (n - 1 - t >= 0) ? yload(n - 1 - t) : vzero<V>();
    for (int jj = 0; jj < n; jj += WB) {
      // columns n-1-jj .. n-1-jj-(WB-1); the type of column n-1-jj-s is
      // (OFF - 1 - s) mod NT
      const bool sparse = (n - 1 - jj < n - Masks::hi) && (n - 1 - jj - (WB - 1) >= Masks::lo);
#pragma unroll
      for (int s = 0; s < WB; ++s) {
        const int j = n - 1 - (jj + s);
        if (j >= 0) {
          const double *col = ab + (size_t)j * U + u;
          const V x = scal(w[s], col[(size_t)KV * sn]);
          out(j, x);
          if (sparse) {
#pragma unroll
            for (int t = 1; t <= KV; ++t)
              if ((Masks::u((OFF - 1 - s % NT + 2 * NT) % NT) >> t) & 1ull)
                fms(w[(s + t) % WB], col[(size_t)(KV - t) * sn], x);
          } else {
#pragma unroll
            for (int t = 1; t <= KV; ++t) fms(w[(s + t) % WB], col[(size_t)(KV - t) * sn], x);
          }
          w[s] = (j - WB >= 0) ? yload(j - WB) : vzero<V>();
        }
      }
    }
  }
}

// The backward sweep with two register rings: the full-band columns near the
// walls need the whole upper band (KL + KU + 1 values in flight), the masked
// interior only its deepest upper offset + 1 (WBI; 20 against 32 for the
// v-system), and the smaller ring is what keeps the mode kernel within 128
// registers without spilling.  Phase T: chunks of WBE columns from the top
// while they are not all interior; phase I: chunks of WBI interior columns;
// phase B: the rest in chunks of WBE.  Between phases the rows in flight move
// ring to ring with compile-time slots; rows of the larger ring that the
// smaller one cannot hold go back to the forward-swept values in memory
// (ystore) with their pending updates, and are read again (yload) when they
// enter the window: an interior column updates no row further than WBI - 1
// below it.  Same operations in the same order as band_backward_masked.
template <class Masks, int NT>
__host__ __device__ constexpr int masks_u_reach() {
  int r = 0;
  for (int ty = 0; ty < NT; ++ty)
    for (int t = 1; t < 64; ++t)
      if ((Masks::u(ty) >> t) & 1ull) r = t > r ? t : r;
  return r;
}
template <int KL, int KU, int NT, int OFF, int WBI, class Masks, class V, class YLoad, class YStore, class Out>
__host__ __device__ __forceinline__ void band_backward_masked2(const double *__restrict__ ab, int n, int U, int u, YLoad yload,
                                                      YStore ystore, Out out) {
  constexpr int KV = KL + KU;
  constexpr int WBE = (KV + 1 + NT - 1) / NT * NT;
  static_assert(WBI % NT == 0 && WBI < WBE, "ring sizes");
  static_assert(masks_u_reach<Masks, NT>() < WBI, "interior ring shorter than the masks' upper reach");
  const size_t sn = (size_t)n * U;
  // column j at unrolled step s of a chunk that starts a multiple of NT below
  // n - 1 (n is a multiple of NT): type (OFF - 1 - s) mod NT; ring of R slots
  auto column = [&](auto ring, auto masked, int s, int j, auto &w) {
    constexpr int R = decltype(ring)::value;
    const double *col = ab + (size_t)j * U + u;
    const V x = scal(w[s], col[(size_t)KV * sn]);
    out(j, x);
    if constexpr (decltype(masked)::value) {
#pragma unroll
      for (int t = 1; t < R; ++t)
        if ((Masks::u((OFF - 1 - s % NT + 2 * NT) % NT) >> t) & 1ull)
          fms(w[(s + t) % R], col[(size_t)(KV - t) * sn], x);
    } else {
      static_assert(R > KV, "a full-band column needs the full ring");
#pragma unroll
      for (int t = 1; t <= KV; ++t) fms(w[(s + t) % R], col[(size_t)(KV - t) * sn], x);
    }
    w[s] = (j - R >= 0) ? yload(j - R) : vzero<V>();
  };
  using E = std::integral_constant<int, WBE>;
  using I = std::integral_constant<int, WBI>;
  using Masked = std::true_type;
  using Full = std::false_type;
  auto interior = [&](int top, int len) { return top < n - Masks::hi && top - (len - 1) >= Masks::lo; };
  int jj = 0;  // columns done, from the top
  V we[WBE];
#pragma unroll
  for (int t = 0; t < WBE; ++t) we[t] = (n - 1 - t >= 0) ? yload(n - 1 - t) : vzero<V>();
  // phase T: full-ring chunks until an interior-ring chunk would be all interior
  for (; jj < n && !interior(n - 1 - jj, WBI); jj += WBE) {
    if (interior(n - 1 - jj, WBE)) {
#pragma unroll
      for (int s = 0; s < WBE; ++s) column(E{}, Masked{}, s, n - 1 - (jj + s), we);
    } else {
#pragma unroll
      for (int s = 0; s < WBE; ++s)
        if (n - 1 - (jj + s) >= 0) column(E{}, Full{}, s, n - 1 - (jj + s), we);
    }
  }
  if (jj >= n) return;
  // to the interior ring: row n-1-jj-s in slot s; the deeper rows back to memory
  V wi[WBI];
#pragma unroll
  for (int t = 0; t < WBI; ++t) wi[t] = we[t];
#pragma unroll
  for (int t = WBI; t < WBE; ++t)
    if (n - 1 - jj - t >= 0) ystore(n - 1 - jj - t, we[t]);
  // phase I
  for (; jj < n && interior(n - 1 - jj, WBI); jj += WBI) {
#pragma unroll
    for (int s = 0; s < WBI; ++s) column(I{}, Masked{}, s, n - 1 - (jj + s), wi);
  }
  if (jj >= n) return;
  // back to the full ring for the bottom columns
#pragma unroll
  for (int t = 0; t < WBI; ++t) we[t] = wi[t];
#pragma unroll
  for (int t = WBI; t < WBE; ++t) we[t] = (n - 1 - jj - t >= 0) ? yload(n - 1 - jj - t) : vzero<V>();
  // phase B
  for (; jj < n; jj += WBE) {
#pragma unroll
    for (int s = 0; s < WBE; ++s)
      if (n - 1 - (jj + s) >= 0) column(E{}, Full{}, s, n - 1 - (jj + s), we);
  }
}

template <int KL, int KU, int NT, int OFF, int W, int WB, class Masks, class Rhs, class YStore,
          class YLoad, class Out>
__host__ __device__ __forceinline__ void band_solve_masked(const double *__restrict__ ab, const uint8_t *__restrict__ piv,
                                                  int n, int U, int u, Rhs rhs, YStore ystore, YLoad yload,
                                                  Out out) {
  using V = decltype(rhs(0));
  band_forward_masked<KL, KU, NT, OFF, W, Masks>(ab, piv, n, U, u, rhs, ystore);
  band_backward_masked<KL, KU, NT, OFF, WB, Masks, V>(ab, n, U, u, yload, out);
}

// VM: VMasks (the reference's eighth-order operators) or VMasks6
template <class VM = VMasks, class Rhs, class YStore, class YLoad, class Out>
__host__ __device__ __forceinline__ void band_solve_v_sparse(const double *__restrict__ ab, const uint8_t *__restrict__ piv,
                                                    int n, int U, int u, Rhs rhs, YStore ystore, YLoad yload,
                                                    Out out) {
  band_solve_masked<kVKL, kVKU, 4, 2, 16, 32, VM>(ab, piv, n, U, u, rhs, ystore, yload, out);
}
template <class VM = VMasks, class Rhs, class YStore>
__host__ __device__ __forceinline__ void band_forward_v_sparse(const double *__restrict__ ab, const uint8_t *__restrict__ piv,
                                                      int n, int U, int u, Rhs rhs, YStore ystore) {
  band_forward_masked<kVKL, kVKU, 4, 2, 16, VM>(ab, piv, n, U, u, rhs, ystore);
}
template <class VM = VMasks, class YLoad, class YStore, class Out>
__host__ __device__ __forceinline__ void band_backward_v_sparse(const double *__restrict__ ab, int n, int U, int u,
                                                       YLoad yload, YStore ystore, Out out) {
  band_backward_masked2<kVKL, kVKU, 4, 2, 20, VM, double>(ab, n, U, u, yload, ystore, out);
}
template <class Rhs, class YStore, class YLoad, class Out>
__host__ __device__ __forceinline__ void band_solve_g_sparse(const double *__restrict__ ab, const uint8_t *__restrict__ piv,
                                                    int n, int U, int u, Rhs rhs, YStore ystore, YLoad yload,
                                                    Out out) {
  band_solve_masked<6, 6, 2, 0, 8, 14, GMasks>(ab, piv, n, U, u, rhs, ystore, yload, out);
}

// ---------------------------------------------------------------------------
// Transposed solve A^T x = b on the factors of band_solve (the order of LAPACK
// dgbtrs with trans = 'T'): U^T y = b by forward substitution, then for
// j = n-1 .. 0: b_j -= sum_i L(j+i, j) b_(j+i) and undo row interchange j.
// Band entries outside the matrix are zero in the factorization layout, so
// the rings start at zero and need no edge tests.
//   rhs(p)      : entry p of b, requested for p = 0 .. n-1
//   ystore/yload: scratch for y
//   out(c, x)   : solution entry c, produced for c = n-1 .. 0
// ---------------------------------------------------------------------------
template <int KL, int KU, class Rhs, class YStore, class YLoad, class Out>
__host__ __device__ __forceinline__ void band_solve_t(const double *__restrict__ ab, const uint8_t *__restrict__ piv, int n,
                                             int U, int u, Rhs rhs, YStore ystore, YLoad yload, Out out) {
  using V = decltype(rhs(0));
  constexpr int KV = KL + KU;
  const size_t sn = (size_t)n * U;
  {
    // y_j = (b_j - sum_t U(j-t, j) y_(j-t)) / U(j, j); y_(j-t) in slot (s - t) mod W
    constexpr int W = KV + 1;
    V w[W];
#pragma unroll
    for (int t = 0; t < W; ++t) w[t] = vzero<V>();
    for (int j0 = 0; j0 < n; j0 += W) {
#pragma unroll
      for (int s = 0; s < W; ++s) {
        const int j = j0 + s;
        if (j < n) {
          const double *col = ab + (size_t)j * U + u;
          V acc = rhs(j);
#pragma unroll
          for (int t = 1; t <= KV; ++t) fms(acc, col[(size_t)(KV - t) * sn], w[(s - t + W) % W]);
          acc = scal(acc, col[(size_t)KV * sn]);
          w[s] = acc;
          ystore(j, acc);
        }
      }
    }
  }
  {
    // window b_j .. b_(j+KL): entry j + i in slot (s - i) mod W at the step of
    // column j = n-1 - (jj + s); entry j + KL is final once column j is done
    constexpr int W = KL + 1;
    V w[W];
#pragma unroll
    for (int t = 0; t < W; ++t) w[t] = vzero<V>();
    for (int jj = 0; jj < n + KL; jj += W) {
#pragma unroll
      for (int s = 0; s < W; ++s) {
        const int j = n - 1 - (jj + s);
        if (j >= 0) {
          const double *col = ab + (size_t)j * U + u;
          V acc = yload(j);
#pragma unroll
          for (int i = 1; i <= KL; ++i) fms(acc, col[(size_t)(KV + i) * sn], w[(s - i + W) % W]);
          w[s] = acc;
          const int off = piv[(size_t)j * U + u];
#pragma unroll
          for (int i = 1; i <= KL; ++i) {
            if (off == i) {
              const V tmp = w[s];
              w[s] = w[(s - i + W) % W];
              w[(s - i + W) % W] = tmp;
            }
          }
        } else {
          w[s] = vzero<V>();
        }
        const int c = j + KL;
        if (c >= 0 && c < n) out(c, w[(s + 1) % W]);
      }
    }
  }
}


// The transposed solve with the interior columns of the factors restricted
// to the fill and interchange masks of their type (Masks, column type
// (c + OFF) mod NT), as band_solve_masked does for the solve itself: a ring
// chunk whose columns all lie between the full-band edges (Masks::lo,
// Masks::hi) skips the entries outside its columns' masks, which are exact
// zeros in every factorization the setup check admits, so the result is
// bitwise that of band_solve_t.  Needs n a multiple of NT (the column types
// of the backward pass are then compile-time constants).
template <int KL, int KU, int NT, int OFF, class Masks, class Rhs, class YStore, class YLoad, class Out>
__host__ __device__ __forceinline__ void band_solve_t_masked(const double *__restrict__ ab, const uint8_t *__restrict__ piv,
                                                    int n, int U, int u, Rhs rhs, YStore ystore, YLoad yload,
                                                    Out out) {
  using V = decltype(rhs(0));
  constexpr int KV = KL + KU;
  const size_t sn = (size_t)n * U;
  {
    // U^T y = b: column j's entries U(j - t, j), t in its type's upper mask
    constexpr int W = KV + 1;
    static_assert(W % NT == 0, "ring size");
    V w[W];
#pragma unroll
    for (int t = 0; t < W; ++t) w[t] = vzero<V>();
    for (int j0 = 0; j0 < n; j0 += W) {
      const bool sparse = (j0 >= Masks::lo) && (j0 + W - 1 < n - Masks::hi);
#pragma unroll
      for (int s = 0; s < W; ++s) {
        const int j = j0 + s;
        if (j < n) {
          const double *col = ab + (size_t)j * U + u;
          V acc = rhs(j);
          if (sparse) {
#pragma unroll
            for (int t = 1; t <= KV; ++t)
              if ((Masks::u((s + OFF) % NT) >> t) & 1ull) fms(acc, col[(size_t)(KV - t) * sn], w[(s - t + W) % W]);
          } else {
#pragma unroll
            for (int t = 1; t <= KV; ++t) fms(acc, col[(size_t)(KV - t) * sn], w[(s - t + W) % W]);
          }
          acc = scal(acc, col[(size_t)KV * sn]);
          w[s] = acc;
          ystore(j, acc);
        }
      }
    }
  }
  {
    // L^T and the interchanges, j = n-1 .. 0; with n and jj multiples of NT
    // the type of column j = n-1 - (jj + s) is (OFF - 1 - s) mod NT
    constexpr int W = KL + 1;
    static_assert(W % NT == 0, "ring size");
    V w[W];
#pragma unroll
    for (int t = 0; t < W; ++t) w[t] = vzero<V>();
    for (int jj = 0; jj < n + KL; jj += W) {
      const bool sparse = (n - 1 - jj - (W - 1) >= Masks::lo) && (n - 1 - jj < n - Masks::hi);
#pragma unroll
      for (int s = 0; s < W; ++s) {
        const int ty = (((OFF - 1 - s) % NT) + NT) % NT;
        const int j = n - 1 - (jj + s);
        if (j >= 0) {
          const double *col = ab + (size_t)j * U + u;
          V acc = yload(j);
          if (sparse) {
#pragma unroll
            for (int i = 1; i <= KL; ++i)
              if ((Masks::l(ty) >> i) & 1ull) fms(acc, col[(size_t)(KV + i) * sn], w[(s - i + W) % W]);
          } else {
#pragma unroll
            for (int i = 1; i <= KL; ++i) fms(acc, col[(size_t)(KV + i) * sn], w[(s - i + W) % W]);
          }
          w[s] = acc;
          const int off = piv[(size_t)j * U + u];
#pragma unroll
          for (int i = 1; i <= KL; ++i) {
            if ((!sparse || ((Masks::p(ty) >> i) & 1ull)) && off == i) {
              const V tmp = w[s];
              w[s] = w[(s - i + W) % W];
              w[(s - i + W) % W] = tmp;
            }
          }
        } else {
          w[s] = vzero<V>();
        }
        const int c = j + KL;
        if (c >= 0 && c < n) out(c, w[(s + 1) % W]);
      }
    }
  }
}
}  // namespace owt

// Discrete Fourier transforms of a few points held in registers, with every
// index and every internal twiddle factor a compile-time constant.
//
// dft<N, BACKWARD>(x) transforms x[0..N) in place (unnormalised, sign -1
// forward and +1 backward, as FFTW): N = 2, 3, 4, 5 are written out; larger N
// split as N = R M (R the first of 4, 3, 2, 5 dividing N) by decimation in
// time: the R sub-sequences x[r + R m] are transformed (length M), each
// output k1 of sub-sequence r is multiplied by w_N^(r k1), and the R values
// of each k1 are combined by a length-R transform into outputs k1 + M k2.
// The twiddle constants are cos and sin of 2 pi e / N evaluated at compile
// time (angle reduced to [0, pi/4] with integer arithmetic, then Taylor
// series to x^27 in double), then rounded to the arithmetic type.
//
// Two-pass transforms of a line of length L = A B (used by the transform
// kernels) are built from these: A-point transforms of the B interleaved
// sub-sequences x[b + B a], the twiddle w_L^(b a'), then B-point transforms.
#pragma once
#include <cuda_runtime.h>

#include <type_traits>
#include <utility>

#include "owt_device.cuh"

namespace owt {
namespace ct {

constexpr double kPi = 3.14159265358979323846264338327950288;

__host__ __device__ constexpr double sin_small(double x) {
  double x2 = x * x, term = x, sum = x;
  for (int n = 1; n <= 13; ++n) {
    term *= -x2 / (double)((2 * n) * (2 * n + 1));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double cos_small(double x) {
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int n = 1; n <= 13; ++n) {
    term *= -x2 / (double)((2 * n - 1) * (2 * n));
    sum += term;
  }
  return sum;
}
// (cos, sin) of 2 pi k / n: octant o = floor(8 k / n) and remainder r give
// the angle o pi/4 + (pi/4) r/n; odd octants use the complement
// (pi/4)(n - r)/n so that the series argument stays in [0, pi/4].
struct CS {
  double c, s;
};
__host__ __device__ constexpr CS cs2pi(long k, long n) {
  k %= n;
  if (k < 0) k += n;
  const long o = (8 * k) / n, r = 8 * k - o * n;
  const long q = o / 2;
  const bool odd = (o & 1) != 0;
  const double a = odd ? (kPi / 4) * (double)(n - r) / (double)n : (kPi / 4) * (double)r / (double)n;
  const double c0 = odd ? sin_small(a) : cos_small(a);
  const double s0 = odd ? cos_small(a) : sin_small(a);
  if (q == 0) return CS{c0, s0};
  if (q == 1) return CS{-s0, c0};
  if (q == 2) return CS{-c0, -s0};
  return CS{s0, -c0};
}

}  // namespace ct

// Call f(std::integral_constant<int, I>) for I = B .. E-1.
template <int B, int E, class F>
__host__ __device__ __forceinline__ void static_for(F &&f) {
  if constexpr (B < E) {
    f(std::integral_constant<int, B>{});
    static_for<B + 1, E>(f);
  }
}

// x * w_N^E, w_N = exp(sign 2 pi i / N), sign -1 forward, +1 backward.
template <int E, int N, bool BACKWARD, typename T>
__host__ __device__ __forceinline__ cpx<T> twc(cpx<T> x) {
  constexpr int e = ((E % N) + N) % N;
  if constexpr (e == 0) {
    return x;
  } else if constexpr (2 * e == N) {
    return mk<T>(-x.x, -x.y);
  } else if constexpr (4 * e == N) {  // forward -i, backward +i
    return BACKWARD ? mk<T>(-x.y, x.x) : mk<T>(x.y, -x.x);
  } else if constexpr (4 * e == 3 * N) {  // forward +i, backward -i
    return BACKWARD ? mk<T>(x.y, -x.x) : mk<T>(-x.y, x.x);
  } else {
    constexpr ct::CS w = ct::cs2pi(e, N);
    constexpr T c = (T)w.c;
    constexpr T s = (T)(BACKWARD ? w.s : -w.s);
    return mk<T>(x.x * c - x.y * s, x.x * s + x.y * c);
  }
}

template <int N> struct FirstRadix {
  static constexpr int value = (N % 4 == 0) ? 4 : (N % 3 == 0) ? 3 : (N % 2 == 0) ? 2 : (N % 5 == 0) ? 5 : N;
};

template <int N, bool BACKWARD, typename T>
__host__ __device__ __forceinline__ void dft(cpx<T> *x) {
  if constexpr (N == 1) {
    return;
  } else if constexpr (N == 2) {
    const cpx<T> a = x[0], b = x[1];
    x[0] = cadd(a, b);
    x[1] = csub(a, b);
  } else if constexpr (N == 4) {
    const cpx<T> t0 = cadd(x[0], x[2]), t1 = csub(x[0], x[2]), t2 = cadd(x[1], x[3]), d = csub(x[1], x[3]);
    const cpx<T> t3 = BACKWARD ? mk<T>(-d.y, d.x) : mk<T>(d.y, -d.x);
    x[0] = cadd(t0, t2);
    x[1] = cadd(t1, t3);
    x[2] = csub(t0, t2);
    x[3] = csub(t1, t3);
  } else if constexpr (N == 3) {
    constexpr T s60 = (T)0.86602540378443864676372317075294;
    const cpx<T> t = cadd(x[1], x[2]), d = csub(x[1], x[2]);
    const cpx<T> m = mk<T>(x[0].x - (T)0.5 * t.x, x[0].y - (T)0.5 * t.y);
    const cpx<T> u = BACKWARD ? mk<T>(-s60 * d.y, s60 * d.x) : mk<T>(s60 * d.y, -s60 * d.x);
    x[0] = cadd(x[0], t);
    x[1] = cadd(m, u);
    x[2] = csub(m, u);
  } else if constexpr (N == 5) {
    constexpr T c1 = (T)0.30901699437494742410229341718281906, c2 = (T)-0.80901699437494742410229341718281906;
    constexpr T s1 = (T)0.95105651629515357211643933337938214, s2 = (T)0.58778525229247312916870595463907277;
    const cpx<T> x0 = x[0];
    const cpx<T> t1 = cadd(x[1], x[4]), t2 = cadd(x[2], x[3]), d1 = csub(x[1], x[4]), d2 = csub(x[2], x[3]);
    const cpx<T> a1 = mk<T>(x0.x + c1 * t1.x + c2 * t2.x, x0.y + c1 * t1.y + c2 * t2.y);
    const cpx<T> a2 = mk<T>(x0.x + c2 * t1.x + c1 * t2.x, x0.y + c2 * t1.y + c1 * t2.y);
    const cpx<T> b1 = mk<T>(s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y);
    const cpx<T> b2 = mk<T>(s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y);
    const cpx<T> e1 = BACKWARD ? mk<T>(-b1.y, b1.x) : mk<T>(b1.y, -b1.x);
    const cpx<T> e2 = BACKWARD ? mk<T>(-b2.y, b2.x) : mk<T>(b2.y, -b2.x);
    x[0] = cadd(x0, cadd(t1, t2));
    x[1] = cadd(a1, e1);
    x[2] = cadd(a2, e2);
    x[3] = csub(a2, e2);
    x[4] = csub(a1, e1);
  } else {
    constexpr int R = FirstRadix<N>::value, M = N / R;
    static_assert(R > 1 && R < N, "dft: N must factor into 2, 3, 4 and 5");
    cpx<T> y[R][M];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int m = 0; m < M; ++m) y[r][m] = x[r + R * m];
#pragma unroll
    for (int r = 0; r < R; ++r) dft<M, BACKWARD, T>(y[r]);
    static_for<0, M>([&](auto k1c) {
      constexpr int k1 = decltype(k1c)::value;
      cpx<T> z[R];
      static_for<0, R>([&](auto rc) {
        constexpr int r = decltype(rc)::value;
        z[r] = twc<r * k1, N, BACKWARD, T>(y[r][k1]);
      });
      dft<R, BACKWARD, T>(z);
#pragma unroll
      for (int k2 = 0; k2 < R; ++k2) x[k1 + M * k2] = z[k2];
    });
  }
}


}  // namespace owt

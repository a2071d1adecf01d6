// Host check of the register transforms (csrc/fft_reg.cuh): dft<N> in double
// and float against a direct O(N^2) transform in long double, both signs,
// and the two-pass line transform of length A B against the same, for the
// factorisations the transform kernels use.  Built with nvcc as host code and
// run by tests/test_fft_reg_host.py; prints the worst errors, exits non-zero
// past the bounds (double: 4e-15, float: 1.5e-6, relative to the largest
// output).
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "fft_reg.cuh"

using namespace owt;

template <typename T>
static double direct_err(const std::vector<cpx<T>> &in, const std::vector<cpx<T>> &out, bool backward) {
  const int n = (int)in.size();
  long double worst = 0, scale = 0;
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int k = 0; k < n; ++k) {
    long double re = 0, im = 0;
    for (int j = 0; j < n; ++j) {
      const long double a = (backward ? 2 : -2) * pi * (long double)((long long)j * k % n) / n;
      re += (long double)in[j].x * cosl(a) - (long double)in[j].y * sinl(a);
      im += (long double)in[j].x * sinl(a) + (long double)in[j].y * cosl(a);
    }
    worst = fmaxl(worst, fabsl(re - out[k].x));
    worst = fmaxl(worst, fabsl(im - out[k].y));
    scale = fmaxl(scale, fmaxl(fabsl(re), fabsl(im)));
  }
  return (double)(worst / scale);
}

template <int N, typename T, bool B>
static double check_dft(std::mt19937 &g) {
  std::normal_distribution<double> d;
  std::vector<cpx<T>> in(N), out(N);
  cpx<T> x[N];
  for (int j = 0; j < N; ++j) x[j] = in[j] = mk<T>((T)d(g), (T)d(g));
  dft<N, B, T>(x);
  for (int j = 0; j < N; ++j) out[j] = x[j];
  return direct_err<T>(in, out, B);
}

// Line of length L = A B: pass 1 (thread b) transforms x[b + B a] over a,
// multiplies output a' by w_L^(b a'), pass 2 (thread a') transforms over b
// and gives X[a' + A b'].
template <int A, int Bn, typename T, bool BACK>
static double check_line(std::mt19937 &g) {
  constexpr int L = A * Bn;
  std::normal_distribution<double> d;
  std::vector<cpx<T>> in(L), mid(L), out(L);
  for (auto &v : in) v = mk<T>((T)d(g), (T)d(g));
  for (int b = 0; b < Bn; ++b) {
    cpx<T> x[A];
    for (int a = 0; a < A; ++a) x[a] = in[b + Bn * a];
    dft<A, BACK, T>(x);
    for (int a = 0; a < A; ++a) {
      const ct::CS w = ct::cs2pi((long)b * a, L);
      const T c = (T)w.c, s = (T)(BACK ? w.s : -w.s);
      mid[a * Bn + b] = mk<T>(x[a].x * c - x[a].y * s, x[a].x * s + x[a].y * c);
    }
  }
  for (int a = 0; a < A; ++a) {
    cpx<T> y[Bn];
    for (int b = 0; b < Bn; ++b) y[b] = mid[a * Bn + b];
    dft<Bn, BACK, T>(y);
    for (int b = 0; b < Bn; ++b) out[a + A * b] = y[b];
  }
  return direct_err<T>(in, out, BACK);
}

template <int N>
static void both(std::mt19937 &g, double &wd, double &wf) {
  wd = std::fmax(wd, std::fmax(check_dft<N, double, false>(g), check_dft<N, double, true>(g)));
  wf = std::fmax(wf, std::fmax(check_dft<N, float, false>(g), check_dft<N, float, true>(g)));
}
template <int A, int B>
static void line(std::mt19937 &g, double &wd, double &wf) {
  wd = std::fmax(wd, std::fmax(check_line<A, B, double, false>(g), check_line<A, B, double, true>(g)));
  wf = std::fmax(wf, std::fmax(check_line<A, B, float, false>(g), check_line<A, B, float, true>(g)));
}

int main() {
  std::mt19937 g(12345);
  double wd = 0, wf = 0;
  both<2>(g, wd, wf); both<3>(g, wd, wf); both<4>(g, wd, wf); both<5>(g, wd, wf); both<6>(g, wd, wf);
  both<8>(g, wd, wf); both<9>(g, wd, wf); both<10>(g, wd, wf); both<12>(g, wd, wf); both<15>(g, wd, wf);
  both<16>(g, wd, wf); both<18>(g, wd, wf); both<20>(g, wd, wf); both<24>(g, wd, wf); both<30>(g, wd, wf);
  both<32>(g, wd, wf); both<36>(g, wd, wf);
  std::printf("register transforms: worst relative error double %.2e, float %.2e\n", wd, wf);
  double ld = 0, lf = 0;
  line<24, 24>(g, ld, lf); line<16, 12>(g, ld, lf); line<12, 8>(g, ld, lf); line<9, 8>(g, ld, lf);
  line<8, 6>(g, ld, lf); line<20, 24>(g, ld, lf);
  std::printf("two-pass lines: worst relative error double %.2e, float %.2e\n", ld, lf);
  // the constants themselves against long double
  double wc = 0;
  for (long n : {5L, 8L, 9L, 12L, 24L, 192L, 576L, 960L})
    for (long k = 0; k < n; ++k) {
      const ct::CS w = ct::cs2pi(k, n);
      const long double a = 2 * 3.141592653589793238462643383279502884L * k / n;
      wc = std::fmax(wc, (double)fmaxl(fabsl(w.c - cosl(a)), fabsl(w.s - sinl(a))));
    }
  std::printf("twiddle constants: worst absolute error %.2e\n", wc);
  const bool ok = wd < 4e-15 && wf < 1.5e-6 && ld < 4e-15 && lf < 1.5e-6 && wc < 3e-16;
  std::printf("%s\n", ok ? "ok" : "FAIL");
  return ok ? 0 : 1;
}

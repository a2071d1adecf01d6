// Test infrastructure (oracle): project-written CPU FFT used by the oracle only.
//
// Complex DFT of any length n = product of small factors, computed by a
// self-sorting (Stockham) mixed-radix schedule with radices 4, 2, 3, 5 and a
// generic O(R^2) butterfly for any other prime factor.  Sign convention follows
// FFTW's (reference src/FFT.cpp:24-27): sign -1 is the forward transform
// X[k] = sum_j x[j] exp(-2 pi i jk/n), sign +1 the backward one; both are
// unnormalised.  Twiddles are evaluated in long double and rounded once.
#pragma once
#include <cmath>
#include <complex>
#include <stdexcept>
#include <vector>

namespace owt_oracle {

using cplx = std::complex<double>;

class CpuFft {
 public:
  CpuFft() = default;
  CpuFft(int n, int sign) : n_(n), sign_(sign) {
    if (n < 1) throw std::invalid_argument("CpuFft: length must be positive");
    int m = n;
    while (m % 4 == 0) { radices_.push_back(4); m /= 4; }
    while (m % 2 == 0) { radices_.push_back(2); m /= 2; }
    while (m % 3 == 0) { radices_.push_back(3); m /= 3; }
    while (m % 5 == 0) { radices_.push_back(5); m /= 5; }
    for (int p = 7; m > 1; p += 2)
      while (m % p == 0) { radices_.push_back(p); m /= p; }
    tw_.resize(n);
    const long double two_pi = 6.283185307179586476925286766559005768L;
    for (int k = 0; k < n; ++k) {
      long double a = two_pi * (long double)k / (long double)n;
      tw_[k] = cplx((double)std::cos(a), (double)(sign * std::sin(a)));
    }
  }
  int size() const { return n_; }
  // in and out may alias; work must hold n values.
  void exec(const cplx* in, cplx* out, cplx* work) const {
    std::vector<cplx> a(in, in + n_);
    cplx* src = a.data();
    cplx* dst = work;
    int ns = 1;
    for (int R : radices_) {
      const int nr = n_ / R;
      const int step = n_ / (ns * R);
      cplx v[64];
      std::vector<cplx> big;
      cplx* vv = v;
      if (R > 64) { big.resize(R); vv = big.data(); }
      for (int j = 0; j < nr; ++j) {
        const int k = j % ns;
        for (int r = 0; r < R; ++r) {
          cplx x = src[j + r * nr];
          vv[r] = (r == 0 || k == 0) ? x : x * tw_[(long)k * r * step % n_];
        }
        butterfly(vv, R);
        const int base = (j / ns) * ns * R + k;
        for (int r = 0; r < R; ++r) dst[base + r * ns] = vv[r];
      }
      ns *= R;
      std::swap(src, dst);
    }
    for (int i = 0; i < n_; ++i) out[i] = src[i];
  }

 private:
  void butterfly(cplx* v, int R) const {
    const double s = (double)sign_;
    if (R == 2) {
      cplx a = v[0], b = v[1];
      v[0] = a + b; v[1] = a - b;
    } else if (R == 4) {
      cplx a = v[0], b = v[1], c = v[2], d = v[3];
      cplx t0 = a + c, t1 = a - c, t2 = b + d, t3 = (b - d) * cplx(0.0, s);
      v[0] = t0 + t2; v[1] = t1 + t3; v[2] = t0 - t2; v[3] = t1 - t3;
    } else if (R == 3) {
      const double c1 = -0.5, s1 = s * 0.86602540378443864676372317075294;
      cplx a = v[0], b = v[1], c = v[2];
      cplx t = b + c, u = (b - c) * cplx(0.0, s1);
      cplx m = a + c1 * t;
      v[0] = a + t; v[1] = m + u; v[2] = m - u;
    } else {
      std::vector<cplx> x(v, v + R);
      const int stride = n_ / R;
      for (int q = 0; q < R; ++q) {
        cplx acc = 0.0;
        for (int r = 0; r < R; ++r) acc += x[r] * tw_[(long)q * r % R * stride];
        v[q] = acc;
      }
    }
  }
  int n_ = 0;
  int sign_ = -1;
  std::vector<int> radices_;
  std::vector<cplx> tw_;
};

}  // namespace owt_oracle

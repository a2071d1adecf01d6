// Host check of the banded augmented systems (csrc/setup_host.cpp) against
// the reference's dense per-mode systems (src/solver.cpp:577-603, as the
// oracle restates them): for a sweep of grids, both finite-difference orders
// and a sweep of wavenumbers, the v-system (unknowns v and h^t d_t, d4
// substituted on interior nodes, right-hand sides through the row tables)
// and the omega_y-system (unknowns h d1, h^2 d2 of g, g recovered from them)
// are assembled from their templates, rows equilibrated, factored by partial-
// pivoting band LU in LAPACK dgbtf2 order and solved with the library's own
// band solve (host-callable, csrc/owt_device.cuh); the dense systems
//   Av = -nu DY4 + a DY2 - b I,  Ag = -nu DY2 + cg I,
// DYn = sum_m diag(c_nm) A_m^-1 B_m from the same stencils, boundary rows
// v = DY1 v = 0 and g = 0 on both walls, are solved by dense partial-pivoting
// LU.  The v-system is ill-conditioned (DY4 on the stretched grid: the two
// solutions differ by up to ~1e-7 of max |v| at these sizes, which is its
// conditioning, not an error of either), so its criterion is the normwise
// backward error of the banded solution in the reference's dense system,
// evaluated in long double: at most 2e-14 (the dense LU's own is ~1e-16).
// The omega_y-system is well conditioned: its g agrees with the dense
// solution to 1e-12 of max |g|.  Built with nvcc as host code and run by
// tests/test_augmented_host.py; exits non-zero past either bound.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "owt_device.cuh"
#include "setup_host.h"

using namespace owt;

using Mat = std::vector<double>;  // dense N x N, row-major

static void dense_solve(Mat A, std::vector<double> &b, int N) {
  for (int k = 0; k < N; ++k) {
    int p = k;
    for (int i = k + 1; i < N; ++i)
      if (std::fabs(A[(size_t)i * N + k]) > std::fabs(A[(size_t)p * N + k])) p = i;
    if (p != k) {
      for (int c = 0; c < N; ++c) std::swap(A[(size_t)k * N + c], A[(size_t)p * N + c]);
      std::swap(b[k], b[p]);
    }
    const double piv = A[(size_t)k * N + k];
    for (int i = k + 1; i < N; ++i) {
      const double l = A[(size_t)i * N + k] / piv;
      if (l == 0.0) continue;
      for (int c = k; c < N; ++c) A[(size_t)i * N + c] -= l * A[(size_t)k * N + c];
      b[i] -= l * b[k];
    }
  }
  for (int k = N - 1; k >= 0; --k) {
    double s = b[k];
    for (int c = k + 1; c < N; ++c) s -= A[(size_t)k * N + c] * b[c];
    b[k] = s / A[(size_t)k * N + k];
  }
}

// D = A^-1 B for the stencil pair of derivative m (0-based)
static Mat derivative(const Stencils &st, int m) {
  const int N = st.N;
  Mat D((size_t)N * N);
  for (int c = 0; c < N; ++c) {
    std::vector<double> col(N);
    for (int r = 0; r < N; ++r) col[r] = st.b(m, r, c);
    dense_solve(st.A[m], col, N);
    for (int r = 0; r < N; ++r) D[(size_t)r * N + c] = col[r];
  }
  return D;
}

struct Factors {
  int n = 0, kl = 0, ku = 0;
  std::vector<double> ab, rs;  // factors (diagonal as its reciprocal), row scales 1 / max |row|
  std::vector<uint8_t> piv;
};

static Factors factor(const BandTemplate &t, double s1, double s2) {
  Factors f;
  f.n = t.n; f.kl = t.kl; f.ku = t.ku;
  const int n = t.n, KL = t.kl, KU = t.ku, KV = KL + KU, NB = 2 * KL + KU + 1;
  f.ab.assign((size_t)NB * n, 0.0);
  f.rs.assign(n, 1.0);
  f.piv.assign(n, 0);
  auto AB = [&](int b, int c) -> double & { return f.ab[(size_t)b * n + c]; };
  for (int c = 0; c < n; ++c)
    for (int b = KL; b < NB; ++b) {
      const size_t at = (size_t)(b - KL) * n + c;
      AB(b, c) = t.t0[at] + s1 * t.t1[at] + s2 * t.t2[at];
    }
  for (int p = 0; p < n; ++p) {
    const int c0 = std::max(0, p - KL), c1 = std::min(n - 1, p + KU);
    double mx = 0;
    for (int c = c0; c <= c1; ++c) mx = std::fmax(mx, std::fabs(AB(KV + p - c, c)));
    for (int c = c0; c <= c1; ++c) AB(KV + p - c, c) /= mx;
    f.rs[p] = 1.0 / mx;
  }
  int ju = 0;
  for (int j = 0; j < n; ++j) {
    const int km = std::min(KL, n - 1 - j);
    int jp = 0;
    double best = std::fabs(AB(KV, j));
    for (int i = 1; i <= km; ++i)
      if (std::fabs(AB(KV + i, j)) > best) { best = std::fabs(AB(KV + i, j)); jp = i; }
    f.piv[j] = (uint8_t)jp;
    ju = std::max(ju, std::min(j + KU + jp, n - 1));
    if (jp)
      for (int c = j; c <= ju; ++c) std::swap(AB(KV + jp - (c - j), c), AB(KV - (c - j), c));
    const double rp = 1.0 / AB(KV, j);
    for (int i = 1; i <= km; ++i) AB(KV + i, j) *= rp;
    for (int c = j + 1; c <= ju; ++c) {
      const double tt = AB(KV - (c - j), c);
      if (tt != 0.0)
        for (int i = 1; i <= km; ++i) AB(KV + i - (c - j), c) -= AB(KV + i, j) * tt;
    }
  }
  for (int j = 0; j < n; ++j) AB(KV, j) = 1.0 / AB(KV, j);
  return f;
}

template <int KL, int KU>
static std::vector<double> band(const Factors &f, const std::vector<double> &b) {
  std::vector<double> y(f.n), x(f.n);
  band_solve<KL, KU>(f.ab.data(), f.piv.data(), f.n, 1, 0, [&](int p) { return b[p]; },
                     [&](int p, double v) { y[p] = v; }, [&](int p) { return y[p]; },
                     [&](int c, double v) { x[c] = v; });
  return x;
}

// normwise backward error |A x - b| / (|A| |x| + |b|) (infinity norms), in long double
static double backward_error(const Mat &A, const std::vector<double> &x, const std::vector<double> &b, int N) {
  long double res = 0, an = 0, xn = 0, bn = 0;
  for (int i = 0; i < N; ++i) {
    long double s = 0, rowsum = 0;
    for (int c = 0; c < N; ++c) {
      s += (long double)A[(size_t)i * N + c] * x[c];
      rowsum += fabsl((long double)A[(size_t)i * N + c]);
    }
    res = fmaxl(res, fabsl(s - b[i]));
    an = fmaxl(an, rowsum);
    xn = fmaxl(xn, fabsl((long double)x[i]));
    bn = fmaxl(bn, fabsl((long double)b[i]));
  }
  return (double)(res / (an * xn + bn));
}

static double rel(const std::vector<double> &a, const std::vector<double> &b) {
  double d = 0, s = 0;
  for (size_t i = 0; i < a.size(); ++i) {
    d = std::fmax(d, std::fabs(a[i] - b[i]));
    s = std::fmax(s, std::fabs(b[i]));
  }
  return d / s;
}

int main() {
  struct Cfg { int N; double alpha, dt, nu; };
  const Cfg cfgs[] = {{33, 2.0, 0.005, 1.0 / 2800}, {65, 2.5, 0.001, 1e-4}, {97, 2.0, 0.004, 1.0 / 3000},
                      {129, 2.0, 0.005, 1.0 / 2800}, {257, 2.2, 0.002, 1e-4}};
  const double kBackward = 2e-14, kForwardG = 1e-12;
  std::mt19937_64 rng(11);
  std::normal_distribution<double> gauss;
  bool ok = true;
  for (const Cfg &cf : cfgs) {
    const int N = cf.N;
    const Grid g = make_grid(N, cf.alpha);
    for (int order : {8, 6}) {
      const Stencils st = make_stencils(N, g.ds, order);
      Mat D[4];
      for (int m = 0; m < 4; ++m) D[m] = derivative(st, m);
      Mat DY1((size_t)N * N), DY2((size_t)N * N), DY4((size_t)N * N);
      for (int r = 0; r < N; ++r)
        for (int c = 0; c < N; ++c) {
          const size_t at = (size_t)r * N + c;
          DY1[at] = g.c11[r] * D[0][at];
          DY2[at] = g.c21[r] * D[0][at] + g.c22[r] * D[1][at];
          DY4[at] = g.c41[r] * D[0][at] + g.c42[r] * D[1][at] + g.c43[r] * D[2][at] + g.c44[r] * D[3][at];
        }
      BandTemplate tv = build_v_system(g, st, cf.nu), tg = build_g_system(g, st, cf.nu);
      pad_band(tv, kVKL, kVKU);
      pad_band(tg, 6, 6);
      double worst_v = 0, worst_g = 0, berr_band = 0, berr_dense = 0;
      const double g0 = 11.0 / 6.0;
      for (int q = 0; q < 8; ++q) {
        const double k = 0.5 * std::pow(600.0, q / 7.0), k2 = k * k;
        const double ca = g0 / cf.dt + 2 * cf.nu * k2, cb = cf.nu * k2 * k2 + g0 * k2 / cf.dt;
        const double cg = cf.nu * k2 + g0 / cf.dt;
        std::vector<double> r(N);
        for (double &x : r) x = gauss(rng);
        // dense reference
        Mat Av((size_t)N * N), Ag((size_t)N * N);
        for (int i = 0; i < N; ++i)
          for (int c = 0; c < N; ++c) {
            const size_t at = (size_t)i * N + c;
            Av[at] = -cf.nu * DY4[at] + ca * DY2[at] - (i == c ? cb : 0.0);
            Ag[at] = -cf.nu * DY2[at] + (i == c ? cg : 0.0);
          }
        for (int c = 0; c < N; ++c) {
          Av[c] = 0.0; Av[(size_t)1 * N + c] = DY1[c]; Av[(size_t)(N - 2) * N + c] = DY1[(size_t)(N - 1) * N + c];
          Av[(size_t)(N - 1) * N + c] = 0.0;
          Ag[c] = 0.0; Ag[(size_t)(N - 1) * N + c] = 0.0;
        }
        Av[0] = 1.0; Av[(size_t)(N - 1) * N + N - 1] = 1.0; Ag[0] = 1.0; Ag[(size_t)(N - 1) * N + N - 1] = 1.0;
        std::vector<double> sv = r, sg = r;
        sv[0] = sv[1] = sv[N - 2] = sv[N - 1] = 0.0;
        sg[0] = sg[N - 1] = 0.0;
        const std::vector<double> rhs_v = sv;
        dense_solve(Av, sv, N);
        dense_solve(Ag, sg, N);
        // v-system: rows' right-hand sides from the tables, v = unknown (0, j)
        const Factors fv = factor(tv, ca, cb);
        std::vector<double> bv(fv.n, 0.0);
        for (int p = 0; p < fv.n; ++p)
          if (tv.rhs_node[p] == kRhsTable) {
            double s = 0;
            for (int e = 0; e < 4; ++e) s += tv.rbv_val[(size_t)p * 4 + e] * r[tv.rbv_col[(size_t)p * 4 + e]];
            bv[p] = fv.rs[p] * s;
          }
        const std::vector<double> xv = band<kVKL, kVKU>(fv, bv);
        std::vector<double> v(N);
        for (int j = 0; j < N; ++j) v[j] = xv[vcol(0, j, N)];
        worst_v = std::fmax(worst_v, rel(v, sv));
        berr_band = std::fmax(berr_band, backward_error(Av, v, rhs_v, N));
        berr_dense = std::fmax(berr_dense, backward_error(Av, sv, rhs_v, N));
        // omega_y-system: rows (1/cg) B r, g from the solved h d1, h^2 d2
        const Factors fg = factor(tg, 1.0 / cg, 0.0);
        std::vector<double> bg(fg.n, 0.0);
        for (int p = 0; p < fg.n; ++p) {
          double s = 0;
          for (int e = 0; e < 5; ++e) s += tg.rb_val[(size_t)p * 5 + e] * r[tg.rb_col[(size_t)p * 5 + e]];
          bg[p] = fg.rs[p] * s / cg;
        }
        const std::vector<double> xg = band<6, 6>(fg, bg);
        std::vector<double> gg(N, 0.0);
        for (int j = 1; j < N - 1; ++j) {
          const double d1 = xg[2 * j] / g.ds, d2 = xg[2 * j + 1] / (g.ds * g.ds);
          gg[j] = (r[j] + cf.nu * g.c21[j] * d1 + cf.nu * g.c22[j] * d2) / cg;
        }
        worst_g = std::fmax(worst_g, rel(gg, sg));
      }
      const bool pass = berr_band <= kBackward && worst_g <= kForwardG;
      ok = ok && pass;
      std::printf("N=%d order %d: v backward error %.2e (dense LU %.2e), v difference %.2e; g difference %.2e%s\n",
                  N, order, berr_band, berr_dense, worst_v, worst_g, pass ? "" : "  FAILED");
    }
  }
  std::printf(ok ? "augmented systems agree with the dense ones\n" : "FAILED\n");
  return ok ? 0 : 1;
}

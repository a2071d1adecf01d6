// Host check of the masked band solves (csrc/owt_device.cuh): the v-system's
// masked solve (one ring and the mode kernel's two-ring backward sweep), the
// omega_y-system's masked solve and the masked transposed v solve of the
// adjoint, each against its full-band form on the same factors and the same
// right-hand sides, bitwise.  The factors are built here the way the setup
// builds them (band templates of setup_host.cpp assembled per wavenumber,
// rows equilibrated, partial-pivoting band LU in LAPACK dgbtf2 order, the
// diagonal stored as its reciprocal); a factorization whose interior fill or
// interchanges leave the masks is one the setup check would refuse, and is
// counted and skipped.  Built with nvcc as host code and run by
// tests/test_band_masks_host.py; exits non-zero on any difference.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "owt_device.cuh"
#include "setup_host.h"

using namespace owt;

struct Factors {
  int n = 0, kl = 0, ku = 0;
  std::vector<double> ab;    // (2 kl + ku + 1) rows of n, LAPACK factorization layout
  std::vector<uint8_t> piv;  // row interchange offset per column
};

static Factors factor(const BandTemplate &t, double s1, double s2) {
  Factors f;
  f.n = t.n; f.kl = t.kl; f.ku = t.ku;
  const int n = t.n, KL = t.kl, KU = t.ku, KV = KL + KU, NB = 2 * KL + KU + 1;
  f.ab.assign((size_t)NB * n, 0.0);
  f.piv.assign(n, 0);
  auto AB = [&](int b, int c) -> double & { return f.ab[(size_t)b * n + c]; };
  for (int c = 0; c < n; ++c)
    for (int b = KL; b < NB; ++b) {
      const size_t at = (size_t)(b - KL) * n + c;
      AB(b, c) = t.t0[at] + s1 * t.t1[at] + s2 * t.t2[at];
    }
  for (int p = 0; p < n; ++p) {  // each row divided by its largest coefficient
    const int c0 = std::max(0, p - KL), c1 = std::min(n - 1, p + KU);
    double mx = 0;
    for (int c = c0; c <= c1; ++c) mx = std::fmax(mx, std::fabs(AB(KV + p - c, c)));
    for (int c = c0; c <= c1; ++c) AB(KV + p - c, c) /= mx;
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

// interior columns [lo, n - hi) inside their type's fill and interchange masks
template <class Masks>
static bool admitted(const Factors &f, int NT, int OFF) {
  const int n = f.n, KL = f.kl, KV = f.kl + f.ku;
  for (int c = Masks::lo; c < n - Masks::hi; ++c) {
    const int ty = (c + OFF) % NT;
    for (int t = 1; t <= KL; ++t)
      if (f.ab[(size_t)(KV + t) * n + c] != 0.0 && !((Masks::l(ty) >> t) & 1ull)) return false;
    for (int t = 1; t <= KV && t <= c; ++t)
      if (f.ab[(size_t)(KV - t) * n + c] != 0.0 && !((Masks::u(ty) >> t) & 1ull)) return false;
    if (f.piv[c] && !((Masks::p(ty) >> f.piv[c]) & 1ull)) return false;
  }
  return true;
}

// x = solve(b) through the callback interface of the band solves
template <class Solve>
static std::vector<double> run(int n, const std::vector<double> &b, Solve solve) {
  std::vector<double> y(n, 0.0), x(n, 0.0);
  auto rhs = [&](int p) { return b[p]; };
  auto ys = [&](int p, double v) { y[p] = v; };
  auto yl = [&](int p) { return y[p]; };
  auto out = [&](int c, double v) { x[c] = v; };
  solve(rhs, ys, yl, out);
  return x;
}

static bool same(const std::vector<double> &a, const std::vector<double> &b) {
  return a.size() == b.size() && std::memcmp(a.data(), b.data(), a.size() * sizeof(double)) == 0;
}

struct Tally { int checked = 0, skipped = 0, bad = 0; };

template <class VM>
static void check_v(const Factors &f, std::mt19937_64 &rng, Tally &tl, const char *what) {
  if (!admitted<VM>(f, 4, 2)) { ++tl.skipped; return; }
  const int n = f.n;
  const double *ab = f.ab.data();
  const uint8_t *pv = f.piv.data();
  std::normal_distribution<double> g;
  for (int rep = 0; rep < 2; ++rep) {
    std::vector<double> b(n);
    for (double &v : b) v = g(rng);
    const auto full = run(n, b, [&](auto r, auto s, auto l, auto o) { band_solve<kVKL, kVKU>(ab, pv, n, 1, 0, r, s, l, o); });
    const auto one = run(n, b, [&](auto r, auto s, auto l, auto o) {
      band_solve_masked<kVKL, kVKU, 4, 2, 16, 32, VM>(ab, pv, n, 1, 0, r, s, l, o);
    });
    const auto two = run(n, b, [&](auto r, auto s, auto l, auto o) {
      band_forward_v_sparse<VM>(ab, pv, n, 1, 0, r, s);
      band_backward_v_sparse<VM>(ab, n, 1, 0, l, s, o);
    });
    const auto tfull = run(n, b, [&](auto r, auto s, auto l, auto o) { band_solve_t<kVKL, kVKU>(ab, pv, n, 1, 0, r, s, l, o); });
    const auto tmask = run(n, b, [&](auto r, auto s, auto l, auto o) {
      band_solve_t_masked<kVKL, kVKU, 4, 2, VM>(ab, pv, n, 1, 0, r, s, l, o);
    });
    ++tl.checked;
    if (!same(full, one) || !same(full, two) || !same(tfull, tmask)) {
      ++tl.bad;
      std::printf("MISMATCH %s n=%d: one-ring %d two-ring %d transposed %d\n", what, n, (int)same(full, one),
                  (int)same(full, two), (int)same(tfull, tmask));
    }
  }
}

static void check_g(const Factors &f, std::mt19937_64 &rng, Tally &tl) {
  if (!admitted<GMasks>(f, 2, 0)) { ++tl.skipped; return; }
  const int n = f.n;
  const double *ab = f.ab.data();
  const uint8_t *pv = f.piv.data();
  std::normal_distribution<double> g;
  std::vector<double> b(n);
  for (double &v : b) v = g(rng);
  const auto full = run(n, b, [&](auto r, auto s, auto l, auto o) { band_solve<6, 6>(ab, pv, n, 1, 0, r, s, l, o); });
  const auto mask = run(n, b, [&](auto r, auto s, auto l, auto o) { band_solve_g_sparse(ab, pv, n, 1, 0, r, s, l, o); });
  ++tl.checked;
  if (!same(full, mask)) {
    ++tl.bad;
    std::printf("MISMATCH omega_y n=%d\n", n);
  }
}

int main() {
  struct Cfg { int N; double alpha, dt, nu; };
  const Cfg cfgs[] = {{65, 2.5, 0.001, 1e-4}, {97, 2.0, 0.004, 1.0 / 3000}, {129, 2.0, 0.005, 1.0 / 2800},
                      {193, 2.0, 0.003, 1.0 / 5000}, {257, 2.2, 0.002, 1e-4}};
  std::mt19937_64 rng(7);
  Tally v8, v6, gg;
  for (const Cfg &cf : cfgs) {
    const Grid grid = make_grid(cf.N, cf.alpha);
    for (int order : {8, 6}) {
      const Stencils st = make_stencils(cf.N, grid.ds, order);
      BandTemplate tv = build_v_system(grid, st, cf.nu), tg = build_g_system(grid, st, cf.nu);
      pad_band(tv, kVKL, kVKU);
      pad_band(tg, 6, 6);
      const double g0 = 11.0 / 6.0;
      for (int q = 1; q <= 12; ++q) {
        const double k = 0.3 * std::pow(1200.0 / 0.3, (q - 1) / 11.0), k2 = k * k;
        const Factors fv = factor(tv, g0 / cf.dt + 2 * cf.nu * k2, cf.nu * k2 * k2 + g0 * k2 / cf.dt);
        if (order == 8) check_v<VMasks>(fv, rng, v8, "v (8th order)");
        else check_v<VMasks6>(fv, rng, v6, "v (6th order)");
        if (order == 8) check_g(factor(tg, 1.0 / (cf.nu * k2 + g0 / cf.dt), 0.0), rng, gg);
      }
    }
  }
  std::printf("v-system 8th order: %d right-hand sides checked, %d factorizations outside the masks\n", v8.checked,
              v8.skipped);
  std::printf("v-system 6th order: %d checked, %d outside\n", v6.checked, v6.skipped);
  std::printf("omega_y-system: %d checked, %d outside\n", gg.checked, gg.skipped);
  const int bad = v8.bad + v6.bad + gg.bad;
  if (bad || v8.checked == 0 || v6.checked == 0 || gg.checked == 0) {
    std::printf("FAILED: %d mismatches\n", bad);
    return 1;
  }
  std::printf("all bitwise equal\n");
  return 0;
}

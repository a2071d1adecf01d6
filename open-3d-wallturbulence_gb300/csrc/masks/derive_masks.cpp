// Derives the interior fill and pivot masks of the masked band solves
// (vmask_*, gmask_* in owt_device.cuh): builds the band templates exactly as
// the library does (setup_host.cpp), assembles them for a sweep of
// wavenumbers, grids, time steps, viscosities and stretchings, equilibrates
// the rows and factorises in the order of k_band_factor (LAPACK dgbtf2), and
// prints the union of the nonzero offsets of L and U and of the row
// interchanges per column type over the interior columns.  Not part of the
// library; every factorization is still checked against the masks at setup.
//
//   g++ -std=c++17 -O2 derive_masks.cpp ../setup_host.cpp -o derive_masks && ./derive_masks
#include "../setup_host.h"
#include <cmath>
#include <cstdlib>
#include <iterator>
#include <cstdio>
#include <vector>
using namespace owt;
struct Stat { unsigned long long L[8] = {0}, U[8] = {0}, P[8] = {0}; };
static void factor_and_scan(const BandTemplate &t, double s1, double s2, int NT, int OFF, int LO, int HI, Stat &st) {
  const int n = t.n, KL = t.kl, KU = t.ku, KV = KL + KU, NB = 2 * KL + KU + 1;
  std::vector<double> ab((size_t)NB * n, 0.0);
  auto AB = [&](int b, int c) -> double & { return ab[(size_t)b * n + c]; };
  for (int c = 0; c < n; ++c)
    for (int b = KL; b < NB; ++b) { const size_t at = (size_t)(b - KL) * n + c; AB(b, c) = t.t0[at] + s1 * t.t1[at] + s2 * t.t2[at]; }
  for (int p = 0; p < n; ++p) {
    const int c0 = std::max(0, p - KL), c1 = std::min(n - 1, p + KU);
    double mx = 0; for (int c = c0; c <= c1; ++c) mx = std::fmax(mx, std::fabs(AB(KV + p - c, c)));
    for (int c = c0; c <= c1; ++c) AB(KV + p - c, c) /= mx;
  }
  std::vector<int> piv(n);
  int ju = 0;
  for (int j = 0; j < n; ++j) {
    const int km = std::min(KL, n - 1 - j);
    int jp = 0; double best = std::fabs(AB(KV, j));
    for (int i = 1; i <= km; ++i) { const double v = std::fabs(AB(KV + i, j)); if (v > best) { best = v; jp = i; } }
    piv[j] = jp;
    ju = std::max(ju, std::min(j + KU + jp, n - 1));
    if (jp) for (int c = j; c <= ju; ++c) std::swap(AB(KV + jp - (c - j), c), AB(KV - (c - j), c));
    const double rp = 1.0 / AB(KV, j);
    for (int i = 1; i <= km; ++i) AB(KV + i, j) *= rp;
    for (int c = j + 1; c <= ju; ++c) { const double tt = AB(KV - (c - j), c); if (tt != 0.0) for (int i = 1; i <= km; ++i) AB(KV + i - (c - j), c) -= AB(KV + i, j) * tt; }
  }
  for (int c = LO; c < n - HI; ++c) {
    const int ty = (c + OFF) % NT;
    for (int tt = 1; tt <= KL; ++tt) if (AB(KV + tt, c) != 0.0) st.L[ty] |= 1ull << tt;
    for (int tt = 1; tt <= KV; ++tt) if (AB(KV - tt, c) != 0.0) st.U[ty] |= 1ull << tt;
    if (piv[c]) st.P[ty] |= 1ull << piv[c];
  }
}
int main() {
  struct Cfg { int N; double alpha, dt, nu, dkx, dkz; };
  const Cfg base[] = {{257, 2.2, 0.002, 1e-4, 1.0, 2.0}, {129, 2.0, 0.005, 1.0 / 2800, 0.5, 1.5}, {97, 1.5, 0.01, 1.0 / 2000, 1, 2},
                      {193, 2.0, 0.003, 1.0 / 5000, 1, 2}, {65, 2.5, 0.001, 1e-4, 1, 2}, {129, 2.2, 0.004, 1.0 / 4000, 1, 2}, {97, 2.0, 0.004, 1.0 / 3000, 1, 3}};
  const Cfg batch[] = {{97, 2.0, 0.004, 1.0 / 4400, 1, 2}, {97, 2.0, 0.004, 1.0 / 8200, 1, 2}, {97, 2.0, 0.004, 1.0 / 6000, 1, 2}};
  // ONLY_BATCH=1: the minimal-channel ensemble's parameter range alone
  const bool only_batch = getenv("ONLY_BATCH") != nullptr;
  std::vector<Cfg> cfgs;
  if (only_batch) cfgs.assign(std::begin(batch), std::end(batch)); else cfgs.assign(std::begin(base), std::end(base));
  for (int order : {8, 6}) {
    Stat sv, sg;
    for (const Cfg &cf : cfgs) {
      Grid g = make_grid(cf.N, cf.alpha); Stencils st = make_stencils(cf.N, g.ds, order);
      BandTemplate tv = build_v_system(g, st, cf.nu), tg = build_g_system(g, st, cf.nu);
      pad_band(tv, kVKL, kVKU); pad_band(tg, 6, 6);
      const double g0 = 11.0 / 6.0;
      for (int q = 0; q <= 40; ++q) {
        const double k = q == 0 ? 0.0 : 0.2 * std::pow(1500.0 / 0.2, (q - 1) / 39.0);
        const double k2 = k * k;
        // the full-band widths at both ends (VMasks, VMasks6, GMasks)
        factor_and_scan(tv, g0 / cf.dt + 2 * cf.nu * k2, cf.nu * k2 * k2 + g0 * k2 / cf.dt, 4, 2, 44, 32, sv);
        factor_and_scan(tg, 1.0 / (cf.nu * k2 + g0 / cf.dt), 0.0, 2, 0, 16, 16, sg);
      }
    }
    std::printf("order %d\n v L:", order); for (int i = 0; i < 4; ++i) std::printf(" 0x%llx", sv.L[i]);
    std::printf("\n v U:"); for (int i = 0; i < 4; ++i) std::printf(" 0x%llx", sv.U[i]);
    std::printf("\n v P:"); for (int i = 0; i < 4; ++i) std::printf(" 0x%llx", sv.P[i]);
    std::printf("\n g L: 0x%llx 0x%llx  U: 0x%llx 0x%llx  P: 0x%llx 0x%llx\n", sg.L[0], sg.L[1], sg.U[0], sg.U[1], sg.P[0], sg.P[1]);
  }
}

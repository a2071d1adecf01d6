// Host check of the operator tables owt_dy1_noalloc builds in its static
// device array (csrc/noalloc_setup.h) against the handle's setup
// (csrc/setup_host.cpp: make_grid, make_stencils at the reference's order):
//  - the B1 rows equal the first-derivative B stencil entry for entry, bitwise;
//  - the unfactored A1 band equals the A stencil, bitwise;
//  - c11 agrees with make_grid's to round-off;
//  - the factored band solves A1 x = b (residual at round-off).
// Built and run by tests/test_noalloc_host.py; prints one line per case and
// exits non-zero on a mismatch.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "noalloc_setup.h"
#include "setup_host.h"

using namespace owt;

static int check_case(int NY, double alpha) {
  std::vector<unsigned char> buf(noalloc_setup_bytes() + 64);
  const NoallocSetup s = noalloc_layout(buf.data());
  noalloc_assemble(s, NY, alpha);
  const Grid g = make_grid(NY, alpha);
  const Stencils st = make_stencils(NY, g.ds, 8);
  int bad = 0;
  // B1 rows: the nonzero entries of row j in increasing column order
  for (int j = 0; j < NY; ++j) {
    int e = 0;
    for (int c = 0; c < NY; ++c) {
      const double b = st.b(0, j, c);
      if (b == 0.0) continue;
      if (e >= 5 || s.bcol[j * 5 + e] != c || s.bval[j * 5 + e] != b) ++bad;
      ++e;
    }
    for (; e < 5; ++e)
      if (s.bval[j * 5 + e] != 0.0) ++bad;
  }
  // A1 band entries (row KV + i - j of column j) against the dense stencil
  for (int i = 0; i < NY; ++i)
    for (int j = 0; j < NY; ++j) {
      const int r = kNoallocKV + i - j;
      const double want = st.a(0, i, j);
      if (r < 0 || r >= kNoallocBandRows) {
        if (want != 0.0) ++bad;
        continue;
      }
      if (s.ab[r * NY + j] != want) ++bad;
    }
  double c11_dev = 0.0;
  for (int j = 0; j < NY; ++j) c11_dev = std::fmax(c11_dev, std::fabs(s.c11[j] - g.c11[j]) / std::fabs(g.c11[j]));
  // factor and solve A1 x = b with the band factors (forward with the row
  // interchanges and unit-lower multipliers, then back substitution)
  noalloc_factor(s, NY);
  std::vector<double> b(NY), x(NY);
  for (int j = 0; j < NY; ++j) b[j] = std::sin(0.37 * j + alpha) + 0.1 * j;
  x = b;
  auto AB = [&](int r, int c) { return s.ab[r * NY + c]; };
  for (int j = 0; j < NY; ++j) {
    const int off = s.piv[j];
    if (off) std::swap(x[j], x[j + off]);
    for (int t = 1; t <= kNoallocKL && j + t < NY; ++t) x[j + t] -= AB(kNoallocKV + t, j) * x[j];
  }
  for (int j = NY - 1; j >= 0; --j) {
    x[j] *= AB(kNoallocKV, j);  // the diagonal row holds 1/U_jj
    for (int t = 1; t <= kNoallocKV && j - t >= 0; ++t) x[j - t] -= AB(kNoallocKV - t, j) * x[j];
  }
  double res = 0.0, nb = 0.0;
  for (int i = 0; i < NY; ++i) {
    double r = -b[i];
    for (int j = 0; j < NY; ++j) r += st.a(0, i, j) * x[j];
    res = std::fmax(res, std::fabs(r));
    nb = std::fmax(nb, std::fabs(b[i]));
  }
  const bool ok = bad == 0 && c11_dev < 1e-14 && res / nb < 1e-13;
  std::printf("NY=%d alpha=%.2f: stencil mismatches %d, c11 max rel dev %.1e, solve residual %.1e %s\n", NY, alpha,
              bad, c11_dev, res / nb, ok ? "ok" : "FAIL");
  return ok ? 0 : 1;
}

int main() {
  int fails = 0;
  const int nys[] = {7, 17, 33, 65, 129, 257, 1025};
  const double alphas[] = {1.7, 2.0, 2.2};
  for (int ny : nys)
    for (double al : alphas) fails += check_case(ny, al);
  return fails ? 1 : 0;
}

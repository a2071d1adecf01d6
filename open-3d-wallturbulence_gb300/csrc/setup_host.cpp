// Host-side setup; see setup_host.h for what is built and why.
#include "setup_host.h"

#include <algorithm>
#include <cmath>
#include <map>
#include <numeric>
#include <stdexcept>

namespace owt {

Grid make_grid(int N, double alpha) {
  // src/solver.cpp:57-106: s uniform in [-1, 1], y = tanh(alpha s)/tanh(alpha),
  // analytic dy/ds .. d4y/ds4, and the chain-rule coefficients c11..c44.
  Grid g;
  g.N = N;
  g.ds = 2.0 / (N - 1.0);
  auto alloc = [&](std::vector<double> &v) { v.assign(N, 0.0); };
  for (auto *v : {&g.s, &g.y, &g.dyds1, &g.dyds2, &g.dyds3, &g.dyds4, &g.c11, &g.c21, &g.c22, &g.c31, &g.c32,
                  &g.c33, &g.c41, &g.c42, &g.c43, &g.c44})
    alloc(*v);
  const double ap = alpha, ap2 = std::pow(alpha, 2), ap3 = std::pow(alpha, 3), ap4 = std::pow(alpha, 4);
  const double coth_ap = 1.0 / std::tanh(ap);
  for (int i = 0; i < N; ++i) {
    g.s[i] = 2 * i / (N - 1.0) - 1.0;
    const double as = ap * g.s[i];
    const double sech = 1.0 / std::cosh(as);
    g.y[i] = std::tanh(as) / std::tanh(ap);
    g.dyds1[i] = ap * coth_ap * std::pow(sech, 2);
    g.dyds2[i] = -2 * ap2 * coth_ap * std::pow(sech, 2) * std::tanh(as);
    g.dyds3[i] = 2 * ap3 * (-2 + std::cosh(2 * as)) * coth_ap * std::pow(sech, 4);
    g.dyds4[i] = -2 * ap4 * coth_ap * std::pow(sech, 5) * (-11 * std::sinh(as) + std::sinh(3 * as));
  }
  for (int i = 0; i < N; ++i) {
    const double d1 = g.dyds1[i], d2 = g.dyds2[i], d3 = g.dyds3[i], d4 = g.dyds4[i];
    auto p = [](double x, int e) { return std::pow(x, (double)e); };
    g.c11[i] = p(d1, -1);
    g.c21[i] = -d2 * p(d1, -3);
    g.c22[i] = p(d1, -2);
    g.c31[i] = -d3 * p(d1, -4) + 3.0 * p(d2, 2) * p(d1, -5);
    g.c32[i] = -3.0 * d2 * p(d1, -4);
    g.c33[i] = p(d1, -3);
    g.c41[i] = -d4 * p(d1, -5) + 10.0 * d3 * d2 * p(d1, -6) - 15.0 * p(d2, 3) * p(d1, -7);
    g.c42[i] = -4.0 * d3 * p(d1, -5) + 15.0 * p(d2, 2) * p(d1, -6);
    g.c43[i] = -6.0 * d2 * p(d1, -5);
    g.c44[i] = p(d1, -4);
  }
  return g;
}

Stencils make_stencils(int N, double h, int order) {
  if (N < 7) throw std::invalid_argument("NY must be at least 7 for the 3rd-derivative scheme");
  if (order != 6 && order != 8) throw std::invalid_argument("compact-FD order must be 6 or 8");
  const bool six = order == 6;
  Stencils st;
  st.N = N;
  for (int q = 0; q < 4; ++q) {
    st.A[q].assign((size_t)N * N, 0.0);
    st.B[q].assign((size_t)N * N, 0.0);
  }
  auto A = [&](int q, int i, int j) -> double & { return st.A[q][(size_t)i * N + j]; };
  auto B = [&](int q, int i, int j) -> double & { return st.B[q][(size_t)i * N + j]; };
  // First derivative, src/compdiff.hpp:11-69.
  {
    // sixth order: alpha 1/3, a 14/9, b 1/9 (tridiagonal)
    const double al = six ? 1.0 / 3.0 : 4.0 / 9.0, be = six ? 0.0 : 1.0 / 36.0;
    const double a = six ? 14.0 / 9.0 : 40.0 / 27.0, b = six ? 1.0 / 9.0 : 25.0 / 54.0;
    for (int i = 2; i < N - 2; ++i) {
      A(0, i, i - 2) = be; A(0, i, i - 1) = al; A(0, i, i) = 1.0; A(0, i, i + 1) = al; A(0, i, i + 2) = be;
      B(0, i, i - 2) = -b / (4 * h); B(0, i, i - 1) = -a / (2 * h); B(0, i, i + 1) = a / (2 * h);
      B(0, i, i + 2) = b / (4 * h);
    }
    for (int i : {1, N - 2}) {
      A(0, i, i - 1) = 0.25; A(0, i, i) = 1.0; A(0, i, i + 1) = 0.25;
      B(0, i, i - 1) = -1.5 / (2 * h); B(0, i, i + 1) = 1.5 / (2 * h);
    }
    const double a0 = -17.0 / 6.0, b0 = 1.5, c0 = 1.5, d0 = -1.0 / 6.0;
    A(0, 0, 0) = 1.0; A(0, 0, 1) = 3.0; A(0, N - 1, N - 1) = 1.0; A(0, N - 1, N - 2) = 3.0;
    B(0, 0, 0) = a0 / h; B(0, 0, 1) = b0 / h; B(0, 0, 2) = c0 / h; B(0, 0, 3) = d0 / h;
    B(0, N - 1, N - 1) = -a0 / h; B(0, N - 1, N - 2) = -b0 / h; B(0, N - 1, N - 3) = -c0 / h;
    B(0, N - 1, N - 4) = -d0 / h;
  }
  // Second derivative, src/compdiff.hpp:71-166 (rows 1, N-2 centred on 2, N-3;
  // the top row's (N-1, N-4) entry is 0 and (N-1, N-5) is never set).
  {
    const double h2 = std::pow(h, 2);
    // sixth order: alpha 2/11, a 12/11, b 3/11 (tridiagonal) on rows 3..N-4;
    // rows 2, N-3 keep the reference's scheme, since rows 1, N-2 below are the
    // sixth-order scheme centred on nodes 2, N-3 and must not repeat them
    for (int i = 2; i < N - 2; ++i) {
      const bool s6 = six && i >= 3 && i <= N - 4;
      const double al = s6 ? 2.0 / 11.0 : 344.0 / 1179.0, be = s6 ? 0.0 : 23.0 / 2358.0;
      const double a = s6 ? 12.0 / 11.0 : 320.0 / 393.0, b = s6 ? 3.0 / 11.0 : 310.0 / 393.0;
      A(1, i, i - 2) = be; A(1, i, i - 1) = al; A(1, i, i) = 1.0; A(1, i, i + 1) = al; A(1, i, i + 2) = be;
      B(1, i, i - 2) = b / (4 * h2); B(1, i, i - 1) = a / h2; B(1, i, i) = -2 * b / (4 * h2) - 2 * a / h2;
      B(1, i, i + 1) = a / h2; B(1, i, i + 2) = b / (4 * h2);
    }
    const double al1 = 2.0 / 11.0, a1 = 12.0 / 11.0, b1 = 3.0 / 11.0;
    for (int i : {1, N - 2}) {
      const int c = (i == 1) ? 2 : N - 3;
      A(1, i, c - 1) = al1; A(1, i, c) = 1.0; A(1, i, c + 1) = al1;
      B(1, i, c - 2) = b1 / (4 * h2); B(1, i, c - 1) = a1 / h2; B(1, i, c) = -2 * b1 / (4 * h2) - 2 * a1 / h2;
      B(1, i, c + 1) = a1 / h2; B(1, i, c + 2) = b1 / (4 * h2);
    }
    A(1, 0, 0) = 1.0; A(1, 0, 1) = 10.0; A(1, 0, 2) = 1.0;
    A(1, N - 1, N - 1) = 1.0; A(1, N - 1, N - 2) = 10.0; A(1, N - 1, N - 3) = 1.0;
    B(1, 0, 0) = 12.0 / h2; B(1, 0, 1) = -24.0 / h2; B(1, 0, 2) = 12.0 / h2;
    B(1, N - 1, N - 1) = 12.0 / h2; B(1, N - 1, N - 2) = -24.0 / h2; B(1, N - 1, N - 3) = 12.0 / h2;
  }
  // Third derivative, src/compdiff.hpp:168-259.  Top row as coded: (N-1, N-4)
  // ends up as -e0/h^3 (written twice) and (N-1, N-5) stays 0, so this row
  // does not annihilate constants; it is reproduced on purpose.
  {
    const double h3 = std::pow(h, 3);
    // sixth order: alpha 7/16, a 2, b -1/8 (tridiagonal)
    const double al = six ? 7.0 / 16.0 : 147.0 / 332.0, be = six ? 0.0 : 1.0 / 166.0;
    const double a = six ? 2.0 : 160.0 / 83.0, b = six ? -1.0 / 8.0 : -5.0 / 166.0;
    for (int i = 3; i < N - 3; ++i) {
      A(2, i, i - 2) = be; A(2, i, i - 1) = al; A(2, i, i) = 1.0; A(2, i, i + 1) = al; A(2, i, i + 2) = be;
      B(2, i, i - 3) = -b / (8 * h3); B(2, i, i - 2) = -a / (2 * h3); B(2, i, i - 1) = a / h3 + 3 * b / (8 * h3);
      B(2, i, i + 1) = -a / h3 - 3 * b / (8 * h3); B(2, i, i + 2) = a / (2 * h3); B(2, i, i + 3) = b / (8 * h3);
    }
    const double al2 = 4.0 / 9.0, be2 = 1.0 / 126.0, a2 = 40.0 / 21.0;
    for (int i : {2, N - 3}) {
      A(2, i, i - 2) = be2; A(2, i, i - 1) = al2; A(2, i, i) = 1.0; A(2, i, i + 1) = al2; A(2, i, i + 2) = be2;
      B(2, i, i - 2) = -a2 / (2 * h3); B(2, i, i - 1) = a2 / h3; B(2, i, i + 1) = -a2 / h3;
      B(2, i, i + 2) = a2 / (2 * h3);
    }
    A(2, 1, 1) = 0.5; A(2, 1, 2) = 1.0; A(2, 1, 3) = 0.5;
    A(2, N - 2, N - 4) = 0.5; A(2, N - 2, N - 3) = 1.0; A(2, N - 2, N - 2) = 0.5;
    B(2, 1, 0) = -2.0 / (2 * h3); B(2, 1, 1) = 2.0 / h3; B(2, 1, 3) = -2.0 / h3; B(2, 1, 4) = 2.0 / (2 * h3);
    B(2, N - 2, N - 5) = -2.0 / (2 * h3); B(2, N - 2, N - 4) = 2.0 / h3; B(2, N - 2, N - 2) = -2.0 / h3;
    B(2, N - 2, N - 1) = 2.0 / (2 * h3);
    A(2, 0, 0) = 1.0; A(2, 0, 1) = -7.0; A(2, N - 1, N - 1) = 1.0; A(2, N - 1, N - 2) = -7.0;
    B(2, 0, 0) = 8.0 / h3; B(2, 0, 1) = -26.0 / h3; B(2, 0, 2) = 30.0 / h3; B(2, 0, 3) = -14.0 / h3;
    B(2, 0, 4) = 2.0 / h3;
    B(2, N - 1, N - 1) = -8.0 / h3; B(2, N - 1, N - 2) = 26.0 / h3; B(2, N - 1, N - 3) = -30.0 / h3;
    B(2, N - 1, N - 4) = -2.0 / h3;
  }
  // Fourth derivative, src/compdiff.hpp:261-357.
  {
    const double h4 = std::pow(h, 4);
    const double al = 7.0 / 26.0, a = 19.0 / 13.0, b = 1.0 / 13.0;
    for (int i = 3; i < N - 3; ++i) {
      A(3, i, i - 1) = al; A(3, i, i) = 1.0; A(3, i, i + 1) = al;
      B(3, i, i - 3) = b / (6 * h4); B(3, i, i - 2) = a / h4; B(3, i, i - 1) = -4 * a / h4 - 9 * b / (6 * h4);
      B(3, i, i) = 6 * a / h4 + 16 * b / (6 * h4); B(3, i, i + 1) = -4 * a / h4 - 9 * b / (6 * h4);
      B(3, i, i + 2) = a / h4; B(3, i, i + 3) = b / (6 * h4);
    }
    for (int i : {2, N - 3}) {
      A(3, i, i - 1) = 0.25; A(3, i, i) = 1.0; A(3, i, i + 1) = 0.25;
      B(3, i, i - 2) = 1.5 / h4; B(3, i, i - 1) = -4 * 1.5 / h4; B(3, i, i) = 6 * 1.5 / h4;
      B(3, i, i + 1) = -4 * 1.5 / h4; B(3, i, i + 2) = 1.5 / h4;
    }
    const double r1[5] = {6.0, -24.0, 36.0, -24.0, 6.0};
    A(3, 1, 0) = 1.0; A(3, 1, 1) = -2.0; A(3, 1, 2) = 7.0;
    A(3, N - 2, N - 1) = 1.0; A(3, N - 2, N - 2) = -2.0; A(3, N - 2, N - 3) = 7.0;
    for (int c = 0; c < 5; ++c) { B(3, 1, c) = r1[c] / h4; B(3, N - 2, N - 1 - c) = r1[c] / h4; }
    const double r0[5] = {-1.0, 4.0, -6.0, 4.0, -1.0};
    A(3, 0, 0) = 1.0; A(3, 0, 1) = -2.0; A(3, N - 1, N - 1) = 1.0; A(3, N - 1, N - 2) = -2.0;
    for (int c = 0; c < 5; ++c) { B(3, 0, c) = r0[c] / h4; B(3, N - 1, N - 1 - c) = r0[c] / h4; }
  }
  return st;
}

namespace {

struct Eq {
  std::map<int, Entry> e;  // by column
  int rhs_node = -1;
  int rb_eq = -1, rb_node = -1;  // omega_y-system: which B_m row feeds the rhs
  std::vector<std::pair<int, double>> rhs_w;  // v-system: (node, weight) of the rhs
  void add(int col, double t0, double t1 = 0.0, double t2 = 0.0) {
    auto it = e.find(col);
    if (it == e.end()) e[col] = Entry{col, t0, t1, t2};
    else { it->second.t0 += t0; it->second.t1 += t1; it->second.t2 += t2; }
  }
  // structural entries only (an exact zero does not widen the column span)
  void add_nz(int col, double t0, double t1 = 0.0, double t2 = 0.0) {
    if (t0 != 0.0 || t1 != 0.0 || t2 != 0.0) add(col, t0, t1, t2);
  }
};

// Order equations by the midpoint of their column span and lay the result out
// as a band template.
BandTemplate to_band(std::vector<Eq> &eqs, int n, int per_node) {
  std::vector<int> order(eqs.size());
  std::iota(order.begin(), order.end(), 0);
  std::vector<int> mid2(eqs.size());
  for (size_t q = 0; q < eqs.size(); ++q) {
    if (eqs[q].e.empty()) throw std::logic_error("empty equation");
    mid2[q] = eqs[q].e.begin()->first + eqs[q].e.rbegin()->first;
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return mid2[a] < mid2[b]; });
  BandTemplate bt;
  bt.n = n;
  bt.per_node = per_node;
  for (int p = 0; p < n; ++p)
    for (auto &kv : eqs[order[p]].e) {
      bt.kl = std::max(bt.kl, p - kv.first);
      bt.ku = std::max(bt.ku, kv.first - p);
    }
  const int nb = bt.kl + bt.ku + 1;
  bt.t0.assign((size_t)nb * n, 0.0);
  bt.t1.assign((size_t)nb * n, 0.0);
  bt.t2.assign((size_t)nb * n, 0.0);
  bt.rhs_node.assign(n, -1);
  for (int p = 0; p < n; ++p) {
    const Eq &q = eqs[order[p]];
    for (auto &kv : q.e) {
      const size_t at = (size_t)(bt.ku + p - kv.first) * n + kv.first;
      bt.t0[at] = kv.second.t0;
      bt.t1[at] = kv.second.t1;
      bt.t2[at] = kv.second.t2;
    }
    bt.rhs_node[p] = q.rhs_node;
  }
  bt.rbv_col.assign((size_t)n * 4, 0);
  bt.rbv_val.assign((size_t)n * 4, 0.0);
  for (int p = 0; p < n; ++p) {
    const Eq &q = eqs[order[p]];
    if (q.rhs_w.size() > 4) throw std::logic_error("v-system rhs wider than 4");
    for (size_t e = 0; e < q.rhs_w.size(); ++e) {
      bt.rbv_col[(size_t)p * 4 + e] = q.rhs_w[e].first;
      bt.rbv_val[(size_t)p * 4 + e] = q.rhs_w[e].second;
    }
  }
  // keep the equation order for the omega_y rhs tables
  bt.rb_col.assign((size_t)n * 5, 0);
  bt.rb_val.assign((size_t)n * 5, 0.0);
  for (int p = 0; p < n; ++p) {
    const Eq &q = eqs[order[p]];
    bt.rb_col[(size_t)p * 5] = q.rb_eq;       // placeholders, filled by the caller
    bt.rb_col[(size_t)p * 5 + 1] = q.rb_node;
  }
  return bt;
}

}  // namespace

// Column scaling: the unknown of type t >= 1 (a t-th compact derivative) is
// solved for as h^t d_t, so that every unknown has the magnitude of v.
static void scale_columns(BandTemplate &bt, const std::vector<double> &per_type) {
  const int nb = bt.kl + bt.ku + 1;
  for (int b = 0; b < nb; ++b)
    for (int c = 0; c < bt.n; ++c) {
      const double f = per_type[c % bt.per_node];
      const size_t at = (size_t)b * bt.n + c;
      bt.t0[at] *= f;
      bt.t1[at] *= f;
      bt.t2[at] *= f;
    }
}

BandTemplate build_v_system(const Grid &g, const Stencils &st, double nu) {
  const int N = g.N, n = 4 * N + 4;
  auto bnd = [&](int j) { return j < 2 || j >= N - 2; };
  auto V = [&](int t, int j) { return vcol(t, j, N); };
  std::vector<Eq> eqs;
  eqs.reserve(n);
  // boundary rows (solver.cpp:581-596): v = v_w and DY1 v = 0 on both walls
  for (int j : {0, 1, N - 2, N - 1}) {
    Eq e;
    if (j == 0) { e.add(V(0, 0), 1.0); e.rhs_node = kRhsWallBottom; }
    if (j == 1) e.add(V(1, 0), g.c11[0]);
    if (j == N - 2) e.add(V(1, N - 1), g.c11[N - 1]);
    if (j == N - 1) { e.add(V(0, N - 1), 1.0); e.rhs_node = kRhsWallTop; }
    eqs.push_back(e);
  }
  // A_m d_m - B_m v = 0, m = 1..3
  for (int m = 1; m <= 3; ++m)
    for (int j = 0; j < N; ++j) {
      Eq e;
      for (int c = 0; c < N; ++c) {
        if (st.a(m - 1, j, c) != 0.0) e.add(V(m, c), st.a(m - 1, j, c));
        if (st.b(m - 1, j, c) != 0.0) e.add(V(0, c), -st.b(m - 1, j, c));
      }
      eqs.push_back(e);
    }
  // A_4 d_4 - B_4 v = 0 with d4_c = (r_c + b v_c - G1 d1 - G2 d2 - G3 d3) / G4
  // on interior nodes c: t1 multiplies a, t2 multiplies b
  for (int j = 0; j < N; ++j) {
    Eq e;
    for (int c = 0; c < N; ++c) {
      const double a4 = st.a(3, j, c);
      if (a4 == 0.0) continue;
      if (bnd(c)) {
        e.add(V(4, c), a4);
        continue;
      }
      const double w = a4 / (-nu * g.c44[c]);
      e.add_nz(V(0, c), 0.0, 0.0, w);
      e.add_nz(V(1, c), w * nu * g.c41[c], -w * g.c21[c]);
      e.add_nz(V(2, c), w * nu * g.c42[c], -w * g.c22[c]);
      e.add_nz(V(3, c), w * nu * g.c43[c]);
      e.rhs_w.push_back({c, -w});
    }
    for (int c = 0; c < N; ++c)
      if (st.b(3, j, c) != 0.0) e.add(V(0, c), -st.b(3, j, c));
    e.rhs_node = e.rhs_w.empty() ? kRhsNone : kRhsTable;
    eqs.push_back(e);
  }
  if ((int)eqs.size() != n) throw std::logic_error("v-system: equation count");
  BandTemplate bt = to_band(eqs, n, 4);
  // column scaling: unknown of type t is solved for as h^t d_t
  const double h = g.ds;
  const int nb = bt.kl + bt.ku + 1;
  for (int c = 0; c < n; ++c) {
    int t = 0, j = 0;
    vcol_split(c, N, t, j);
    const double f = 1.0 / std::pow(h, t);
    for (int b = 0; b < nb; ++b) {
      const size_t at = (size_t)b * n + c;
      bt.t0[at] *= f;
      bt.t1[at] *= f;
      bt.t2[at] *= f;
    }
  }
  return bt;
}

BandTemplate build_g_system(const Grid &g, const Stencils &st, double nu) {
  const int N = g.N, T = 2;
  std::vector<Eq> eqs;
  for (int m = 1; m <= 2; ++m)
    for (int j = 0; j < N; ++j) {
      Eq e;
      for (int c = 0; c < N; ++c) {
        if (st.a(m - 1, j, c) != 0.0) e.add(T * c + (m - 1), st.a(m - 1, j, c));
        const double b = st.b(m - 1, j, c);
        if (b != 0.0 && c > 0 && c < N - 1) {
          // t1 multiplies 1/cg
          e.add(T * c, 0.0, -b * nu * g.c21[c]);
          e.add(T * c + 1, 0.0, -b * nu * g.c22[c]);
        }
      }
      e.rb_eq = m - 1;
      e.rb_node = j;
      eqs.push_back(e);
    }
  BandTemplate bt = to_band(eqs, T * N, T);
  scale_columns(bt, {1.0 / g.ds, 1.0 / (g.ds * g.ds)});
  // rhs tables: row p = (1/cg) * sum over interior c of B_m[j][c] r_c
  for (int p = 0; p < bt.n; ++p) {
    const int m = bt.rb_col[(size_t)p * 5], j = bt.rb_col[(size_t)p * 5 + 1];
    int k = 0;
    int cols[5] = {0, 0, 0, 0, 0};
    double vals[5] = {0, 0, 0, 0, 0};
    for (int c = 1; c < N - 1; ++c) {
      const double b = st.b(m, j, c);
      if (b != 0.0) {
        if (k >= 5) throw std::logic_error("B row wider than 5");
        cols[k] = c;
        vals[k] = b;
        ++k;
      }
    }
    for (int e = 0; e < 5; ++e) {
      bt.rb_col[(size_t)p * 5 + e] = cols[e];
      bt.rb_val[(size_t)p * 5 + e] = vals[e];
    }
  }
  return bt;
}

void pad_band(BandTemplate &bt, int kl, int ku) {
  if (kl <= bt.kl && ku <= bt.ku) return;
  const int nkl = std::max(kl, bt.kl), nku = std::max(ku, bt.ku), n = bt.n;
  const int nb = nkl + nku + 1, shift = nku - bt.ku, ob = bt.kl + bt.ku + 1;
  for (std::vector<double> *t : {&bt.t0, &bt.t1, &bt.t2}) {
    std::vector<double> w((size_t)nb * n, 0.0);
    for (int b = 0; b < ob; ++b)
      for (int c = 0; c < n; ++c) w[(size_t)(b + shift) * n + c] = (*t)[(size_t)b * n + c];
    t->swap(w);
  }
  bt.kl = nkl;
  bt.ku = nku;
}

BandTemplate build_plain_band(const Stencils &st, int which, int min_kl, int min_ku) {
  const int N = st.N;
  BandTemplate bt;
  bt.n = N;
  bt.per_node = 1;
  for (int i = 0; i < N; ++i)
    for (int c = 0; c < N; ++c)
      if (st.a(which, i, c) != 0.0) {
        bt.kl = std::max(bt.kl, i - c);
        bt.ku = std::max(bt.ku, c - i);
      }
  const int nb = bt.kl + bt.ku + 1;
  bt.t0.assign((size_t)nb * N, 0.0);
  bt.t1.assign((size_t)nb * N, 0.0);
  bt.t2.assign((size_t)nb * N, 0.0);
  for (int i = 0; i < N; ++i)
    for (int c = 0; c < N; ++c)
      if (st.a(which, i, c) != 0.0) bt.t0[(size_t)(bt.ku + i - c) * N + c] = st.a(which, i, c);
  bt.rhs_node.assign(N, -1);
  pad_band(bt, min_kl, min_ku);
  return bt;
}

std::vector<double> twiddles(int L) {
  std::vector<double> t(2 * (size_t)L);
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (int k = 0; k < L; ++k) {
    const long double a = two_pi * (long double)k / (long double)L;
    t[2 * k] = (double)std::cos(a);
    t[2 * k + 1] = (double)(-std::sin(a));
  }
  return t;
}

bool fft_radices(int L, std::vector<int> &r) {
  r.clear();
  int m = L;
  while (m % 4 == 0) { r.push_back(4); m /= 4; }
  while (m % 2 == 0) { r.push_back(2); m /= 2; }
  while (m % 3 == 0) { r.push_back(3); m /= 3; }
  while (m % 5 == 0) { r.push_back(5); m /= 5; }
  return m == 1 && r.size() <= 8;
}

}  // namespace owt

// Creation and teardown of a handle: grid, metric and compact-FD operators
// on the host (setup_host.cpp), per-mode band factorizations and the check of
// their interior fill on the device, the device tables and buffers; plus the
// status check of synchronising calls.
#include "handle.h"

using namespace owt;

namespace owt {
thread_local size_t *g_alloc_counter = nullptr;
}  // namespace owt

owt_handle::~owt_handle() {
  if (st) cudaStreamSynchronize(st);
  if (gexec) cudaGraphExecDestroy(gexec);
  if (graph) cudaGraphDestroy(graph);
  for (void *q : owned) cudaFree(q);
  for (cudaEvent_t e : {ev_fork, ev_join, ev_fork2, ev_join2})
    if (e) cudaEventDestroy(e);
  if (hs.ready) {
    for (cudaStream_t q : {hs.up, hs.tx, hs.aux, hs.down}) cudaStreamSynchronize(q);
    for (int j = 0; j < HostStep::kChunks; ++j)
      for (cudaEvent_t e : {hs.landed[j], hs.v_done[j], hs.q_done[j], hs.tx_done[j]})
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : {hs.up_done, hs.after_modes, hs.down_done})
      if (e) cudaEventDestroy(e);
    for (cudaStream_t q : {hs.up, hs.tx, hs.aux, hs.down}) cudaStreamDestroy(q);
    if (hs.fric_pin) cudaFreeHost(hs.fric_pin);
  }
  if (st2) cudaStreamDestroy(st2);
  if (st) cudaStreamDestroy(st);
}

void owt_handle::check_launch(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

void owt_handle::setup(const owt_params &prm) {
  using clk = std::chrono::steady_clock;
  auto t_last = clk::now();
  auto phase = [&](const char *name) {
    const auto t = clk::now();
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%s%s %.2fms", setup_report.empty() ? "" : ", ", name,
                  std::chrono::duration<double, std::milli>(t - t_last).count());
    setup_report += buf;
    t_last = t;
  };
  g_alloc_counter = &device_bytes;
  struct Reset { ~Reset() { g_alloc_counter = nullptr; } } reset_counter;
  p = prm;
  NX = (int)p.NX; NY = (int)p.NY; NZ = (int)p.NZ;
  if (p.NX < 4 || p.NZ < 4 || p.NX % 2 || p.NZ % 2)
    throw OwtError(OWT_ERR_INVALID, "NX and NZ must be even and at least 4");
  if (p.NY < 7) throw OwtError(OWT_ERR_INVALID, "N must be at least 7 for 3rd derivative scheme");
  if (!(p.dt > 0) || !(p.nu > 0) || !(p.dkx > 0) || !(p.dkz > 0) || !(p.alpha_mesh > 0))
    throw OwtError(OWT_ERR_INVALID, "dt, nu, dkx, dkz and alpha_mesh must be positive");
  if (p.precision != OWT_PREC_FP64 && p.precision != OWT_PREC_MIXED)
    throw OwtError(OWT_ERR_INVALID, "precision must be OWT_PREC_FP64 or OWT_PREC_MIXED");
  if (p.fd_order != 0 && p.fd_order != 6 && p.fd_order != 8)
    throw OwtError(OWT_ERR_INVALID, "fd_order must be 0 or 8 (the reference's schemes) or 6");
  NXH = NX / 2; NZH = NZ / 2; NX2 = NX / 2 * 3; NZ2 = NZ / 2 * 3;
  M = NZ * NXH;
  Uq = NXH * (NZH + 1);
  fs = (size_t)NY * M;
  precision = p.precision;
  std::vector<int> rx, rz;
  if (!fft_radices(NX2, rx) || !fft_radices(NZ2, rz))
    throw OwtError(OWT_ERR_INVALID, "3NX/2 and 3NZ/2 must be of the form 2^a 3^b 5^c");
  if (NX2 > 1024 || NZ2 > 1024)
    throw OwtError(OWT_ERR_INVALID, "3NX/2 and 3NZ/2 must not exceed 1024 (one thread per point of a line)");
  if (!make_fft_plan(NX2, rx.data(), (int)rx.size(), px) || !make_fft_plan(NZ2, rz.data(), (int)rz.size(), pz))
    throw OwtError(OWT_ERR_INVALID, "3NX/2 and 3NZ/2 need at most 8 FFT stages");
  ck(cudaSetDevice(p.device), "cudaSetDevice");
  ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
  {
    // the mean mode's branch at the highest priority: its single block must
    // not wait for a slot behind the mode kernel's blocks (it would then add
    // its whole duration to the step)
    int lo = 0, hi = 0;
    ck(cudaDeviceGetStreamPriorityRange(&lo, &hi), "stream priorities");
    ck(cudaStreamCreateWithPriority(&st2, cudaStreamNonBlocking, hi), "cudaStreamCreate");
  }
  ck(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming), "cudaEventCreate");
  ck(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming), "cudaEventCreate");
  ck(cudaEventCreateWithFlags(&ev_fork2, cudaEventDisableTiming), "cudaEventCreate");
  ck(cudaEventCreateWithFlags(&ev_join2, cudaEventDisableTiming), "cudaEventCreate");

  // grid, metric, stencils, band templates (host, FP64)
  grid = make_grid(NY, p.alpha_mesh);
  Ly = grid.y[NY - 1] - grid.y[0];
  Stencils sten = make_stencils(NY, grid.ds, p.fd_order == 6 ? 6 : 8);
  BandTemplate tv = build_v_system(grid, sten, p.nu);
  BandTemplate tg = build_g_system(grid, sten, p.nu);
  BandTemplate t1 = build_plain_band(sten, 0);
  BandTemplate t2 = build_plain_band(sten, 1);
  // the kernels are specialised for the bands of the reference's stencils
  pad_band(tv, kVKL, kVKU);
  pad_band(tg, 6, 6);
  for (const BandTemplate *t : {&tv, &tg, &t1, &t2})
    if (!band_supported(t->kl, t->ku))
      throw OwtError(OWT_ERR_INVALID, "unsupported band width " + std::to_string(t->kl) + "/" + std::to_string(t->ku));

  // wavenumbers exactly as allocate_var (src/solver.cpp:25-37, one rank)
  std::vector<double> hkx(NXH), hkz(NZ);
  for (int i = 0; i < NXH; ++i) hkx[i] = (double)i * p.dkx;
  for (int k = 0; k < NZ; ++k) {
    double t = (double)k;
    if (t >= (double)NZH) t -= (double)NZ;
    hkz[k] = t * p.dkz;
  }
  // per unique mode (|kz| index, kx index): a, b of Av and 1/cg of Ag
  const double g0 = 11.0 / 6.0, dt = p.dt, nu = p.nu;
  std::vector<double> sa(Uq), sb(Uq), icg(Uq);
  for (int kabs = 0; kabs <= NZH; ++kabs)
    for (int i = 0; i < NXH; ++i) {
      const double kxv = hkx[i], kzv = hkz[kabs == NZH ? NZH : kabs];
      const double k2 = std::pow(kxv, 2) + std::pow(kzv, 2), k4 = std::pow(k2, 2);
      const int uq = kabs * NXH + i;
      sa[uq] = g0 / dt + 2 * nu * k2;
      sb[uq] = nu * k4 + g0 * k2 / dt;
      icg[uq] = 1.0 / (nu * k2 + g0 / dt);
    }
  inv_cg0 = icg[0];

  kx = upload(hkx, owned, st);
  kz = upload(hkz, owned, st);
  c11 = upload(grid.c11, owned, st);
  c21 = upload(grid.c21, owned, st);
  c22 = upload(grid.c22, owned, st);
  {
    std::vector<double> a21(NY), a22(NY);
    for (int j = 0; j < NY; ++j) { a21[j] = p.nu * grid.c21[j]; a22[j] = p.nu * grid.c22[j]; }
    nc21 = upload(a21, owned, st);
    nc22 = upload(a22, owned, st);
    const double ih = 1.0 / grid.ds, ih2 = 1.0 / (grid.ds * grid.ds);
    std::vector<double> h11(NY), h21(NY), h22(NY), hn21(NY), hn22(NY);
    for (int j = 0; j < NY; ++j) {
      h11[j] = grid.c11[j] * ih;
      h21[j] = grid.c21[j] * ih;
      h22[j] = grid.c22[j] * ih2;
      hn21[j] = a21[j] * ih;
      hn22[j] = a22[j] * ih2;
    }
    c11h = upload(h11, owned, st);
    c21h = upload(h21, owned, st);
    c22h = upload(h22, owned, st);
    nc21h = upload(hn21, owned, st);
    nc22h = upload(hn22, owned, st);
  }
  inv_cg = upload(icg, owned, st);
  d_step = dalloc<long long>(1, owned);
  d_err = dalloc<int>(1, owned);
  ck(cudaMemsetAsync(d_step, 0, sizeof(long long), st), "memset");
  ck(cudaMemsetAsync(d_err, 0, sizeof(int), st), "memset");

  ck(cudaStreamSynchronize(st), "setup");
  phase("host operators");
  // band factorizations
  double *d_sa = upload(sa, owned, st), *d_sb = upload(sb, owned, st), *d_icg = inv_cg;
  auto factor = [&](BandDev &bd, const BandTemplate &t, int U, const double *s1, const double *s2, bool rows) {
    bd.n = t.n; bd.kl = t.kl; bd.ku = t.ku;
    const size_t nb = 2 * (size_t)t.kl + t.ku + 1;
    bd.ab = dalloc<double>(nb * t.n * (size_t)U, owned);
    bd.piv = dalloc<uint8_t>((size_t)t.n * U, owned);
    if (rows) bd.rscale = dalloc<double>((size_t)t.n * U, owned);
    std::vector<void *> tmp;
    double *d0 = upload(t.t0, tmp, st), *d1 = upload(t.t1, tmp, st), *d2 = upload(t.t2, tmp, st);
    launch_band_factor(t.kl, t.ku, bd.ab, bd.piv, t.n, U, d0, d1, d2, s1, s2, bd.rscale, d_err, st);
    ++launches;
    check_launch("band factorization");
    ck(cudaStreamSynchronize(st), "band factorization");
    for (void *q : tmp) cudaFree(q);
  };
  factor(bv, tv, Uq, d_sa, d_sb, true);
  factor(bg, tg, Uq, d_icg, nullptr, true);
  rs_gi = dalloc<double>((size_t)bg.n * Uq, owned);
  launch_scale_by_mode(rs_gi, bg.rscale, inv_cg, bg.n, Uq, st);
  ++launches;
  factor(b1, t1, 1, nullptr, nullptr, false);
  factor(b2, t2, 1, nullptr, nullptr, false);
  int herr = 0;
  ck(cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost), "factor status");
  if (herr) throw OwtError(OWT_ERR_NUMERIC, "LU factorization failed. Matrix A may be singular.");
  phase("band factorizations");
  // interior fill of both systems inside the compile-time masks? then the
  // masked solves apply
  sparse_v = sparse_v6 = false;
  // (systems shorter than the two edges have no masked blocks: full band)
  if (bv.n % 4 == 0 && bg.n % 2 == 0) {
    int *d_bad = dalloc<int>(2, owned);
    ck(cudaMemsetAsync(d_bad, 0, 2 * sizeof(int), st), "memset");
    launch_check_pattern(p.fd_order == 6 ? 2 : 0, bv.ab, bv.piv, bv.n, Uq, d_bad, st);
    launch_check_pattern(1, bg.ab, bg.piv, bg.n, Uq, d_bad + 1, st);
    launches += 2;
    int nbad[2] = {0, 0};
    ck(cudaMemcpyAsync(nbad, d_bad, 2 * sizeof(int), cudaMemcpyDeviceToHost, st), "pattern check");
    ck(cudaStreamSynchronize(st), "pattern check");
    (p.fd_order == 6 ? sparse_v6 : sparse_v) = (nbad[0] == 0 && nbad[1] == 0);
    pattern_violations = nbad[0] + nbad[1];
  }
  phase("pattern check");
  rhs_node_v = upload(tv.rhs_node, owned, st);
  rbv_col = upload(tv.rbv_col, owned, st);
  rbv_val = upload(tv.rbv_val, owned, st);
  rb_col = upload(tg.rb_col, owned, st);
  rb_val = upload(tg.rb_val, owned, st);
  // B1 / B2 rows as (col, val) x 5
  auto brows = [&](int which, int *&dcol, double *&dval) {
    std::vector<int> cols((size_t)NY * 5, 0);
    std::vector<double> vals((size_t)NY * 5, 0.0);
    for (int j = 0; j < NY; ++j) {
      int e = 0;
      for (int c = 0; c < NY; ++c) {
        const double b = sten.b(which, j, c);
        if (b != 0.0) {
          if (e >= 5) throw std::logic_error("stencil row wider than 5");
          // the nonlinear-source kernel applies B1 with four taps per row
          if (which == 0 && e >= 4) throw std::logic_error("first-derivative stencil row wider than 4");
          cols[(size_t)j * 5 + e] = c;
          vals[(size_t)j * 5 + e] = b;
          ++e;
        }
      }
    }
    dcol = upload(cols, owned, st);
    dval = upload(vals, owned, st);
  };
  brows(0, b1_col, b1_val);
  brows(1, b2_col, b2_val);
  {
    std::vector<int> cols((size_t)NY * 8, 0);
    std::vector<double> vals((size_t)NY * 8, 0.0);
    std::vector<int> cnt(NY, 0);
    for (int j = 0; j < NY; ++j)
      for (int c = 0; c < NY; ++c) {
        const double b = sten.b(0, j, c);
        if (b == 0.0) continue;
        if (cnt[c] >= 8) throw std::logic_error("stencil column wider than 8");
        cols[(size_t)c * 8 + cnt[c]] = j;
        vals[(size_t)c * 8 + cnt[c]] = b;
        ++cnt[c];
      }
    b1t_col = upload(cols, owned, st);
    b1t_val = upload(vals, owned, st);
  }

  // state and scratch
  v_ring = dalloc<double2>(3 * fs, owned);
  g_ring = dalloc<double2>(3 * fs, owned);
  hv_ring = dalloc<double2>(3 * fs, owned);
  hg_ring = dalloc<double2>(3 * fs, owned);
  q_ring = dalloc<double2>(3 * fs, owned);
  for (double2 **f : {&u, &w, &ox, &oz, &lx, &ly, &lz, &sg, &dg, &sv, &bf, &yscr, &tmpA, &tmpB, &tmpC, &stage})
    *f = dalloc<double2>(fs, owned);
  lm = dalloc<float2>(3 * fs, owned);
  {
    std::vector<double> wyh(NY, 0.0);
    double tot = 0.0;
    for (int j = 0; j + 1 < NY; ++j) {
      const double h = grid.y[j + 1] - grid.y[j];
      wyh[j] += 0.5 * h;
      wyh[j + 1] += 0.5 * h;
    }
    for (double x : wyh) tot += x;
    for (double &x : wyh) x /= tot;
    ygrid = upload(grid.y, owned, st);
    wy = upload(wyh, owned, st);
    ic_partial = dalloc<double>(ic_partial_values(), owned);
  }
  yv = dalloc<double2>((size_t)bv.n * M, owned);
  yg = dalloc<double2>((size_t)bg.n * M, owned);
  U_ring = dalloc<double2>(3 * (size_t)NY, owned);
  W_ring = dalloc<double2>(3 * (size_t)NY, owned);
  lxm_ring = dalloc<double2>(3 * (size_t)NY, owned);
  lzm_ring = dalloc<double2>(3 * (size_t)NY, owned);
  fx_ring = dalloc<double>(3, owned);
  fz_ring = dalloc<double>(3, owned);
  mean_scratch = dalloc<double2>(2 * (size_t)NY + 2 * (size_t)bg.n, owned);
  mean_dy1 = dalloc<double2>(2 * (size_t)NY, owned);
  XformDims xd{NY, NZ, NXH, NZH, NX2, NZ2};
  ck(lamb_prepare(xd), "transform kernel attributes");
  ck(phys_prepare(xd), "transform kernel attributes");
  mean_smem = mean_prepare(NY, bg.n);
  zbuf = dalloc<unsigned char>(lamb_zbuf_bytes(xd, 0), owned);
  lbuf = dalloc<unsigned char>(lamb_lbuf_bytes(xd, 0), owned);
  for (int prec = 0; prec < 2; ++prec) {
    for (int axis = 0; axis < 2; ++axis) {
      const int L = axis == 0 ? NX2 : NZ2;
      std::vector<double> t = twiddles(L);
      void *d;
      if (prec == 0) {
        d = upload(t, owned, st);
      } else {
        std::vector<float> tf(t.begin(), t.end());
        d = upload(tf, owned, st);
      }
      (axis == 0 ? twx : twz)[prec] = d;
    }
  }
  for (double2 *ring : {v_ring, g_ring, hv_ring, hg_ring, q_ring})
    ck(cudaMemsetAsync(ring, 0, 3 * fs * sizeof(double2), st), "memset");
  for (double2 *f : {u, w, ox, oz, lx, ly, lz})
    ck(cudaMemsetAsync(f, 0, fs * sizeof(double2), st), "memset");
  ck(cudaStreamSynchronize(st), "setup");
  phase("fields and tables");
  tuning = "not tuned yet (the variants are timed before the handle's first own step)";
}

void owt_handle::drop_graph() {
  if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
  if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
}

void owt_handle::free_owned(void *q) {
  for (auto it = owned.begin(); it != owned.end(); ++it)
    if (*it == q) { owned.erase(it); break; }
  cudaFree(q);
}

void owt_handle::d2d(void *dst, const void *src, size_t bytes) {
  ck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st), "device copy");
}

void owt_handle::sync_and_check() {
  ck(cudaStreamSynchronize(st), "synchronize");
  int e = 0;
  ck(cudaMemcpy(&e, d_err, sizeof(int), cudaMemcpyDeviceToHost), "status");
  if (e == 2) throw OwtError(OWT_ERR_NUMERIC, "non-finite friction force: the state has blown up");
  if (e) throw OwtError(OWT_ERR_NUMERIC, "device reported a numeric failure");
}

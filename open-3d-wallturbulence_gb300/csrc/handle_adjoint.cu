// The wall-drag adjoint driver of a handle: full-state images, the forward
// run with checkpoints, and the reverse sweep that recomputes each segment
// and runs the adjoint step kernels (adjoint.cu) backwards through it; with
// their C entry points.
#include "handle.h"

using namespace owt;

// full state: the five 3-slot rings, the four mean rings, the friction rings
void owt_handle::save_image(double2 *img, int64_t &step_out) {
  double2 *o = img;
  for (double2 *ring : {v_ring, g_ring, hv_ring, hg_ring, q_ring}) { d2d(o, ring, 3 * fs * sizeof(double2)); o += 3 * fs; }
  for (double2 *ring : {U_ring, W_ring, lxm_ring, lzm_ring}) { d2d(o, ring, 3 * (size_t)NY * sizeof(double2)); o += 3 * NY; }
  d2d(o, fx_ring, 3 * sizeof(double));
  d2d(reinterpret_cast<double *>(o) + 3, fz_ring, 3 * sizeof(double));
  step_out = steps;
}

void owt_handle::load_image(const double2 *img, int64_t step) {
  const double2 *o = img;
  for (double2 *ring : {v_ring, g_ring, hv_ring, hg_ring, q_ring}) { d2d(ring, o, 3 * fs * sizeof(double2)); o += 3 * fs; }
  for (double2 *ring : {U_ring, W_ring, lxm_ring, lzm_ring}) { d2d(ring, o, 3 * (size_t)NY * sizeof(double2)); o += 3 * NY; }
  d2d(fx_ring, o, 3 * sizeof(double));
  d2d(fz_ring, reinterpret_cast<const double *>(o) + 3, 3 * sizeof(double));
  steps = step;
  staged_step = (long long)step;
  ck(cudaMemcpyAsync(d_step, &staged_step, sizeof(long long), cudaMemcpyHostToDevice, st), "step counter");
  ck(cudaStreamSynchronize(st), "step counter");
}

double owt_handle::drag_forward(int64_t n, int64_t interval) {
  if (precision != OWT_PREC_FP64)
    throw OwtError(OWT_ERR_INVALID, "the wall-drag adjoint differentiates the FP64 step: set OWT_PREC_FP64");
  if (n < 1 || interval < 1) throw OwtError(OWT_ERR_INVALID, "nsteps and interval must be positive");
  recompute_dirty_q();
  const int64_t nseg = (n + interval - 1) / interval;
  while ((int64_t)adj.ckpt.size() < nseg + 1) adj.ckpt.push_back(dalloc<double2>(image_values(), owned));
  adj.ckpt_step.assign(nseg + 1, 0);
  if (!adj.obj) adj.obj = dalloc<double>(1, owned);
  ck(cudaMemsetAsync(adj.obj, 0, sizeof(double), st), "memset");
  const double wgt = 1.0 / (double)n;
  for (int64_t sg_ = 0; sg_ < nseg; ++sg_) {
    save_image(adj.ckpt[sg_], adj.ckpt_step[sg_]);
    const int64_t len = std::min(interval, n - sg_ * interval);
    for (int64_t t = 0; t < len; ++t) {
      run_steps(1);
      launch_objective_add(fx_ring, d_step, wgt, adj.obj, st);
      ++launches;
    }
  }
  save_image(adj.ckpt[nseg], adj.ckpt_step[nseg]);
  double J = 0.0;
  ck(cudaMemcpyAsync(&J, adj.obj, sizeof(double), cudaMemcpyDeviceToHost, st), "objective");
  sync_and_check();
  adj.nsteps = n;
  adj.interval = interval;
  adj.version = state_version;
  return J;
}

void owt_handle::adj_alloc() {
  if (adj.ready) return;
  for (auto &h3 : adj.hist)
    for (auto &p3 : h3) p3 = dalloc<double2>(fs, owned);
  for (auto &m3 : adj.mean)
    for (auto &p3 : m3) p3 = dalloc<double2>(NY, owned);
  adj.fric_block = dalloc<double>(6, owned);
  for (int q = 0; q < 2; ++q)
    for (int l = 0; l < 3; ++l) adj.fric[q][l] = adj.fric_block + 3 * q + l;
  for (auto &p3 : adj.lb) p3 = dalloc<double2>(fs, owned);
  for (auto &p3 : adj.fb) p3 = dalloc<double2>(fs, owned);
  for (auto &p3 : adj.xs) p3 = dalloc<double2>(fs, owned);
  const XformDims xd{NY, NZ, NXH, NZH, NX2, NZ2};
  adj.zbuf = dalloc<double2>(adj_zbuf_values(xd), owned);
  adj.lbuf = dalloc<double2>(adj_lbuf_values(xd), owned);
  adj.yv = dalloc<double2>((size_t)bv.n * M, owned);
  adj.yg = dalloc<double2>((size_t)bg.n * M, owned);
  adj.mscr = dalloc<double2>(2 * (3 * (size_t)NY + bg.n), owned);
  adj.grad = dalloc<double2>(2 * (size_t)M, owned);
  ck(adj_lamb_prepare(xd), "adjoint transform kernel attributes");
  adj.ready = true;
}

void owt_handle::adjoint_step(const double2 *tp, double wgt) {
  AdjNLArgs na{};
  na.NY = NY; na.NXH = NXH; na.M = M; na.kx = kx; na.kz = kz; na.c11 = c11;
  na.hvb = adj.hist[2][0]; na.hgb = adj.hist[3][0]; na.lxmb = adj.mean[2][0]; na.lzmb = adj.mean[3][0];
  na.lxb = adj.lb[0]; na.lyb = adj.lb[1]; na.lzb = adj.lb[2];
  na.ab1 = b1.ab; na.piv1 = b1.piv; na.b1t_col = b1t_col; na.b1t_val = b1t_val;
  na.ys = adj.xs[0]; na.ws = adj.xs[1];
  launch_adj_nl(na, st);

  AdjXformArgs xa{};
  xa.d = XformDims{NY, NZ, NXH, NZH, NX2, NZ2};
  for (int f = 0; f < 6; ++f) { xa.st[f] = tp + (size_t)f * fs; xa.out[f] = adj.fb[f]; }
  for (int f = 0; f < 3; ++f) xa.lb[f] = adj.lb[f];
  xa.zbuf = adj.zbuf; xa.lbuf = adj.lbuf; xa.px = px; xa.pz = pz;
  xa.twx = static_cast<const double2 *>(twx[0]); xa.twz = static_cast<const double2 *>(twz[0]);
  xa.inv_n = 1.0 / ((double)NX2 * (double)NZ2);
  launch_adj_lamb(xa, st);

  AdjMeanArgs ma{};
  ma.NY = NY; ma.M = M; ma.U = Uq; ma.n_g = bg.n;
  ma.inv_dt = 1.0 / p.dt; ma.nu = p.nu; ma.Ly = Ly; ma.inv_cg0 = inv_cg0;
  ma.inv_h = 1.0 / grid.ds; ma.inv_h2 = 1.0 / (grid.ds * grid.ds); ma.weight = wgt;
  ma.c11 = c11; ma.c21 = c21; ma.c22 = c22;
  ma.ab_g = bg.ab; ma.piv_g = bg.piv; ma.rb_col = rb_col; ma.rb_val = rb_val; ma.rs_g = bg.rscale;
  ma.ub = adj.fb[0]; ma.wb = adj.fb[2]; ma.oxb = adj.fb[3]; ma.ozb = adj.fb[5];
  for (int l = 0; l < 3; ++l) {
    ma.Ub[l] = adj.mean[0][l]; ma.Wb[l] = adj.mean[1][l]; ma.Lxb[l] = adj.mean[2][l]; ma.Lzb[l] = adj.mean[3][l];
    ma.fxb[l] = adj.fric[0][l]; ma.fzb[l] = adj.fric[1][l];
  }
  ma.scratch = adj.mscr;
  // the mean mode's adjoint (one block) on the high-priority second stream,
  // beside the mode kernel's: they share only read-only inputs (the adjoint
  // fields of the Lamb vector) and write disjoint buffers
  ck(cudaEventRecord(ev_fork, st), "fork");
  ck(cudaStreamWaitEvent(st2, ev_fork, 0), "fork wait");
  launch_adj_mean(ma, st2);
  ck(cudaEventRecord(ev_join, st2), "join");

  AdjModeArgs mo{};
  mo.NY = NY; mo.NZ = NZ; mo.NXH = NXH; mo.NZH = NZH; mo.M = M; mo.U = Uq;
  mo.inv_dt = 1.0 / p.dt; mo.nu = p.nu; mo.inv_h = 1.0 / grid.ds; mo.inv_h2 = 1.0 / (grid.ds * grid.ds);
  mo.kx = kx; mo.kz = kz; mo.c11 = c11; mo.c21 = c21; mo.c22 = c22; mo.inv_cg = inv_cg;
  mo.ab_v = bv.ab; mo.piv_v = bv.piv; mo.n_v = bv.n; mo.rhs_node_v = rhs_node_v; mo.rs_v = bv.rscale;
  mo.rbv_col = rbv_col; mo.rbv_val = rbv_val;
  mo.ab_g = bg.ab; mo.piv_g = bg.piv; mo.n_g = bg.n; mo.rb_col = rb_col; mo.rb_val = rb_val; mo.rs_g = bg.rscale;
  mo.ub = adj.fb[0]; mo.vb = adj.fb[1]; mo.wb = adj.fb[2]; mo.oxb = adj.fb[3]; mo.gb = adj.fb[4]; mo.ozb = adj.fb[5];
  for (int l = 0; l < 3; ++l) {
    mo.v[l] = adj.hist[0][l]; mo.g[l] = adj.hist[1][l]; mo.hv[l] = adj.hist[2][l];
    mo.hg[l] = adj.hist[3][l]; mo.q[l] = adj.hist[4][l];
  }
  mo.grad = adj.grad; mo.yv = adj.yv; mo.yg = adj.yg;
  mo.xv0 = adj.xs[0]; mo.xv1 = adj.xs[1]; mo.xv2 = adj.xs[2]; mo.xg0 = adj.xs[3]; mo.xg1 = adj.xs[4];
  mo.sgb = adj.xs[5]; mo.svb = adj.xs[6];
  launch_adj_modes(mo, force_dense ? 0 : sparse_v ? 1 : sparse_v6 ? 2 : 0, st);
  ck(cudaStreamWaitEvent(st, ev_join, 0), "join wait");
  launches += 6;
  check_launch("adjoint step");
  // the buffers now hold the adjoints of the levels the step read, level l
  // of the old state in buffer l + 1 (mod 3)
  auto rot = [](auto *x) { auto t = x[0]; x[0] = x[1]; x[1] = x[2]; x[2] = t; };
  for (auto &h3 : adj.hist) rot(h3);
  for (auto &m3 : adj.mean) rot(m3);
  for (auto &f3 : adj.fric) rot(f3);
}

void owt_handle::drag_backward(double gJ, double *grad_bottom, double *grad_top) {
  if (adj.nsteps == 0 || adj.version != state_version)
    throw OwtError(OWT_ERR_STATE, "owt_drag_forward must come first, with no change of state or wall velocity since");
  adj_alloc();
  if (adj.tape_len < adj.interval) {
    if (adj.tape) free_owned(adj.tape);
    adj.tape = nullptr;
    adj.tape = dalloc<double2>(6 * fs * (size_t)adj.interval, owned);
    adj.tape_len = adj.interval;
  }
  for (auto &h3 : adj.hist)
    for (double2 *q : h3) ck(cudaMemsetAsync(q, 0, fs * sizeof(double2), st), "memset");
  for (auto &m3 : adj.mean)
    for (double2 *q : m3) ck(cudaMemsetAsync(q, 0, NY * sizeof(double2), st), "memset");
  ck(cudaMemsetAsync(adj.fric_block, 0, 6 * sizeof(double), st), "memset");
  ck(cudaMemsetAsync(adj.grad, 0, 2 * (size_t)M * sizeof(double2), st), "memset");
  const double wgt = gJ / (double)adj.nsteps;
  const int64_t nseg = (adj.nsteps + adj.interval - 1) / adj.interval;
  for (int64_t sg_ = nseg - 1; sg_ >= 0; --sg_) {
    load_image(adj.ckpt[sg_], adj.ckpt_step[sg_]);
    const int64_t len = std::min(adj.interval, adj.nsteps - sg_ * adj.interval);
    for (int64_t t = 0; t < len; ++t) {
      run_steps(1);
      double2 *tp = adj.tape + 6 * fs * (size_t)t;
      const double2 *src[6] = {u, ring_level(v_ring, 0), w, ox, ring_level(g_ring, 0), oz};
      for (int f = 0; f < 6; ++f) d2d(tp + (size_t)f * fs, src[f], fs * sizeof(double2));
    }
    for (int64_t t = len - 1; t >= 0; --t) adjoint_step(adj.tape + 6 * fs * (size_t)t, wgt);
  }
  load_image(adj.ckpt[nseg], adj.ckpt_step[nseg]);
  ck(cudaMemcpyAsync(grad_bottom, adj.grad, (size_t)M * sizeof(double2), cudaMemcpyDeviceToHost, st), "D2H");
  ck(cudaMemcpyAsync(grad_top, adj.grad + M, (size_t)M * sizeof(double2), cudaMemcpyDeviceToHost, st), "D2H");
  sync_and_check();
}

extern "C" {

int owt_drag_forward(owt_handle *h, int64_t nsteps, int64_t interval, double *objective) {
  return guard(h, [&] {
    if (!h->initialized) throw OwtError(OWT_ERR_STATE, "owt_init_fields (or field uploads) must come first");
    if (!objective) throw OwtError(OWT_ERR_INVALID, "null objective");
    *objective = h->drag_forward(nsteps, interval);
  });
}

int owt_drag_backward(owt_handle *h, double grad_objective, double *grad_bottom, double *grad_top) {
  return guard(h, [&] {
    if (!grad_bottom || !grad_top) throw OwtError(OWT_ERR_INVALID, "null gradient buffer");
    h->drag_backward(grad_objective, grad_bottom, grad_top);
  });
}

}  // extern "C"

// The time step of a handle: the launch sequence of one step
// (src/solver.cpp:541-627) and its CUDA graph, the mode-kernel autotuner,
// the reference routines run one at a time, init_fields, and the layout
// transposes of host <-> device copies.
#include "handle.h"

using namespace owt;

void owt_handle::dapply(int order, const double2 *in, double2 *out) {
  DApplyArgs a{};
  a.NY = NY; a.M = M; a.in = in; a.out = out;
  const BandDev &b = order == 1 ? b1 : b2;
  a.ab = b.ab; a.piv = b.piv;
  a.b_col = order == 1 ? b1_col : b2_col;
  a.b_val = order == 1 ? b1_val : b2_val;
  a.bf = bf; a.yscr = yscr;
  launch_dapply(a, st);
  ++launches;
}

XformArgs owt_handle::xform_args() const {
  XformArgs a{};
  a.d = XformDims{NY, NZ, NXH, NZH, NX2, NZ2};
  a.in[0] = u; a.in[1] = v_ring; a.in[2] = w; a.in[3] = ox; a.in[4] = g_ring; a.in[5] = oz;
  a.ring_mask = (1 << 1) | (1 << 4);
  a.fs = fs;
  a.step = d_step;
  a.mean_split = (precision == OWT_PREC_MIXED && mean_split) ? 1 : 0;
  for (int f = 0; f < 3; ++f) a.lm[f] = lm + (size_t)f * fs;
  a.out[0] = lx; a.out[1] = ly; a.out[2] = lz;
  a.zbuf = zbuf; a.lbuf = lbuf;
  a.px = px; a.pz = pz;
  a.twx = twx[precision]; a.twz = twz[precision];
  a.inv_nx2 = 1.0 / (double)NX2; a.inv_nz2 = 1.0 / (double)NZ2;
  a.stockham = fft_stockham ? 1 : 0;
  return a;
}

NLArgs owt_handle::nl_args(bool record_mean) const {
  NLArgs a{};
  a.NY = NY; a.NZ = NZ; a.NXH = NXH; a.M = M;
  a.kx = kx; a.kz = kz; a.c11 = c11;
  a.lx = lx; a.ly = ly; a.lz = lz;
  a.hv_ring = hv_ring; a.hg_ring = hg_ring;
  a.ab1 = b1.ab; a.piv1 = b1.piv; a.b1_col = b1_col; a.b1_val = b1_val;
  a.fscr = bf;
  a.yscr = yscr;
  a.lx_mean = record_mean ? lxm_ring : nullptr;
  a.lz_mean = record_mean ? lzm_ring : nullptr;
  a.step = d_step;
  return a;
}

// One time step.  Every argument is a fixed device pointer; which ring slot
// is which history level is read from the device step counter, so the same
// launch sequence (or its CUDA graph) serves every step.
// The mean mode runs on a second stream beside the mode kernel (they touch
// disjoint data); both read the counter before it advances.
void owt_handle::enqueue_step(cudaEvent_t after_modes) {
  step_begin();
  stage_modes();
  if (after_modes) ck(cudaEventRecord(after_modes, st), "after modes");
  step_finish();
}

// The mean mode on the second stream, beside the mode kernel.
void owt_handle::step_begin() {
  ck(cudaEventRecord(ev_fork, st), "fork");
  ck(cudaStreamWaitEvent(st2, ev_fork, 0), "fork wait");
  stage_mean(true, st2);
  ck(cudaEventRecord(ev_join, st2), "join");
}

// After the mode kernel: join the mean mode, advance the counter, the Lamb
// vector and the nonlinear source.
void owt_handle::step_finish() {
  ck(cudaStreamWaitEvent(st, ev_join, 0), "join wait");
  launch_advance(d_step, st);
  const XformArgs xa = xform_args();
  int nx = 3;
  if (xa.mean_split) {
    // the mean-flow terms beside the FP32 z backward and x pass
    ck(cudaEventRecord(ev_fork2, st), "fork");
    ck(cudaStreamWaitEvent(st2, ev_fork2, 0), "fork wait");
    launch_lamb_part(xa, precision, 3, st2);
    ck(cudaEventRecord(ev_join2, st2), "join");
    launch_lamb_part(xa, precision, 0, st);
    launch_lamb_part(xa, precision, 1, st);
    ck(cudaStreamWaitEvent(st, ev_join2, 0), "join wait");
    launch_lamb_part(xa, precision, 2, st);
    nx = 4;
  } else {
    nx = launch_lamb(xa, precision, st);
  }
  launch_nl(nl_args(true), st);
  launches += 4 + nx;
}

void owt_handle::stage_modes() {
  if (sparse_v6 && !force_dense) {
    launch_modes_sixth(mode_args(), st);
    return;
  }
  launch_modes(mode_args(), bv.kl, bv.ku, bg.kl, bg.ku, modes_sparse(),
               forced_variant >= 0 ? forced_variant : modes_variant, st);
}

ModeArgs owt_handle::mode_args() const {
  ModeArgs a{};
  a.NY = NY; a.NZ = NZ; a.NXH = NXH; a.NZH = NZH; a.M = M; a.U = Uq;
  a.u0 = 0; a.u1 = Uq;
  a.inv_dt = 1.0 / p.dt; a.nu = p.nu;
  a.kx = kx; a.kz = kz;
  a.v_ring = v_ring; a.g_ring = g_ring; a.hv_ring = hv_ring; a.hg_ring = hg_ring; a.q_ring = q_ring;
  a.u_out = u; a.w_out = w; a.ox_out = ox; a.oz_out = oz;
  a.ab_v = bv.ab; a.piv_v = bv.piv; a.n_v = bv.n;
  a.ab_g = bg.ab; a.piv_g = bg.piv; a.n_g = bg.n;
  a.rhs_node_v = rhs_node_v; a.rb_col = rb_col; a.rb_val = rb_val; a.inv_cg = inv_cg;
  a.rs_v = bv.rscale; a.rs_gi = rs_gi;
  a.sg = sg; a.dg = dg; a.yv = yv; a.yg = yg; a.sv = sv;
  a.rbv_col = rbv_col; a.rbv_val = rbv_val;
  a.c11h = c11h; a.c21h = c21h; a.c22h = c22h; a.nc21h = nc21h; a.nc22h = nc22h;
  a.step = d_step;
  a.vw = vw_on ? vw : nullptr;
  return a;
}

void owt_handle::stage_mean(bool pre_advance, cudaStream_t s) {
  launch_mean(mean_args(pre_advance), mean_smem, s ? s : st);
}

MeanArgs owt_handle::mean_args(bool pre_advance) const {
  MeanArgs ma{};
  ma.pre_advance = pre_advance ? 1 : 0;
  ma.NY = NY; ma.M = M; ma.U = Uq; ma.n_g = bg.n;
  ma.inv_dt = 1.0 / p.dt; ma.nu = p.nu; ma.Ly = Ly; ma.inv_cg0 = inv_cg0;
  ma.c11 = c11; ma.c21 = c21; ma.c22 = c22;
  ma.ab_g = bg.ab; ma.piv_g = bg.piv; ma.rb_col = rb_col; ma.rb_val = rb_val;
  ma.rs_g = bg.rscale; ma.inv_h = 1.0 / grid.ds; ma.inv_h2 = 1.0 / (grid.ds * grid.ds);
  ma.U_ring = U_ring; ma.W_ring = W_ring; ma.lx_ring = lxm_ring; ma.lz_ring = lzm_ring;
  ma.fx_ring = fx_ring; ma.fz_ring = fz_ring;
  ma.u_field = u; ma.w_field = w; ma.ox_field = ox; ma.oz_field = oz;
  ma.scratch = mean_scratch; ma.dy1 = mean_dy1; ma.step = d_step; ma.err = d_err;
  return ma;
}

void owt_handle::run_steps(int64_t n) {
  ensure_tuned();
  recompute_dirty_q();
  if (use_graph) {
    if (!gexec) {
      ck(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
      const int64_t before = launches;
      enqueue_step();
      per_step_launches = launches - before;
      launches = before;
      cudaError_t e = cudaStreamEndCapture(st, &graph);
      ck(e, "end capture");
      // node priorities as the streams had them at capture
      ck(cudaGraphInstantiate(&gexec, graph, cudaGraphInstantiateFlagUseNodePriority), "graph instantiate");
    }
    for (int64_t s = 0; s < n; ++s) {
      ck(cudaGraphLaunch(gexec, st), "graph launch");
      launches += per_step_launches;
      ++steps;
    }
  } else {
    for (int64_t s = 0; s < n; ++s) {
      enqueue_step();
      ++steps;
    }
  }
  check_launch("time step");
}

void owt_handle::ensure_tuned() {
  if (tuned) return;
  tuned = true;
  if (!initialized) {
    autotune_modes();
    return;
  }
  recompute_dirty_q();
  double2 *snap = nullptr;
  ck(cudaMalloc(&snap, 13 * fs * sizeof(double2)), "tuning snapshot");
  try {
    double2 *o = snap;
    for (double2 *ring : {v_ring, g_ring, q_ring}) { d2d(o, ring, 3 * fs * sizeof(double2)); o += 3 * fs; }
    for (double2 *f : {u, w, ox, oz}) { d2d(o, f, fs * sizeof(double2)); o += fs; }
    autotune_modes();
    o = snap;
    for (double2 *ring : {v_ring, g_ring, q_ring}) { d2d(ring, o, 3 * fs * sizeof(double2)); o += 3 * fs; }
    for (double2 *f : {u, w, ox, oz}) { d2d(f, o, fs * sizeof(double2)); o += fs; }
    ck(cudaStreamSynchronize(st), "tuning restore");
  } catch (...) {
    cudaStreamSynchronize(st);
    cudaFree(snap);
    throw;
  }
  cudaFree(snap);
}

void owt_handle::autotune_modes() {
  modes_variant = 0;
  tuning.clear();
  if (sparse_v6) { tuning = "sixth-order masked solve (one variant)"; return; }
  if (!sparse_v) { tuning = "full-band solve (no variants)"; return; }
  cudaEvent_t e0, e1;
  ck(cudaEventCreate(&e0), "event");
  ck(cudaEventCreate(&e1), "event");
  float best = 1e30f;
  for (int v = 0; v < modes_variant_count(); ++v) {
    forced_variant = v;
    stage_modes();  // warm-up
    ck(cudaEventRecord(e0, st), "event");
    for (int r = 0; r < 2; ++r) stage_modes();
    ck(cudaEventRecord(e1, st), "event");
    ck(cudaEventSynchronize(e1), "event");
    float ms = 0.f;
    ck(cudaEventElapsedTime(&ms, e0, e1), "event");
    ms *= 0.5f;
    launches += 3;
    char buf[96];
    std::snprintf(buf, sizeof(buf), "%s%s=%.3fms", tuning.empty() ? "" : " ", modes_variant_name(v), ms);
    tuning += buf;
    if (ms < best) { best = ms; modes_variant = v; }
  }
  forced_variant = -1;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  check_launch("autotune");
  tuning += std::string(" -> ") + modes_variant_name(modes_variant);
}

// DY2 v for history levels whose v was replaced from the host (one launch).
void owt_handle::recompute_dirty_q(cudaStream_t on) {
  DY2Args a{};
  a.NY = NY; a.M = M;
  a.m0 = 0; a.mcount = M;
  a.ab1 = b1.ab; a.piv1 = b1.piv; a.ab2 = b2.ab; a.piv2 = b2.piv;
  a.b1_col = b1_col; a.b1_val = b1_val; a.b2_col = b2_col; a.b2_val = b2_val;
  a.c21 = c21; a.c22 = c22;
  double2 *scr[3] = {tmpA, tmpB, tmpC};
  for (int sl = 0; sl < 3; ++sl) {
    if (!q_dirty[sl]) continue;
    a.in[a.nf] = v_ring + (size_t)sl * fs;
    a.out[a.nf] = q_ring + (size_t)sl * fs;
    a.scr[a.nf] = scr[a.nf];
    ++a.nf;
    q_dirty[sl] = false;
  }
  if (!a.nf) return;
  launch_dy2(a, on ? on : st);
  ++launches;
}

void owt_handle::copy_ring(double2 *ring, size_t n, int from, int to) {
  ck(cudaMemcpyAsync(ring + (size_t)to * n, ring + (size_t)from * n, n * sizeof(double2), cudaMemcpyDeviceToDevice,
                     st), "ring copy");
}

// column of mode 0 of a device-layout field -> contiguous NY vector
void owt_handle::mode0_column(double2 *dst, const double2 *field) {
  ck(cudaMemcpy2DAsync(dst, sizeof(double2), field, (size_t)M * sizeof(double2), sizeof(double2), NY,
                       cudaMemcpyDeviceToDevice, st), "mode-0 column");
}

void owt_handle::get_vor_from_vel() {
  dapply(1, u, tmpA);
  dapply(1, w, tmpB);
  VorArgs va{};
  va.NY = NY; va.NXH = NXH; va.M = M; va.kx = kx; va.kz = kz; va.c11 = c11;
  va.u = u; va.v = ring_level(v_ring, 0); va.w = w; va.d1u = tmpA; va.d1w = tmpB;
  va.ox = ox; va.oy = ring_level(g_ring, 0); va.oz = oz;
  launch_vor(va, st);
  ++launches;
}

void owt_handle::lamb_vec(bool explicit_shift) {
  launches += launch_lamb(xform_args(), precision, st);
  if (explicit_shift) {
    launch_lamb_mean_shift(lxm_ring, lzm_ring, lx, lz, NY, M, d_step, st);
    ++launches;
  }
}

void owt_handle::nonlinear_source(bool record_mean) {
  launch_nl(nl_args(record_mean), st);
  ++launches;
}

void owt_handle::friction(int shift) {
  dapply(1, u, tmpA);
  dapply(1, w, tmpB);
  launch_friction(tmpA, tmpB, c11, NY, M, p.nu, Ly, fx_ring, fz_ring, d_step, shift, d_err, st);
  ++launches;
}

void owt_handle::init_prologue() {
  steps = 0;
  drop_graph();
  ck(cudaMemsetAsync(d_step, 0, sizeof(long long), st), "memset");
  ck(cudaMemsetAsync(d_err, 0, sizeof(int), st), "memset");
}

void owt_handle::init_fields(const double *hu, const double *hv, const double *hw) {
  init_prologue();
  to_device(hu, u);
  to_device(hv, ring_level(v_ring, 0));
  to_device(hw, w);
  init_from_velocity();
}

// The seeded laminar + random divergence-free state, generated on the
// device (seeded_ic.cu); the Chebyshev coefficients live in the mean-flow
// buffer and omega_y in tmpC until the velocity is complete.
void owt_handle::init_seeded(uint64_t seed, double rms) {
  init_prologue();
  SeedArgs a{};
  a.NY = NY; a.NZ = NZ; a.NXH = NXH; a.NZH = NZH; a.M = M; a.degree = 5;
  a.seed = seed;
  a.kmin = std::min(p.dkx, p.dkz);
  a.kx = kx; a.kz = kz; a.y = ygrid; a.c11 = c11; a.wy = wy;
  a.coef = reinterpret_cast<double2 *>(zbuf);  // >= 3 NY M values, free until the transforms
  double2 *v0 = ring_level(v_ring, 0);
  launches += launch_ic_fields(a, v0, tmpC, st);
  dapply(1, v0, tmpA);
  launches += launch_ic_velocity(a, tmpA, tmpC, u, v0, w, ic_partial, rms, st);
  check_launch("seeded initial condition");
  init_from_velocity();
}

void owt_handle::init_from_velocity() {
  get_vor_from_vel();  // also leaves D1 u, D1 w in tmpA, tmpB
  launch_friction(tmpA, tmpB, c11, NY, M, p.nu, Ly, fx_ring, fz_ring, d_step, 0, d_err, st);
  ++launches;
  lamb_vec(false);
  nonlinear_source(true);
  const int s0 = slot(0);
  for (double2 *ring : {v_ring, g_ring, hv_ring, hg_ring})
    for (int l = 1; l < 3; ++l) copy_ring(ring, fs, s0, slot(l));
  for (double2 *ring : {lxm_ring, lzm_ring})
    for (int l = 1; l < 3; ++l) copy_ring(ring, NY, s0, slot(l));
  mode0_column(U_ring + (size_t)s0 * NY, u);
  mode0_column(W_ring + (size_t)s0 * NY, w);
  for (double2 *ring : {U_ring, W_ring})
    for (int l = 1; l < 3; ++l) copy_ring(ring, NY, s0, slot(l));
  for (double *fr : {fx_ring, fz_ring})
    for (int l = 1; l < 3; ++l)
      ck(cudaMemcpyAsync(fr + slot(l), fr + s0, sizeof(double), cudaMemcpyDeviceToDevice, st), "fric copy");
  q_dirty[0] = q_dirty[1] = q_dirty[2] = true;
  recompute_dirty_q();
  check_launch("init_fields");
  initialized = true;
}

void owt_handle::to_device(const double *host, double2 *dst) {
  ck(cudaMemcpyAsync(stage, host, fs * sizeof(double2), cudaMemcpyHostToDevice, st), "H2D");
  launch_transpose(stage, dst, M, NY, st);  // [M][NY] -> [NY][M]
  ++launches;
  check_launch("layout transpose");
}

void owt_handle::to_host(const double2 *src, double *host) {
  launch_transpose(src, stage, NY, M, st);  // [NY][M] -> [M][NY]
  ++launches;
  check_launch("layout transpose");
  ck(cudaMemcpyAsync(host, stage, fs * sizeof(double2), cudaMemcpyDeviceToHost, st), "D2H");
  ck(cudaStreamSynchronize(st), "D2H");
}

double2 *owt_handle::field_ptr(int f, bool for_write) {
  switch (f) {
    case OWT_VELX: return u;
    case OWT_VELZ: return w;
    case OWT_VORX: return ox;
    case OWT_VORZ: return oz;
    case OWT_LMBX: return lx;
    case OWT_LMBY: return ly;
    case OWT_LMBZ: return lz;
    case OWT_VELY: case OWT_VELY_0: case OWT_VELY_1: case OWT_VELY_2: {
      const int l = f == OWT_VELY ? 0 : f - OWT_VELY_0;
      if (for_write) q_dirty[slot(l)] = true;
      return ring_level(v_ring, l);
    }
    case OWT_VORY: return ring_level(g_ring, 0);
    case OWT_VORY_0: case OWT_VORY_1: case OWT_VORY_2: return ring_level(g_ring, f - OWT_VORY_0);
    case OWT_HV: return ring_level(hv_ring, 0);
    case OWT_HV_0: case OWT_HV_1: case OWT_HV_2: return ring_level(hv_ring, f - OWT_HV_0);
    case OWT_HG: return ring_level(hg_ring, 0);
    case OWT_HG_0: case OWT_HG_1: case OWT_HG_2: return ring_level(hg_ring, f - OWT_HG_0);
    default: throw OwtError(OWT_ERR_INVALID, "unknown field id " + std::to_string(f));
  }
}

double2 *owt_handle::mean_ptr(int which) {
  if (which < 0 || which >= OWT_NUM_MEANS) throw OwtError(OWT_ERR_INVALID, "unknown mean id");
  double2 *rings[4] = {lxm_ring, lzm_ring, U_ring, W_ring};
  return rings[which / 3] + (size_t)slot(which % 3) * NY;
}

// FP64 tables whatever the handle's precision; no mean split; field 0 of the
// transform buffers; the state fields are not touched.
static XformArgs phys_args(const owt_handle &h) {
  XformArgs a = h.xform_args();
  a.ring_mask = 0;
  a.mean_split = 0;
  a.twx = h.twx[0];
  a.twz = h.twz[0];
  return a;
}

void owt_handle::fourier2physical(const double *spec, double *phys) {
  const size_t np = (size_t)NZ2 * NX2 * NY;
  std::vector<void *> tmp;
  try {
    double *dphys = dalloc<double>(2 * np, tmp);
    to_device(spec, tmpC);
    XformArgs a = phys_args(*this);
    a.in[0] = tmpC;
    launch_fourier2physical(a, dphys, st);
    launch_transpose_real(dphys, dphys + np, NY, NZ2 * NX2, st);  // [y][z][x] -> [z][x][y]
    launches += 3;
    check_launch("fourier2physical");
    ck(cudaMemcpyAsync(phys, dphys + np, np * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
    ck(cudaStreamSynchronize(st), "fourier2physical");
  } catch (...) {
    cudaStreamSynchronize(st);
    for (void *q : tmp) cudaFree(q);
    throw;
  }
  for (void *q : tmp) cudaFree(q);
}

void owt_handle::physical2fourier(const double *phys, double *spec) {
  const size_t np = (size_t)NZ2 * NX2 * NY;
  std::vector<void *> tmp;
  try {
    double *dphys = dalloc<double>(2 * np, tmp);
    ck(cudaMemcpyAsync(dphys + np, phys, np * sizeof(double), cudaMemcpyHostToDevice, st), "H2D");
    launch_transpose_real(dphys + np, dphys, NZ2 * NX2, NY, st);  // [z][x][y] -> [y][z][x]
    XformArgs a = phys_args(*this);
    a.out[0] = tmpC;
    launch_physical2fourier(a, dphys, st);
    launches += 3;
    check_launch("physical2fourier");
    to_host(tmpC, spec);
  } catch (...) {
    cudaStreamSynchronize(st);
    for (void *q : tmp) cudaFree(q);
    throw;
  }
  for (void *q : tmp) cudaFree(q);
}

// ---- one step on a host-held state ---------------------------------------------
void owt_handle::host_step_prepare() {
  if (hs.ready) return;
  int lo = 0, hi = 0;
  ck(cudaDeviceGetStreamPriorityRange(&lo, &hi), "stream priorities");
  ck(cudaStreamCreateWithFlags(&hs.up, cudaStreamNonBlocking), "stream");
  ck(cudaStreamCreateWithFlags(&hs.aux, cudaStreamNonBlocking), "stream");
  ck(cudaStreamCreateWithPriority(&hs.tx, cudaStreamNonBlocking, hi), "stream");
  ck(cudaStreamCreateWithPriority(&hs.down, cudaStreamNonBlocking, hi), "stream");
  for (int i = 0; i < 12; ++i) hs.stage[i] = dalloc<double2>(fs, owned);
  for (int b = 0; b < 2; ++b) hs.dstage[b] = dalloc<double2>(fs, owned);
  ck(cudaHostAlloc(reinterpret_cast<void **>(&hs.fric_pin), 12 * sizeof(double), cudaHostAllocDefault), "pinned");
  for (int j = 0; j < HostStep::kChunks; ++j)
    for (cudaEvent_t *e : {&hs.landed[j], &hs.v_done[j], &hs.q_done[j], &hs.tx_done[j]})
      ck(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "event");
  for (cudaEvent_t *e : {&hs.up_done, &hs.after_modes, &hs.down_done})
    ck(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "event");
  hs.ready = true;
}

// The device address of a host array the kernels can read directly (pinned
// or registered memory, 16-byte aligned), or null.
static const double2 *device_view(const double *p) {
  if (reinterpret_cast<uintptr_t>(p) % 16 != 0) return nullptr;
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
  return static_cast<const double2 *>(at.devicePointer);
}

// Uploads, by chunks of Fourier modes: the modes with |kz| in a range are
// the host rows kz of that range and of its negative partners, contiguous in
// the reference layout.  Chunk by chunk, the twelve fields' rows are copied
// back to back into staging buffers of their own (one per field), then
// transposed into their ring slots on a high-priority stream (whose blocks
// the scheduler places ahead of those of long kernels), the DY2 v history of
// the chunk's modes is re-derived on a third stream, and the mode kernel
// runs on the chunk's unique modes while the next chunks arrive.  One chunk
// (everything) when the mode-kernel variant in use is not the quad mapping,
// whose unique-mode ranges the chunks are.  History fields in pinned memory
// are uploaded by SM loads (launch_host_load), others by the copy engines:
// at 384x257x384 copy-engine uploads of pinned memory ran at a tenth of the
// host link's rate in every fourth or fifth call (about 230 instead of 80 ms
// a call), SM loads at the full rate in every call.  Downloads: the new v and omega_y
// are final after the mode kernel, so their transposes (high priority) and
// copies run beside the transforms of the same step.
void owt_handle::step_host(const double *const *hist, const double *means, const double *fric, double *v_out,
                           double *g_out, double *fric_out) {
  host_step_prepare();
  ensure_tuned();
  ck(cudaStreamSynchronize(st), "host step");
  const int variant = forced_variant >= 0 ? forced_variant : modes_variant;
  const bool quad = modes_sparse() && !sparse_v6 && modes_variant_is_quad(variant);
  const int want = host_chunks > 0 ? host_chunks : HostStep::kDefaultChunks;
  const int nchunk = quad ? std::min(std::min(want, HostStep::kChunks), NZH + 1) : 1;
  // means first (the mean-mode kernel starts with the step)
  for (int w = 0; w < OWT_NUM_MEANS; ++w)
    ck(cudaMemcpyAsync(mean_ptr(w), means + 2 * (size_t)w * NY, NY * sizeof(double2), cudaMemcpyHostToDevice, hs.up),
       "H2D");
  ck(cudaEventRecord(hs.up_done, hs.up), "means done");
  {
    double *fx = hs.fric_pin, *fz = hs.fric_pin + 3;
    for (int l = 0; l < 3; ++l) {
      fx[slot(l)] = fric[l];
      fz[slot(l)] = fric[3 + l];
    }
    ck(cudaMemcpyAsync(fx_ring, fx, 3 * sizeof(double), cudaMemcpyHostToDevice, st), "H2D");
    ck(cudaMemcpyAsync(fz_ring, fz, 3 * sizeof(double), cudaMemcpyHostToDevice, st), "H2D");
  }
  double2 *rings[4] = {v_ring, g_ring, hv_ring, hg_ring};
  const size_t row = (size_t)NXH * NY;  // complex values of one kz row, reference layout
  const double2 *hdev[12];
  for (int i = 0; i < 12; ++i) hdev[i] = device_view(hist[i]);
  // row blocks [k0, k1) of chunk j: |kz| in [a, b) for kz <= NZH, and the
  // negative partners NZ - |kz| for 1 <= |kz| < NZH
  auto blocks = [&](int j, int (&k0)[2], int (&k1)[2]) {
    if (nchunk == 1) {
      k0[0] = 0; k1[0] = NZ; k0[1] = k1[1] = 0;
      return;
    }
    const int a = (NZH + 1) * j / nchunk, b = (NZH + 1) * (j + 1) / nchunk;
    k0[0] = a; k1[0] = b;
    const int pa = std::max(a, 1), pb = std::min(b, NZH);
    k0[1] = pb > pa ? NZ - pb + 1 : 0;
    k1[1] = pb > pa ? NZ - pa + 1 : 0;
  };
  for (int j = 0; j < nchunk; ++j) {
    int k0[2], k1[2];
    blocks(j, k0, k1);
    for (int i = 0; i < 12; ++i)
      for (int q = 0; q < 2; ++q)
        if (k1[q] > k0[q]) {
          const size_t off = k0[q] * row, bytes = (k1[q] - k0[q]) * row * sizeof(double2);
          if (hdev[i]) {
            launch_host_load(hdev[i] + off, hs.stage[i] + off, bytes, hs.up);
            ++launches;
          } else {
            ck(cudaMemcpyAsync(hs.stage[i] + off, hist[i] + 2 * off, bytes, cudaMemcpyHostToDevice, hs.up), "H2D");
          }
        }
    ck(cudaEventRecord(hs.landed[j], hs.up), "landed");
  }
  ck(cudaStreamWaitEvent(st, hs.up_done, 0), "means wait");
  ++state_version;
  initialized = true;
  const int hn = (head() + 2) % 3;  // the new v, omega_y land in the slot that becomes level 0
  step_begin();
  for (int j = 0; j < nchunk; ++j) {
    int k0[2], k1[2];
    blocks(j, k0, k1);
    ck(cudaStreamWaitEvent(hs.tx, hs.landed[j], 0), "landed wait");
    for (int i = 0; i < 12; ++i) {
      for (int q = 0; q < 2; ++q)
        if (k1[q] > k0[q]) {
          const int m0 = k0[q] * NXH, nm = (k1[q] - k0[q]) * NXH;
          launch_transpose_ld(hs.stage[i] + (size_t)m0 * NY, ring_level(rings[i / 3], i % 3) + m0, nm, NY, M, hs.tx);
          ++launches;
        }
      if (i == 2) {  // the chunk's v levels are in place: their DY2 v on the side
        ck(cudaEventRecord(hs.v_done[j], hs.tx), "v done");
        ck(cudaStreamWaitEvent(hs.aux, hs.v_done[j], 0), "v wait");
        for (int q = 0; q < 2; ++q)
          if (k1[q] > k0[q]) {
            DY2Args a{};
            a.NY = NY; a.M = M;
            a.m0 = k0[q] * NXH; a.mcount = (k1[q] - k0[q]) * NXH;
            a.ab1 = b1.ab; a.piv1 = b1.piv; a.ab2 = b2.ab; a.piv2 = b2.piv;
            a.b1_col = b1_col; a.b1_val = b1_val; a.b2_col = b2_col; a.b2_val = b2_val;
            a.c21 = c21; a.c22 = c22;
            double2 *scr[3] = {tmpA, tmpB, tmpC};
            for (int l = 0; l < 3; ++l) {
              a.in[l] = ring_level(v_ring, l);
              a.out[l] = ring_level(q_ring, l);
              a.scr[l] = scr[l];
            }
            a.nf = 3;
            launch_dy2(a, hs.aux);
            ++launches;
          }
        ck(cudaEventRecord(hs.q_done[j], hs.aux), "q done");
      }
    }
    ck(cudaEventRecord(hs.tx_done[j], hs.tx), "transposes done");
    ck(cudaStreamWaitEvent(st, hs.tx_done[j], 0), "transposes wait");
    ck(cudaStreamWaitEvent(st, hs.q_done[j], 0), "DY2 v wait");
    if (nchunk == 1) {
      stage_modes();
    } else {
      ModeArgs a = mode_args();
      a.u0 = ((NZH + 1) * j / nchunk) * NXH;
      a.u1 = ((NZH + 1) * (j + 1) / nchunk) * NXH;
      launch_modes(a, bv.kl, bv.ku, bg.kl, bg.ku, true, variant, st);
    }
    ++launches;
  }
  q_dirty[0] = q_dirty[1] = q_dirty[2] = false;
  ck(cudaEventRecord(hs.after_modes, st), "after modes");
  step_finish();
  ++steps;
  ck(cudaStreamWaitEvent(hs.down, hs.after_modes, 0), "modes wait");
  double *outs[2] = {v_out, g_out};
  double2 *src[2] = {v_ring + (size_t)hn * fs, g_ring + (size_t)hn * fs};
  for (int b = 0; b < 2; ++b) {
    launch_transpose(src[b], hs.dstage[b], NY, M, hs.down);  // [NY][M] -> [M][NY]
    ++launches;
    ck(cudaMemcpyAsync(outs[b], hs.dstage[b], fs * sizeof(double2), cudaMemcpyDeviceToHost, hs.down), "D2H");
  }
  ck(cudaEventRecord(hs.down_done, hs.down), "downloads done");
  ck(cudaStreamWaitEvent(st, hs.down_done, 0), "downloads wait");
  check_launch("host step");
  double *fx = hs.fric_pin + 6, *fz = hs.fric_pin + 9;
  ck(cudaMemcpyAsync(fx, fx_ring, 3 * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
  ck(cudaMemcpyAsync(fz, fz_ring, 3 * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
  sync_and_check();
  for (int l = 0; l < 3; ++l) {
    fric_out[l] = fx[slot(l)];
    fric_out[3 + l] = fz[slot(l)];
  }
}

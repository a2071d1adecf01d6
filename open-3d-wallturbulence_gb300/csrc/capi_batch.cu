// Batches of channels (owt_batch_*): every kernel of the step launched once
// over all channels of a group, the mode kernel as one persistent launch,
// the whole batch step as one CUDA graph.
#include <tuple>

#include "handle.h"

using namespace owt;

// ---------------------------------------------------------------------------
// Batches.  A batch step is one CUDA graph of batched launches: each kernel of
// the time step runs once over every channel of a group (channels that share
// the kernel's template and block shape; at most kBatchChannels per launch),
// in the order of the single-channel step.  The mode kernel (every per-mode
// banded solve of every channel) is one persistent launch working through the
// channels' work items, longest systems first; its variant is chosen at
// creation by timing every variant on the batch itself.
// ---------------------------------------------------------------------------
template <class A>
using TablePtr = std::unique_ptr<BatchTable<A>>;

// Tables over the channels `order` (indices into args) in that order, at most
// kBatchChannels channels each; blocks[i] is channel i's block count.
template <class A>
static std::vector<TablePtr<A>> make_tables(const std::vector<A> &args, const std::vector<int> &blocks,
                                            const std::vector<int> &order) {
  std::vector<TablePtr<A>> out;
  for (size_t q = 0; q < order.size(); ++q) {
    if (q % kBatchChannels == 0) out.emplace_back(new BatchTable<A>());
    BatchTable<A> &t = *out.back();
    const int i = order[q];
    t.a[t.n] = args[i];
    t.start[t.n + 1] = t.start[t.n] + blocks[i];
    ++t.n;
  }
  return out;
}

struct owt_batch {
  std::vector<owt_handle *> hs;
  cudaStream_t st = nullptr, st2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;    // the mean mode beside the mode kernel
  cudaEvent_t ev_fork2 = nullptr, ev_join2 = nullptr;  // the mean-flow terms beside the transforms
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int *work = nullptr;        // counter pairs of the persistent mode launches
  int64_t step_launches = 0;  // kernels in one batch step
  int64_t launches = 0;       // kernels launched by batch steps
  int modes_variant = -1;     // variant of the channels with the sparse solve
  std::string tuning;

  struct ModeLaunch {
    TablePtr<ModeArgs> t;
    int variant, grid;
  };
  struct LambLaunch {
    TablePtr<XformArgs> t;
    int precision, part;
  };
  std::vector<ModeLaunch> modes;
  std::vector<TablePtr<MeanArgs>> mean[2];  // by staged (shared-memory) solve
  size_t mean_bytes = 0;
  std::vector<StepCounters> counters;
  std::vector<LambLaunch> lamb;  // in launch order
  std::vector<TablePtr<NLArgs>> nl;

  ~owt_batch() {
    if (st) cudaStreamSynchronize(st);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (work) cudaFree(work);
    for (cudaEvent_t e : {ev_fork, ev_join, ev_fork2, ev_join2})
      if (e) cudaEventDestroy(e);
    if (st2) cudaStreamDestroy(st2);
    if (st) cudaStreamDestroy(st);
  }

  // channels by decreasing wall-normal size (the longest solves first), stable
  std::vector<int> by_size(bool sparse) const {
    std::vector<int> o;
    for (size_t i = 0; i < hs.size(); ++i)
      if (hs[i]->modes_sparse() == sparse) o.push_back((int)i);
    std::stable_sort(o.begin(), o.end(), [&](int a, int b) { return hs[a]->NY > hs[b]->NY; });
    return o;
  }
  // mode-kernel launches with `variant` for the sparse channels (the others
  // take the full-band solve); only the sparse group when sparse_only
  void build_modes(int variant, bool sparse_only) {
    modes.clear();
    std::vector<ModeArgs> args;
    for (owt_handle *h : hs) args.push_back(h->mode_args());
    for (int sparse = 1; sparse >= (sparse_only ? 1 : 0); --sparse) {
      const int v = sparse ? variant : -1;
      const ModeBatchShape sh = modes_batch_shape(v);
      std::vector<int> blocks(hs.size(), 0);
      for (size_t i = 0; i < hs.size(); ++i) {
        const long long threads = sh.quad ? 4LL * hs[i]->Uq : 2LL * hs[i]->M;
        blocks[i] = (int)((threads + sh.block - 1) / sh.block);
      }
      for (auto &t : make_tables(args, blocks, by_size(sparse == 1))) {
        const int total = t->start[t->n];
        modes.push_back({std::move(t), v, std::min(sh.grid, total)});
      }
    }
  }
  void launch_modes_all(cudaStream_t s) {
    for (size_t q = 0; q < modes.size(); ++q) {
      launch_modes_batch(*modes[q].t, modes[q].variant, work + 2 * q, modes[q].grid, s);
      ++step_launches;
    }
  }

  void build_rest() {
    const int n = (int)hs.size();
    std::vector<int> all(n);
    for (int i = 0; i < n; ++i) all[i] = i;
    // mean mode, one block per channel
    std::vector<MeanArgs> margs;
    std::vector<int> ones(n, 1), staged, plain;
    for (int i = 0; i < n; ++i) {
      margs.push_back(hs[i]->mean_args(true));
      (hs[i]->mean_smem ? staged : plain).push_back(i);
      if (hs[i]->mean_smem) mean_bytes = std::max(mean_bytes, mean_smem_bytes(hs[i]->NY, hs[i]->bg.n));
    }
    if (!staged.empty()) ck(mean_batch_prepare(mean_bytes), "mean kernel attributes");
    mean[0] = make_tables(margs, ones, plain);
    mean[1] = make_tables(margs, ones, staged);
    // step counters
    for (int i = 0; i < n; ++i) {
      if (i % kBatchChannels == 0) counters.push_back(StepCounters{});
      StepCounters &c = counters.back();
      c.p[c.n++] = hs[i]->d_step;
    }
    // transforms: grouped by precision and the line length of the kernel
    std::vector<XformArgs> xargs;
    for (owt_handle *h : hs) xargs.push_back(h->xform_args());
    for (int part = 0; part < 4; ++part) {
      std::map<std::tuple<int, int, int>, std::vector<int>> groups;  // (precision, line length, Stockham kernels)
      std::vector<int> blocks(n, 0);
      for (int i = 0; i < n; ++i) {
        const owt_handle *h = hs[i];
        if (part == 3 && !xargs[i].mean_split) continue;
        const XformDims &d = xargs[i].d;
        const int prec = h->precision == OWT_PREC_MIXED ? 1 : 0;
        if (part == 0) ck(lamb_batch_prepare(d, prec), "transform kernel attributes");
        blocks[i] = lamb_batch_blocks(d, prec, part, xargs[i].stockham != 0);
        const int len = part == 1 ? d.NX2 : part == 3 ? 0 : d.NZ2;
        groups[std::make_tuple(prec, len, xargs[i].stockham)].push_back(i);
      }
      for (auto &g : groups)
        for (auto &t : make_tables(xargs, blocks, g.second)) lamb.push_back({std::move(t), std::get<0>(g.first), part});
    }
    // nonlinear source
    std::vector<NLArgs> nargs;
    std::vector<int> nblocks;
    for (owt_handle *h : hs) {
      nargs.push_back(h->nl_args(true));
      nblocks.push_back(nl_batch_blocks(nargs.back()));
    }
    nl = make_tables(nargs, nblocks, all);
  }

  // One batch step, the single-channel step's order: the mean mode on a
  // second stream beside the mode kernel, then the counters, the transforms
  // and the nonlinear source.
  void enqueue() {
    step_launches = 0;
    ck(cudaEventRecord(ev_fork, st), "fork");
    ck(cudaStreamWaitEvent(st2, ev_fork, 0), "fork wait");
    for (int staged = 0; staged < 2; ++staged)
      for (auto &t : mean[staged]) {
        launch_mean_batch(*t, staged == 1, mean_bytes, st2);
        ++step_launches;
      }
    ck(cudaEventRecord(ev_join, st2), "join");
    launch_modes_all(st);
    ck(cudaStreamWaitEvent(st, ev_join, 0), "join wait");
    for (const StepCounters &c : counters) {
      launch_advance_batch(c, st);
      ++step_launches;
    }
    // the mean-flow terms of the mixed-precision channels beside the z
    // backward and x pass; the z forward adds them
    bool split = false;
    for (auto &l : lamb) split = split || l.part == 3;
    if (split) {
      ck(cudaEventRecord(ev_fork2, st), "fork");
      ck(cudaStreamWaitEvent(st2, ev_fork2, 0), "fork wait");
    }
    for (int part : {3, 0, 1, 2}) {
      if (part == 2 && split) ck(cudaStreamWaitEvent(st, ev_join2, 0), "join wait");
      for (auto &l : lamb)
        if (l.part == part) {
          launch_lamb_batch(*l.t, l.precision, l.part, part == 3 ? st2 : st);
          ++step_launches;
        }
      if (part == 3 && split) ck(cudaEventRecord(ev_join2, st2), "join");
    }
    for (auto &t : nl) {
      launch_nl_batch(*t, st);
      ++step_launches;
    }
  }

  // Time every variant of the batched mode kernel on the channels' current
  // state, then put back what the trials overwrote (the v, omega_y and DY2 v
  // rings and the horizontal fields) and keep the fastest.
  void autotune() {
    if (by_size(true).empty()) {
      tuning = "full-band solve (no variants)";
      return;
    }
    std::vector<double2 *> snap(hs.size(), nullptr);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    step_launches = 0;
    auto cleanup = [&] {
      for (double2 *p : snap)
        if (p) cudaFree(p);
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
    };
    try {
      for (size_t i = 0; i < hs.size(); ++i) {
        owt_handle *h = hs[i];
        const size_t fs = h->fs;
        ck(cudaMalloc(&snap[i], 13 * fs * sizeof(double2)), "tuning snapshot");
        double2 *o = snap[i];
        for (double2 *ring : {h->v_ring, h->g_ring, h->q_ring}) {
          ck(cudaMemcpyAsync(o, ring, 3 * fs * sizeof(double2), cudaMemcpyDeviceToDevice, st), "snapshot");
          o += 3 * fs;
        }
        for (double2 *f : {h->u, h->w, h->ox, h->oz}) {
          ck(cudaMemcpyAsync(o, f, fs * sizeof(double2), cudaMemcpyDeviceToDevice, st), "snapshot");
          o += fs;
        }
      }
      ck(cudaEventCreate(&e0), "event");
      ck(cudaEventCreate(&e1), "event");
      float best = 1e30f;
      for (int v = 0; v < modes_batch_variant_count(); ++v) {
        build_modes(v, true);
        launch_modes_all(st);  // warm-up
        ck(cudaEventRecord(e0, st), "event");
        for (int r = 0; r < 2; ++r) launch_modes_all(st);
        ck(cudaEventRecord(e1, st), "event");
        ck(cudaEventSynchronize(e1), "event");
        float ms = 0.f;
        ck(cudaEventElapsedTime(&ms, e0, e1), "event");
        ms *= 0.5f;
        char buf[96];
        std::snprintf(buf, sizeof(buf), "%s%s=%.3fms", tuning.empty() ? "" : " ", modes_variant_name(v), ms);
        tuning += buf;
        if (ms < best) { best = ms; modes_variant = v; }
      }
      launches += step_launches;
      step_launches = 0;
      for (size_t i = 0; i < hs.size(); ++i) {
        owt_handle *h = hs[i];
        const size_t fs = h->fs;
        const double2 *o = snap[i];
        for (double2 *ring : {h->v_ring, h->g_ring, h->q_ring}) {
          ck(cudaMemcpyAsync(ring, o, 3 * fs * sizeof(double2), cudaMemcpyDeviceToDevice, st), "restore");
          o += 3 * fs;
        }
        for (double2 *f : {h->u, h->w, h->ox, h->oz}) {
          ck(cudaMemcpyAsync(f, o, fs * sizeof(double2), cudaMemcpyDeviceToDevice, st), "restore");
          o += fs;
        }
      }
      ck(cudaStreamSynchronize(st), "restore");
    } catch (...) {
      cudaStreamSynchronize(st);
      cleanup();
      throw;
    }
    cleanup();
    tuning += std::string(" -> ") + modes_variant_name(modes_variant);
  }
};

extern "C" {

int owt_batch_create(owt_handle *const *handles, int count, owt_batch **out) {
  if (!handles || count < 1 || !out) {
    g_create_error = "owt_batch_create: need at least one handle";
    return OWT_ERR_INVALID;
  }
  *out = nullptr;
  owt_batch *b = new owt_batch();
  try {
    for (int q = 0; q < count; ++q) {
      owt_handle *h = handles[q];
      if (!h || !h->initialized) throw OwtError(OWT_ERR_STATE, "every handle must be initialised");
      if (h->p.device != handles[0]->p.device) throw OwtError(OWT_ERR_INVALID, "handles on different devices");
      for (int r = 0; r < q; ++r)
        if (handles[r] == h) throw OwtError(OWT_ERR_INVALID, "a handle appears twice in the batch");
      ck(cudaStreamSynchronize(h->st), "batch");
      h->recompute_dirty_q();
      ck(cudaStreamSynchronize(h->st), "batch");
      b->hs.push_back(h);
    }
    ck(cudaSetDevice(handles[0]->p.device), "cudaSetDevice");
    ck(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking), "stream");
    {
      int lo = 0, hi = 0;  // the mean modes' branch at the highest priority, as in a single channel's step
      ck(cudaDeviceGetStreamPriorityRange(&lo, &hi), "stream priorities");
      ck(cudaStreamCreateWithPriority(&b->st2, cudaStreamNonBlocking, hi), "stream");
    }
    ck(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming), "event");
    ck(cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming), "event");
    ck(cudaEventCreateWithFlags(&b->ev_fork2, cudaEventDisableTiming), "event");
    ck(cudaEventCreateWithFlags(&b->ev_join2, cudaEventDisableTiming), "event");
    const size_t n_mode_tables = (b->by_size(true).size() + kBatchChannels - 1) / kBatchChannels +
                                 (b->by_size(false).size() + kBatchChannels - 1) / kBatchChannels;
    ck(cudaMalloc(&b->work, 2 * n_mode_tables * sizeof(int)), "work counters");
    ck(cudaMemsetAsync(b->work, 0, 2 * n_mode_tables * sizeof(int), b->st), "memset");
    b->autotune();
    b->build_modes(b->modes_variant, false);
    b->build_rest();
    ck(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal), "begin capture");
    b->enqueue();
    ck(cudaStreamEndCapture(b->st, &b->graph), "end capture");
    ck(cudaGraphInstantiate(&b->exec, b->graph, cudaGraphInstantiateFlagUseNodePriority), "instantiate");
    ck(cudaStreamSynchronize(b->st), "batch setup");
  } catch (const std::exception &e) {
    g_create_error = e.what();
    cudaGetLastError();
    delete b;
    return OWT_ERR_CUDA;
  }
  *out = b;
  return OWT_OK;
}

int owt_batch_step(owt_batch *b, int64_t nsteps) {
  if (!b || nsteps < 0) return OWT_ERR_INVALID;
  for (int64_t s = 0; s < nsteps; ++s) {
    if (cudaGraphLaunch(b->exec, b->st) != cudaSuccess) {
      g_create_error = "batch graph launch failed";
      return OWT_ERR_CUDA;
    }
    b->launches += b->step_launches;
    for (owt_handle *h : b->hs) {
      ++h->steps;
      ++h->state_version;
    }
  }
  return OWT_OK;
}

int owt_batch_synchronize(owt_batch *b) {
  if (!b) return OWT_ERR_INVALID;
  if (cudaStreamSynchronize(b->st) != cudaSuccess) {
    g_create_error = "batch synchronize failed";
    return OWT_ERR_CUDA;
  }
  for (owt_handle *h : b->hs) {
    const int rc = owt_synchronize(h);
    if (rc != OWT_OK) {
      g_create_error = owt_last_error(h);
      return rc;
    }
  }
  return OWT_OK;
}

int owt_batch_get_stream(const owt_batch *b, void **stream) {
  if (!b || !stream) return OWT_ERR_INVALID;
  *stream = (void *)b->st;
  return OWT_OK;
}

int owt_batch_get_launch_count(const owt_batch *b, int64_t *count) {
  if (!b || !count) return OWT_ERR_INVALID;
  *count = b->launches;
  return OWT_OK;
}

int owt_batch_get_step_launches(const owt_batch *b, int64_t *count) {
  if (!b || !count) return OWT_ERR_INVALID;
  *count = b->step_launches;
  return OWT_OK;
}

const char *owt_batch_tuning_report(const owt_batch *b) { return b ? b->tuning.c_str() : ""; }

int owt_batch_destroy(owt_batch *b) {
  delete b;
  return OWT_OK;
}

}  // extern "C"

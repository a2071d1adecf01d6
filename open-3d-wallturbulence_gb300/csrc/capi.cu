// C ABI of the GPU time step (declared in include/owt_gpu.h).
//
// One handle = one channel on one GPU: parameters, device-resident state,
// per-mode band factorizations, scratch, and a CUDA stream.  A step is seven
// launches: mode kernel, counter advance, mean mode, three transform kernels,
// nonlinear source; it can be captured once as a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "adjoint_kernels.h"
#include "owt_gpu.h"
#include "setup_host.h"
#include "solve_kernels.h"

using namespace owt;

namespace {

thread_local std::string g_create_error;

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct OwtError : std::runtime_error {
  int code;
  OwtError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void ck(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

thread_local size_t *g_alloc_counter = nullptr;

template <typename T>
T *dalloc(size_t n, std::vector<void *> &owned) {
  void *p = nullptr;
  if (n == 0) n = 1;
  if (g_alloc_counter) *g_alloc_counter += n * sizeof(T);
  cudaError_t e = cudaMalloc(&p, n * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw OwtError(OWT_ERR_NOMEM, std::string("cudaMalloc of ") + std::to_string(n * sizeof(T)) +
                                      " bytes failed: " + cudaGetErrorString(e));
  }
  owned.push_back(p);
  return static_cast<T *>(p);
}

template <typename T>
T *upload(const std::vector<T> &v, std::vector<void *> &owned, cudaStream_t st) {
  T *d = dalloc<T>(v.size(), owned);
  ck(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st), "upload");
  return d;
}

struct BandDev {
  double *ab = nullptr;
  uint8_t *piv = nullptr;
  double *rscale = nullptr;  // inverse row scales [n][U] (null: rows not scaled)
  int n = 0, kl = 0, ku = 0;
};

}  // namespace

void owt_set_thread_error(const std::string &m) { g_create_error = m; }

struct owt_handle {
  std::string err;
  owt_params p{};
  int NX = 0, NY = 0, NZ = 0, NXH = 0, NZH = 0, NX2 = 0, NZ2 = 0, M = 0, Uq = 0;
  int precision = 0;
  cudaStream_t st = nullptr;
  cudaStream_t st2 = nullptr;                    // the mean-mode branch of a step
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;    // the mean mode beside the mode kernel
  cudaEvent_t ev_fork2 = nullptr, ev_join2 = nullptr;  // the mean-flow terms beside the transforms
  std::vector<void *> owned;
  int64_t steps = 0;
  int64_t launches = 0;
  bool initialized = false;
  bool use_graph = false;
  cudaGraphExec_t gexec = nullptr;
  cudaGraph_t graph = nullptr;
  bool q_dirty[3] = {false, false, false};
  bool sparse_v = false;        // interior fill of every v-system inside the masks
  bool sparse_v6 = false;       // the same against the sixth-order masks (fd_order 6)
  int pattern_violations = 0;   // modes that forced the dense solve
  Grid grid;
  double Ly = 0, inv_cg0 = 0;
  size_t fs = 0;  // complex values per spectral field
  // device constants
  double *kx = nullptr, *kz = nullptr, *c11 = nullptr, *c21 = nullptr, *c22 = nullptr, *inv_cg = nullptr;
  double *nc21 = nullptr, *nc22 = nullptr;  // nu c21, nu c22
  // state
  double2 *v_ring = nullptr, *g_ring = nullptr, *hv_ring = nullptr, *hg_ring = nullptr, *q_ring = nullptr;
  double2 *u = nullptr, *w = nullptr, *ox = nullptr, *oz = nullptr, *lx = nullptr, *ly = nullptr, *lz = nullptr;
  double2 *U_ring = nullptr, *W_ring = nullptr, *lxm_ring = nullptr, *lzm_ring = nullptr;
  double *fx_ring = nullptr, *fz_ring = nullptr;
  double2 *lm = nullptr;  // mixed precision: FP64 mean-flow terms of the Lamb vector [3][NY][M]
  double *ygrid = nullptr, *wy = nullptr;  // y and its trapezoidal weights (summing to 1)
  double *ic_partial = nullptr;            // seeded initial condition: RMS partial sums
  long long *d_step = nullptr;
  int *d_err = nullptr;
  // factors and tables
  BandDev bv, bg, b1, b2;
  int *rhs_node_v = nullptr, *rb_col = nullptr, *b1_col = nullptr, *b2_col = nullptr, *rbv_col = nullptr;
  double *rbv_val = nullptr;
  double *rb_val = nullptr, *b1_val = nullptr, *b2_val = nullptr;
  // scratch
  double2 *sg = nullptr, *dg = nullptr, *yv = nullptr, *yg = nullptr, *sv = nullptr;
  double2 *mean_scratch = nullptr, *mean_dy1 = nullptr;
  double2 *bf = nullptr, *yscr = nullptr, *tmpA = nullptr, *tmpB = nullptr, *tmpC = nullptr, *stage = nullptr;
  void *zbuf = nullptr, *lbuf = nullptr;
  void *twx[2] = {nullptr, nullptr}, *twz[2] = {nullptr, nullptr};
  FftPlan px{}, pz{};
  // wall blowing/suction: v on the walls, [2][M] (bottom, top); null = no-slip
  double2 *vw = nullptr;
  bool vw_on = false;
  int *b1t_col = nullptr;  // B_1 transposed, (row, val) x 8 per column
  double *b1t_val = nullptr;
  // changes whenever the state or the wall velocity is replaced from outside
  // the drag runs, so a reverse sweep can tell that its record is stale
  int64_t state_version = 0;

  int head() const { return (int)((2 * (steps % 3)) % 3); }
  int slot(int level) const { return (head() + level) % 3; }
  double2 *ring_level(double2 *ring, int level) const { return ring + (size_t)slot(level) * fs; }

  ~owt_handle() {
    if (st) cudaStreamSynchronize(st);
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    for (void *q : owned) cudaFree(q);
    for (cudaEvent_t e : {ev_fork, ev_join, ev_fork2, ev_join2})
      if (e) cudaEventDestroy(e);
    if (st2) cudaStreamDestroy(st2);
    if (st) cudaStreamDestroy(st);
  }

  void check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
  }

  // ---- setup -----------------------------------------------------------------
  size_t device_bytes = 0;
  std::string setup_report;  // wall time of the setup phases
  void setup(const owt_params &prm) {
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
    ck(cudaStreamCreateWithFlags(&st2, cudaStreamNonBlocking), "cudaStreamCreate");
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
    pad_band(tv, 15, 13);
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
    lm = dalloc<double2>(3 * fs, owned);
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

  // ---- kernel sequences --------------------------------------------------------
  void dapply(int order, const double2 *in, double2 *out) {
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
  XformArgs xform_args() const {
    XformArgs a{};
    a.d = XformDims{NY, NZ, NXH, NZH, NX2, NZ2};
    a.in[0] = u; a.in[1] = v_ring; a.in[2] = w; a.in[3] = ox; a.in[4] = g_ring; a.in[5] = oz;
    a.ring_mask = (1 << 1) | (1 << 4);
    a.fs = fs;
    a.step = d_step;
    a.mean_split = precision == OWT_PREC_MIXED ? 1 : 0;
    for (int f = 0; f < 3; ++f) a.lm[f] = lm + (size_t)f * fs;
    a.out[0] = lx; a.out[1] = ly; a.out[2] = lz;
    a.zbuf = zbuf; a.lbuf = lbuf;
    a.px = px; a.pz = pz;
    a.twx = twx[precision]; a.twz = twz[precision];
    a.inv_nx2 = 1.0 / (double)NX2; a.inv_nz2 = 1.0 / (double)NZ2;
    return a;
  }
  NLArgs nl_args(bool record_mean) const {
    NLArgs a{};
    a.NY = NY; a.NZ = NZ; a.NXH = NXH; a.M = M;
    a.kx = kx; a.kz = kz; a.c11 = c11;
    a.lx = lx; a.ly = ly; a.lz = lz;
    a.hv_ring = hv_ring; a.hg_ring = hg_ring;
    a.ab1 = b1.ab; a.piv1 = b1.piv; a.b1_col = b1_col; a.b1_val = b1_val;
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
  void enqueue_step() {
    ck(cudaEventRecord(ev_fork, st), "fork");
    ck(cudaStreamWaitEvent(st2, ev_fork, 0), "fork wait");
    stage_mean(true, st2);
    ck(cudaEventRecord(ev_join, st2), "join");
    stage_modes();
    ck(cudaStreamWaitEvent(st, ev_join, 0), "join wait");
    launch_advance(d_step, st);
    const XformArgs xa = xform_args();
    int nx = 3;
    if (xa.mean_split) {
      // the FP64 mean-flow terms beside the FP32 z backward and x pass
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
  void stage_modes() {
    if (sparse_v6 && !force_dense) {
      launch_modes_sixth(mode_args(), st);
      return;
    }
    launch_modes(mode_args(), bv.kl, bv.ku, bg.kl, bg.ku, modes_sparse(),
                 forced_variant >= 0 ? forced_variant : modes_variant, st);
  }
  bool modes_sparse() const { return sparse_v && !force_dense; }
  ModeArgs mode_args() const {
    ModeArgs a{};
    a.NY = NY; a.NZ = NZ; a.NXH = NXH; a.NZH = NZH; a.M = M; a.U = Uq;
    a.inv_dt = 1.0 / p.dt; a.nu = p.nu;
    a.kx = kx; a.kz = kz; a.c11 = c11; a.c21 = c21; a.c22 = c22;
    a.v_ring = v_ring; a.g_ring = g_ring; a.hv_ring = hv_ring; a.hg_ring = hg_ring; a.q_ring = q_ring;
    a.u_out = u; a.w_out = w; a.ox_out = ox; a.oz_out = oz;
    a.ab_v = bv.ab; a.piv_v = bv.piv; a.n_v = bv.n;
    a.ab_g = bg.ab; a.piv_g = bg.piv; a.n_g = bg.n;
    a.rhs_node_v = rhs_node_v; a.rb_col = rb_col; a.rb_val = rb_val; a.inv_cg = inv_cg;
    a.rs_v = bv.rscale; a.rs_g = bg.rscale;
    a.inv_h = 1.0 / grid.ds; a.inv_h2 = 1.0 / (grid.ds * grid.ds);
    a.sg = sg; a.dg = dg; a.yv = yv; a.yg = yg; a.sv = sv;
    a.rbv_col = rbv_col; a.rbv_val = rbv_val;
    a.nc21 = nc21; a.nc22 = nc22;
    a.step = d_step;
    a.vw = vw_on ? vw : nullptr;
    return a;
  }
  void stage_mean(bool pre_advance = false, cudaStream_t s = nullptr) {
    launch_mean(mean_args(pre_advance), mean_smem, s ? s : st);
  }
  MeanArgs mean_args(bool pre_advance) const {
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

  void run_steps(int64_t n) {
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
        ck(cudaGraphInstantiate(&gexec, graph, 0), "graph instantiate");
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
  int64_t per_step_launches = 0;
  bool force_dense = false;  // testing aid: always sweep the full band
  bool mean_smem = false;    // staged mean-mode solve in shared memory
  int modes_variant = 0;     // chosen by the autotuner
  int forced_variant = -1;   // testing aid: run this variant instead
  std::string tuning;        // autotuner report

  // Autotuner: time every mode-kernel variant, keep the fastest.  Variants
  // differ only in thread mapping and block shape; their results are bitwise
  // identical, so the choice affects speed only.  It runs once, before the
  // handle's first own step (a handle stepped only inside a batch never needs
  // it); on a live state the rings and fields the trials overwrite are copied
  // aside and put back.
  bool tuned = false;
  void ensure_tuned() {
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
  void autotune_modes() {
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

  void drop_graph() {
    if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
    if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
  }

  // DY2 v for history levels whose v was replaced from the host (one launch).
  void recompute_dirty_q() {
    DY2Args a{};
    a.NY = NY; a.M = M;
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
    launch_dy2(a, st);
    ++launches;
  }

  void copy_ring(double2 *ring, size_t n, int from, int to) {
    ck(cudaMemcpyAsync(ring + (size_t)to * n, ring + (size_t)from * n, n * sizeof(double2), cudaMemcpyDeviceToDevice,
                       st), "ring copy");
  }
  // column of mode 0 of a device-layout field -> contiguous NY vector
  void mode0_column(double2 *dst, const double2 *field) {
    ck(cudaMemcpy2DAsync(dst, sizeof(double2), field, (size_t)M * sizeof(double2), sizeof(double2), NY,
                         cudaMemcpyDeviceToDevice, st), "mode-0 column");
  }

  void get_vor_from_vel() {
    dapply(1, u, tmpA);
    dapply(1, w, tmpB);
    VorArgs va{};
    va.NY = NY; va.NXH = NXH; va.M = M; va.kx = kx; va.kz = kz; va.c11 = c11;
    va.u = u; va.v = ring_level(v_ring, 0); va.w = w; va.d1u = tmpA; va.d1w = tmpB;
    va.ox = ox; va.oy = ring_level(g_ring, 0); va.oz = oz;
    launch_vor(va, st);
    ++launches;
  }
  void lamb_vec(bool explicit_shift) {
    launches += launch_lamb(xform_args(), precision, st);
    if (explicit_shift) {
      launch_lamb_mean_shift(lxm_ring, lzm_ring, lx, lz, NY, M, d_step, st);
      ++launches;
    }
  }
  void nonlinear_source(bool record_mean) {
    launch_nl(nl_args(record_mean), st);
    ++launches;
  }
  void friction(int shift) {
    dapply(1, u, tmpA);
    dapply(1, w, tmpB);
    launch_friction(tmpA, tmpB, c11, NY, M, p.nu, Ly, fx_ring, fz_ring, d_step, shift, d_err, st);
    ++launches;
  }

  void init_prologue() {
    steps = 0;
    drop_graph();
    ck(cudaMemsetAsync(d_step, 0, sizeof(long long), st), "memset");
    ck(cudaMemsetAsync(d_err, 0, sizeof(int), st), "memset");
  }
  void init_fields(const double *hu, const double *hv, const double *hw) {
    init_prologue();
    to_device(hu, u);
    to_device(hv, ring_level(v_ring, 0));
    to_device(hw, w);
    init_from_velocity();
  }
  // The seeded laminar + random divergence-free state, generated on the
  // device (seeded_ic.cu); the Chebyshev coefficients live in the mean-flow
  // buffer and omega_y in tmpC until the velocity is complete.
  void init_seeded(uint64_t seed, double rms) {
    init_prologue();
    SeedArgs a{};
    a.NY = NY; a.NZ = NZ; a.NXH = NXH; a.NZH = NZH; a.M = M; a.degree = 5;
    a.seed = seed;
    a.kmin = std::min(p.dkx, p.dkz);
    a.kx = kx; a.kz = kz; a.y = ygrid; a.c11 = c11; a.wy = wy;
    a.coef = lm;  // 3 NY M >= 12 M values
    double2 *v0 = ring_level(v_ring, 0);
    launches += launch_ic_fields(a, v0, tmpC, st);
    dapply(1, v0, tmpA);
    launches += launch_ic_velocity(a, tmpA, tmpC, u, v0, w, ic_partial, rms, st);
    check_launch("seeded initial condition");
    init_from_velocity();
  }
  void init_from_velocity() {
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

  // ---- host <-> device in the reference layout ---------------------------------
  void to_device(const double *host, double2 *dst) {
    ck(cudaMemcpyAsync(stage, host, fs * sizeof(double2), cudaMemcpyHostToDevice, st), "H2D");
    launch_transpose(stage, dst, M, NY, st);  // [M][NY] -> [NY][M]
    ++launches;
    check_launch("layout transpose");
  }
  void to_host(const double2 *src, double *host) {
    launch_transpose(src, stage, NY, M, st);  // [NY][M] -> [M][NY]
    ++launches;
    check_launch("layout transpose");
    ck(cudaMemcpyAsync(host, stage, fs * sizeof(double2), cudaMemcpyDeviceToHost, st), "D2H");
    ck(cudaStreamSynchronize(st), "D2H");
  }
  double2 *field_ptr(int f, bool for_write) {
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
  double2 *mean_ptr(int which) {
    if (which < 0 || which >= OWT_NUM_MEANS) throw OwtError(OWT_ERR_INVALID, "unknown mean id");
    double2 *rings[4] = {lxm_ring, lzm_ring, U_ring, W_ring};
    return rings[which / 3] + (size_t)slot(which % 3) * NY;
  }
  // ---- wall-drag adjoint -------------------------------------------------------
  // Objective J = (1/N) sum_{n=1..N} fx_n over the N steps of a forward run,
  // fx_n the driving force of step n (src/solver.cpp:306-312), which equals
  // the wall shear stress averaged over both walls.  The forward run keeps a
  // device image of the full state every `interval` steps; the reverse sweep
  // recomputes each segment from its image, recording the six spectral fields
  // every step reads in its Lamb vector (the tape), and runs the adjoint steps
  // of that segment backwards.
  struct Adjoint {
    bool ready = false;
    double2 *hist[5][3] = {};  // adjoints of the v, omega_y, Hv, Hg, DY2 v histories
    double2 *mean[4][3] = {};  // U, W, mean lx, mean lz
    double *fric[2][3] = {};   // fx, fz
    double2 *lb[3] = {}, *fb[6] = {}, *xs[7] = {};
    double2 *zbuf = nullptr, *lbuf = nullptr, *yv = nullptr, *yg = nullptr, *mscr = nullptr, *grad = nullptr;
    double *fric_block = nullptr;
    double *obj = nullptr;
    std::vector<double2 *> ckpt;
    std::vector<int64_t> ckpt_step;
    double2 *tape = nullptr;
    int64_t tape_len = 0;
    int64_t nsteps = 0, interval = 0;
    int64_t version = -1;  // state_version right after the forward run
  } adj;
  long long staged_step = 0;  // host source of the step-counter upload
  double2 *kept = nullptr;    // owt_state_keep's image
  int64_t kept_step = -1;

  void free_owned(void *q) {
    for (auto it = owned.begin(); it != owned.end(); ++it)
      if (*it == q) { owned.erase(it); break; }
    cudaFree(q);
  }
  void d2d(void *dst, const void *src, size_t bytes) {
    ck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st), "device copy");
  }
  size_t image_values() const { return 15 * fs + 12 * (size_t)NY + 3; }
  // full state: the five 3-slot rings, the four mean rings, the friction rings
  void save_image(double2 *img, int64_t &step_out) {
    double2 *o = img;
    for (double2 *ring : {v_ring, g_ring, hv_ring, hg_ring, q_ring}) { d2d(o, ring, 3 * fs * sizeof(double2)); o += 3 * fs; }
    for (double2 *ring : {U_ring, W_ring, lxm_ring, lzm_ring}) { d2d(o, ring, 3 * (size_t)NY * sizeof(double2)); o += 3 * NY; }
    d2d(o, fx_ring, 3 * sizeof(double));
    d2d(reinterpret_cast<double *>(o) + 3, fz_ring, 3 * sizeof(double));
    step_out = steps;
  }
  void load_image(const double2 *img, int64_t step) {
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

  double drag_forward(int64_t n, int64_t interval) {
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

  void adj_alloc() {
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

  void adjoint_step(const double2 *tp, double wgt) {
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
    launch_adj_mean(ma, st);

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
    launch_adj_modes(mo, st);
    launches += 6;
    check_launch("adjoint step");
    // the buffers now hold the adjoints of the levels the step read, level l
    // of the old state in buffer l + 1 (mod 3)
    auto rot = [](auto *x) { auto t = x[0]; x[0] = x[1]; x[1] = x[2]; x[2] = t; };
    for (auto &h3 : adj.hist) rot(h3);
    for (auto &m3 : adj.mean) rot(m3);
    for (auto &f3 : adj.fric) rot(f3);
  }

  void drag_backward(double gJ, double *grad_bottom, double *grad_top) {
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

  void sync_and_check() {
    ck(cudaStreamSynchronize(st), "synchronize");
    int e = 0;
    ck(cudaMemcpy(&e, d_err, sizeof(int), cudaMemcpyDeviceToHost), "status");
    if (e == 2) throw OwtError(OWT_ERR_NUMERIC, "non-finite friction force: the state has blown up");
    if (e) throw OwtError(OWT_ERR_NUMERIC, "device reported a numeric failure");
  }
};

namespace {

template <typename F>
int guard(owt_handle *h, F &&f) {
  if (!h) return OWT_ERR_INVALID;
  try {
    f();
    h->err.clear();
    return OWT_OK;
  } catch (const OwtError &e) {
    h->err = e.what();
    return e.code;
  } catch (const CudaError &e) {
    h->err = e.what();
    return OWT_ERR_CUDA;
  } catch (const std::exception &e) {
    h->err = e.what();
    return OWT_ERR_INVALID;
  }
}

}  // namespace

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
      std::map<std::pair<int, int>, std::vector<int>> groups;
      std::vector<int> blocks(n, 0);
      for (int i = 0; i < n; ++i) {
        const owt_handle *h = hs[i];
        if (part == 3 && h->precision != OWT_PREC_MIXED) continue;
        const XformDims &d = xargs[i].d;
        const int prec = h->precision == OWT_PREC_MIXED ? 1 : 0;
        if (part == 0) ck(lamb_batch_prepare(d, prec), "transform kernel attributes");
        blocks[i] = lamb_batch_blocks(d, prec, part);
        const int len = part == 1 ? d.NX2 : part == 3 ? 0 : d.NZ2;
        groups[{prec, len}].push_back(i);
      }
      for (auto &g : groups)
        for (auto &t : make_tables(xargs, blocks, g.second)) lamb.push_back({std::move(t), g.first.first, part});
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
      for (int v = 0; v < modes_variant_count(); ++v) {
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

int owt_create(const owt_params *params, owt_handle **out) {
  if (!params || !out) {
    g_create_error = "null argument";
    return OWT_ERR_INVALID;
  }
  *out = nullptr;
  owt_handle *h = new owt_handle();
  try {
    h->setup(*params);
  } catch (const OwtError &e) {
    g_create_error = e.what();
    delete h;
    return e.code;
  } catch (const std::exception &e) {
    g_create_error = e.what();
    delete h;
    return dynamic_cast<const CudaError *>(&e) ? OWT_ERR_CUDA : OWT_ERR_INVALID;
  }
  *out = h;
  return OWT_OK;
}

int owt_destroy(owt_handle *h) {
  delete h;
  return OWT_OK;
}

const char *owt_last_error(const owt_handle *h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int owt_init_fields(owt_handle *h, const double *velx, const double *vely, const double *velz) {
  return guard(h, [&] {
    if (!velx || !vely || !velz) throw OwtError(OWT_ERR_INVALID, "null field");
    ++h->state_version;
    h->init_fields(velx, vely, velz);
    h->sync_and_check();
  });
}

int owt_band_factor_selftest(int kl, int ku, int n, int U, uint64_t seed, int64_t *mismatches, float *ms_thread,
                             float *ms_warp) {
  if (!mismatches || !ms_thread || !ms_warp || n < 1 || U < 1 || !band_supported(kl, ku)) {
    g_create_error = "owt_band_factor_selftest: bad arguments";
    return OWT_ERR_INVALID;
  }
  long long bad = 0;
  if (band_factor_selftest(kl, ku, n, U, seed, &bad, ms_thread, ms_warp) != 0) {
    g_create_error = "owt_band_factor_selftest: CUDA error";
    cudaGetLastError();
    return OWT_ERR_CUDA;
  }
  *mismatches = bad;
  return OWT_OK;
}

int owt_init_seeded(owt_handle *h, uint64_t seed, double rms) {
  return guard(h, [&] {
    if (!(rms >= 0.0)) throw OwtError(OWT_ERR_INVALID, "rms must be non-negative");
    ++h->state_version;
    h->init_seeded(seed, rms);
    h->sync_and_check();
  });
}

int owt_time_integration(owt_handle *h, int64_t nsteps) {
  return guard(h, [&] {
    if (!h->initialized) throw OwtError(OWT_ERR_STATE, "owt_init_fields (or field uploads) must come first");
    if (nsteps < 0) throw OwtError(OWT_ERR_INVALID, "negative step count");
    ++h->state_version;
    h->run_steps(nsteps);
  });
}

int owt_call(owt_handle *h, int routine) {
  return guard(h, [&] {
    ++h->state_version;
    switch (routine) {
      case OWT_CALL_GET_VOR_FROM_VEL: h->get_vor_from_vel(); break;
      case OWT_CALL_LAMB_VEC: h->lamb_vec(true); break;
      case OWT_CALL_NONLINEAR_SOURCE: h->nonlinear_source(false); break;
      case OWT_CALL_SOLVE_FRICTION_FORCE: h->friction(1); break;
      case OWT_CALL_TIME_INTEGRATION:
        if (!h->initialized) throw OwtError(OWT_ERR_STATE, "owt_init_fields (or field uploads) must come first");
        h->run_steps(1);
        break;
      default: throw OwtError(OWT_ERR_INVALID, "unknown routine id");
    }
    h->check_launch("owt_call");
    h->sync_and_check();
  });
}

int owt_synchronize(owt_handle *h) {
  return guard(h, [&] { h->sync_and_check(); });
}

int owt_get_field(owt_handle *h, int field, double *host) {
  return guard(h, [&] {
    if (!host) throw OwtError(OWT_ERR_INVALID, "null buffer");
    h->to_host(h->field_ptr(field, false), host);
  });
}

int owt_set_field(owt_handle *h, int field, const double *host) {
  return guard(h, [&] {
    if (!host) throw OwtError(OWT_ERR_INVALID, "null buffer");
    ++h->state_version;
    h->to_device(host, h->field_ptr(field, true));
    ck(cudaStreamSynchronize(h->st), "set field");
    h->initialized = true;
  });
}

int owt_get_mean(owt_handle *h, int which, double *host) {
  return guard(h, [&] {
    if (!host) throw OwtError(OWT_ERR_INVALID, "null buffer");
    ck(cudaMemcpyAsync(host, h->mean_ptr(which), h->NY * sizeof(double2), cudaMemcpyDeviceToHost, h->st), "D2H");
    ck(cudaStreamSynchronize(h->st), "D2H");
  });
}

int owt_set_mean(owt_handle *h, int which, const double *host) {
  return guard(h, [&] {
    if (!host) throw OwtError(OWT_ERR_INVALID, "null buffer");
    ++h->state_version;
    ck(cudaMemcpyAsync(h->mean_ptr(which), host, h->NY * sizeof(double2), cudaMemcpyHostToDevice, h->st), "H2D");
    ck(cudaStreamSynchronize(h->st), "H2D");
  });
}

int owt_get_friction(owt_handle *h, double *out6) {
  return guard(h, [&] {
    if (!out6) throw OwtError(OWT_ERR_INVALID, "null buffer");
    double fx[3], fz[3];
    ck(cudaMemcpyAsync(fx, h->fx_ring, sizeof(fx), cudaMemcpyDeviceToHost, h->st), "D2H");
    ck(cudaMemcpyAsync(fz, h->fz_ring, sizeof(fz), cudaMemcpyDeviceToHost, h->st), "D2H");
    h->sync_and_check();
    for (int l = 0; l < 3; ++l) {
      out6[l] = fx[h->slot(l)];
      out6[3 + l] = fz[h->slot(l)];
    }
  });
}

int owt_set_friction(owt_handle *h, const double *in6) {
  return guard(h, [&] {
    if (!in6) throw OwtError(OWT_ERR_INVALID, "null buffer");
    double fx[3], fz[3];
    ++h->state_version;
    for (int l = 0; l < 3; ++l) {
      fx[h->slot(l)] = in6[l];
      fz[h->slot(l)] = in6[3 + l];
    }
    ck(cudaMemcpyAsync(h->fx_ring, fx, sizeof(fx), cudaMemcpyHostToDevice, h->st), "H2D");
    ck(cudaMemcpyAsync(h->fz_ring, fz, sizeof(fz), cudaMemcpyHostToDevice, h->st), "H2D");
    ck(cudaStreamSynchronize(h->st), "H2D");
  });
}

int owt_set_precision(owt_handle *h, int precision) {
  return guard(h, [&] {
    if (precision != OWT_PREC_FP64 && precision != OWT_PREC_MIXED)
      throw OwtError(OWT_ERR_INVALID, "precision must be OWT_PREC_FP64 or OWT_PREC_MIXED");
    if (precision != h->precision) {
      ++h->state_version;
      ck(cudaStreamSynchronize(h->st), "set precision");
      h->drop_graph();
      h->precision = precision;
    }
  });
}

int owt_use_graph(owt_handle *h, int on) {
  return guard(h, [&] {
    ck(cudaStreamSynchronize(h->st), "use graph");
    if (!on) h->drop_graph();
    h->use_graph = on != 0;
  });
}

int owt_get_step(const owt_handle *h, int64_t *step) {
  if (!h || !step) return OWT_ERR_INVALID;
  *step = h->steps;
  return OWT_OK;
}

int owt_get_stream(const owt_handle *h, void **stream) {
  if (!h || !stream) return OWT_ERR_INVALID;
  *stream = (void *)h->st;
  return OWT_OK;
}

int owt_get_launch_count(const owt_handle *h, int64_t *count) {
  if (!h || !count) return OWT_ERR_INVALID;
  *count = h->launches;
  return OWT_OK;
}

int owt_get_grid(const owt_handle *h, double *y) {
  if (!h || !y) return OWT_ERR_INVALID;
  std::memcpy(y, h->grid.y.data(), h->grid.y.size() * sizeof(double));
  return OWT_OK;
}

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
    ck(cudaStreamCreateWithFlags(&b->st2, cudaStreamNonBlocking), "stream");
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
    ck(cudaGraphInstantiate(&b->exec, b->graph, 0), "instantiate");
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

int owt_statistics(owt_handle *h, double *out7ny) {
  return guard(h, [&] {
    if (!out7ny) throw OwtError(OWT_ERR_INVALID, "null buffer");
    double *d = reinterpret_cast<double *>(h->tmpA);  // 7 NY doubles fit easily
    launch_stats(h->u, h->ring_level(h->v_ring, 0), h->w, h->NY, h->NZ, h->NXH, d, h->st);
    ++h->launches;
    h->check_launch("statistics");
    ck(cudaMemcpyAsync(out7ny, d, 7 * (size_t)h->NY * sizeof(double), cudaMemcpyDeviceToHost, h->st), "D2H");
    h->sync_and_check();
  });
}

// Checkpoint image: header, then fields in level order (independent of the
// ring slots), then the NY-vectors and scalars.
namespace {
struct CkptHeader {
  char magic[8];
  int64_t version, NX, NY, NZ, step, precision;
  double dt, dkx, dkz, alpha_mesh, nu;
};
const int kRings = 5, kFields = 7;
}  // namespace

int owt_checkpoint_bytes(const owt_handle *h, int64_t *bytes) {
  if (!h || !bytes) return OWT_ERR_INVALID;
  const size_t f = h->fs * sizeof(double2), v = (size_t)h->NY * sizeof(double2);
  *bytes = (int64_t)(sizeof(CkptHeader) + (3 * kRings + kFields) * f + 12 * v + 6 * sizeof(double));
  return OWT_OK;
}

int owt_checkpoint_save(owt_handle *h, void *host, int64_t bytes) {
  return guard(h, [&] {
    int64_t need = 0;
    owt_checkpoint_bytes(h, &need);
    if (!host || bytes < need) throw OwtError(OWT_ERR_INVALID, "checkpoint buffer too small");
    ck(cudaStreamSynchronize(h->st), "checkpoint");
    h->recompute_dirty_q();
    CkptHeader hd{};
    std::memcpy(hd.magic, "OWTCKPT1", 8);
    hd.version = 1; hd.NX = h->NX; hd.NY = h->NY; hd.NZ = h->NZ; hd.step = h->steps; hd.precision = h->precision;
    hd.dt = h->p.dt; hd.dkx = h->p.dkx; hd.dkz = h->p.dkz; hd.alpha_mesh = h->p.alpha_mesh; hd.nu = h->p.nu;
    char *o = static_cast<char *>(host);
    std::memcpy(o, &hd, sizeof(hd));
    o += sizeof(hd);
    const size_t f = h->fs * sizeof(double2), v = (size_t)h->NY * sizeof(double2);
    for (double2 *ring : {h->v_ring, h->g_ring, h->hv_ring, h->hg_ring, h->q_ring})
      for (int l = 0; l < 3; ++l, o += f)
        ck(cudaMemcpyAsync(o, h->ring_level(ring, l), f, cudaMemcpyDeviceToHost, h->st), "D2H");
    for (double2 *fld : {h->u, h->w, h->ox, h->oz, h->lx, h->ly, h->lz}) {
      ck(cudaMemcpyAsync(o, fld, f, cudaMemcpyDeviceToHost, h->st), "D2H");
      o += f;
    }
    for (double2 *ring : {h->lxm_ring, h->lzm_ring, h->U_ring, h->W_ring})
      for (int l = 0; l < 3; ++l, o += v)
        ck(cudaMemcpyAsync(o, ring + (size_t)h->slot(l) * h->NY, v, cudaMemcpyDeviceToHost, h->st), "D2H");
    for (double *fr : {h->fx_ring, h->fz_ring})
      for (int l = 0; l < 3; ++l, o += sizeof(double))
        ck(cudaMemcpyAsync(o, fr + h->slot(l), sizeof(double), cudaMemcpyDeviceToHost, h->st), "D2H");
    ck(cudaStreamSynchronize(h->st), "checkpoint");
  });
}

int owt_checkpoint_load(owt_handle *h, const void *host, int64_t bytes) {
  return guard(h, [&] {
    int64_t need = 0;
    owt_checkpoint_bytes(h, &need);
    if (!host || bytes < need) throw OwtError(OWT_ERR_INVALID, "checkpoint image too small");
    CkptHeader hd;
    std::memcpy(&hd, host, sizeof(hd));
    if (std::memcmp(hd.magic, "OWTCKPT1", 8) != 0 || hd.version != 1)
      throw OwtError(OWT_ERR_INVALID, "not a checkpoint image of this library");
    if (hd.NX != h->NX || hd.NY != h->NY || hd.NZ != h->NZ || hd.dt != h->p.dt || hd.dkx != h->p.dkx ||
        hd.dkz != h->p.dkz || hd.alpha_mesh != h->p.alpha_mesh || hd.nu != h->p.nu)
      throw OwtError(OWT_ERR_INVALID, "checkpoint parameters differ from the handle's");
    ck(cudaStreamSynchronize(h->st), "restore");
    ++h->state_version;
    h->drop_graph();
    h->steps = hd.step;
    const long long dstep = (long long)hd.step;
    ck(cudaMemcpyAsync(h->d_step, &dstep, sizeof(dstep), cudaMemcpyHostToDevice, h->st), "H2D");
    const char *o = static_cast<const char *>(host) + sizeof(hd);
    const size_t f = h->fs * sizeof(double2), v = (size_t)h->NY * sizeof(double2);
    for (double2 *ring : {h->v_ring, h->g_ring, h->hv_ring, h->hg_ring, h->q_ring})
      for (int l = 0; l < 3; ++l, o += f)
        ck(cudaMemcpyAsync(h->ring_level(ring, l), o, f, cudaMemcpyHostToDevice, h->st), "H2D");
    for (double2 *fld : {h->u, h->w, h->ox, h->oz, h->lx, h->ly, h->lz}) {
      ck(cudaMemcpyAsync(fld, o, f, cudaMemcpyHostToDevice, h->st), "H2D");
      o += f;
    }
    for (double2 *ring : {h->lxm_ring, h->lzm_ring, h->U_ring, h->W_ring})
      for (int l = 0; l < 3; ++l, o += v)
        ck(cudaMemcpyAsync(ring + (size_t)h->slot(l) * h->NY, o, v, cudaMemcpyHostToDevice, h->st), "H2D");
    for (double *fr : {h->fx_ring, h->fz_ring})
      for (int l = 0; l < 3; ++l, o += sizeof(double))
        ck(cudaMemcpyAsync(fr + h->slot(l), o, sizeof(double), cudaMemcpyHostToDevice, h->st), "H2D");
    h->q_dirty[0] = h->q_dirty[1] = h->q_dirty[2] = false;
    h->initialized = true;
    ck(cudaStreamSynchronize(h->st), "restore");
  });
}

int owt_set_option(owt_handle *h, int option, int64_t value) {
  return guard(h, [&] {
    ck(cudaStreamSynchronize(h->st), "set option");
    h->drop_graph();
    if (option == OWT_OPT_FORCE_DENSE_BANDS) {
      h->force_dense = value != 0;
    } else if (option == OWT_OPT_MODES_VARIANT) {
      if (value < -1 || value >= modes_variant_count()) throw OwtError(OWT_ERR_INVALID, "no such variant");
      h->forced_variant = (int)value;
    } else {
      throw OwtError(OWT_ERR_INVALID, "unknown option");
    }
  });
}

const char *owt_tuning_report(const owt_handle *h) { return h ? h->tuning.c_str() : ""; }
const char *owt_setup_report(const owt_handle *h) { return h ? h->setup_report.c_str() : ""; }

int owt_get_info(const owt_handle *h, int what, int64_t *value) {
  if (!h || !value) return OWT_ERR_INVALID;
  switch (what) {
    case OWT_INFO_SPARSE_SOLVE: *value = ((h->sparse_v || h->sparse_v6) && !h->force_dense) ? 1 : 0; return OWT_OK;
    case OWT_INFO_PATTERN_VIOLATIONS: *value = h->pattern_violations; return OWT_OK;
    case OWT_INFO_DEVICE_BYTES: *value = (int64_t)h->device_bytes; return OWT_OK;
    case OWT_INFO_MODES_VARIANT: *value = h->forced_variant >= 0 ? h->forced_variant : h->modes_variant; return OWT_OK;
    case OWT_INFO_MODES_VARIANTS: *value = modes_variant_count(); return OWT_OK;
    default: return OWT_ERR_INVALID;
  }
}

int owt_enqueue_stage(owt_handle *h, int stage) {
  return guard(h, [&] {
    if (!h->initialized) throw OwtError(OWT_ERR_STATE, "owt_init_fields must come first");
    switch (stage) {
      case OWT_STAGE_MODES: h->ensure_tuned(); h->stage_modes(); h->launches += 1; break;
      case OWT_STAGE_MEAN: h->stage_mean(); h->launches += 1; break;
      case OWT_STAGE_LAMB: h->launches += launch_lamb(h->xform_args(), h->precision, h->st); break;
      case OWT_STAGE_NONLINEAR: launch_nl(h->nl_args(true), h->st); h->launches += 1; break;
      case OWT_STAGE_ZBACK: case OWT_STAGE_XLAMB: case OWT_STAGE_ZFWD: case OWT_STAGE_MEAN_LAMB:
        launch_lamb_part(h->xform_args(), h->precision, stage - OWT_STAGE_ZBACK, h->st);
        h->launches += 1;
        break;
      default: throw OwtError(OWT_ERR_INVALID, "unknown stage");
    }
    h->check_launch("stage");
  });
}

int owt_set_wall_velocity(owt_handle *h, const double *vw_bottom, const double *vw_top) {
  return guard(h, [&] {
    if (!vw_bottom != !vw_top) throw OwtError(OWT_ERR_INVALID, "give both walls' velocities, or neither");
    ck(cudaStreamSynchronize(h->st), "wall velocity");
    ++h->state_version;
    const bool on = vw_bottom != nullptr;
    if (on) {
      if (!h->vw) h->vw = dalloc<double2>(2 * (size_t)h->M, h->owned);
      const size_t b = (size_t)h->M * sizeof(double2);
      ck(cudaMemcpyAsync(h->vw, vw_bottom, b, cudaMemcpyHostToDevice, h->st), "H2D");
      ck(cudaMemcpyAsync(h->vw + h->M, vw_top, b, cudaMemcpyHostToDevice, h->st), "H2D");
      ck(cudaStreamSynchronize(h->st), "H2D");
    }
    if (on != h->vw_on) h->drop_graph();  // the captured mode kernel holds the pointer
    h->vw_on = on;
  });
}

int owt_get_wall_velocity(owt_handle *h, double *vw_bottom, double *vw_top) {
  return guard(h, [&] {
    if (!vw_bottom || !vw_top) throw OwtError(OWT_ERR_INVALID, "null buffer");
    const size_t b = (size_t)h->M * sizeof(double2);
    if (!h->vw_on) {
      std::memset(vw_bottom, 0, b);
      std::memset(vw_top, 0, b);
      return;
    }
    ck(cudaMemcpyAsync(vw_bottom, h->vw, b, cudaMemcpyDeviceToHost, h->st), "D2H");
    ck(cudaMemcpyAsync(vw_top, h->vw + h->M, b, cudaMemcpyDeviceToHost, h->st), "D2H");
    ck(cudaStreamSynchronize(h->st), "D2H");
  });
}

int owt_state_keep(owt_handle *h) {
  return guard(h, [&] {
    if (!h->initialized) throw OwtError(OWT_ERR_STATE, "owt_init_fields (or field uploads) must come first");
    h->recompute_dirty_q();
    if (!h->kept) h->kept = dalloc<double2>(h->image_values(), h->owned);
    h->save_image(h->kept, h->kept_step);
    ck(cudaStreamSynchronize(h->st), "keep state");
  });
}

int owt_state_restore(owt_handle *h) {
  return guard(h, [&] {
    if (!h->kept) throw OwtError(OWT_ERR_STATE, "owt_state_keep must come first");
    ++h->state_version;
    h->load_image(h->kept, h->kept_step);
  });
}

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

int owt_dy_apply(owt_handle *h, int order, const double *in, double *out) {
  return guard(h, [&] {
    if (order != 1 && order != 2) throw OwtError(OWT_ERR_INVALID, "order must be 1 or 2");
    if (!in || !out) throw OwtError(OWT_ERR_INVALID, "null buffer");
    h->to_device(in, h->tmpC);
    h->dapply(1, h->tmpC, h->tmpA);
    if (order == 1) {
      launch_combine_y(h->tmpB, h->tmpA, h->c11, nullptr, nullptr, h->NY, h->M, h->st);
    } else {
      h->dapply(2, h->tmpC, h->tmpB);
      launch_combine_y(h->tmpB, h->tmpA, h->c21, h->tmpB, h->c22, h->NY, h->M, h->st);
    }
    ++h->launches;
    h->check_launch("dy apply");
    h->to_host(h->tmpB, out);
  });
}

}  // extern "C"

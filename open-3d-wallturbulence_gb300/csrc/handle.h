// The handle behind the C ABI (include/owt_gpu.h): one channel on one GPU --
// parameters, device-resident state, per-mode band factorizations, scratch
// and CUDA streams.  Its methods live in
//   handle_setup.cu   : creation (grid, operators, factorizations, buffers),
//                       teardown, synchronisation and status;
//   handle_step.cu    : the step's launch sequence, CUDA graph, autotuner,
//                       the reference routines one by one, init_fields, and
//                       the layout transposes of the host <-> device copies;
//   handle_adjoint.cu : state images, the wall-drag forward run and the
//                       reverse sweep of the discrete adjoint.
// The C entry points are in capi.cu (handles), capi_batch.cu (batches) and
// capi_checkpoint.cu (checkpoints and kept states).
#pragma once
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

namespace owt {

// Message of the calling thread's last failed call that takes no handle.
extern thread_local std::string g_create_error;
// While set, device allocations of dalloc are counted here.
extern thread_local size_t *g_alloc_counter;

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct OwtError : std::runtime_error {
  int code;
  OwtError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void ck(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

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

}  // namespace owt

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
  owt::Grid grid;
  double Ly = 0, inv_cg0 = 0;
  size_t fs = 0;  // complex values per spectral field
  // device constants
  double *kx = nullptr, *kz = nullptr, *c11 = nullptr, *c21 = nullptr, *c22 = nullptr, *inv_cg = nullptr;
  double *nc21 = nullptr, *nc22 = nullptr;  // nu c21, nu c22
  // the mode kernel's coefficients with the unscaling of its solved h d1,
  // h^2 d2: c11/h, c21/h, c22/h^2, nu c21/h, nu c22/h^2
  double *c11h = nullptr, *c21h = nullptr, *c22h = nullptr, *nc21h = nullptr, *nc22h = nullptr;
  double *rs_gi = nullptr;  // omega_y-system row scales times 1/cg of the mode [n_g][U]
  // state
  double2 *v_ring = nullptr, *g_ring = nullptr, *hv_ring = nullptr, *hg_ring = nullptr, *q_ring = nullptr;
  double2 *u = nullptr, *w = nullptr, *ox = nullptr, *oz = nullptr, *lx = nullptr, *ly = nullptr, *lz = nullptr;
  double2 *U_ring = nullptr, *W_ring = nullptr, *lxm_ring = nullptr, *lzm_ring = nullptr;
  double *fx_ring = nullptr, *fz_ring = nullptr;
  float2 *lm = nullptr;  // mixed precision: the mean-flow terms of the Lamb vector [3][NY][M], FP32
  double *ygrid = nullptr, *wy = nullptr;  // y and its trapezoidal weights (summing to 1)
  double *ic_partial = nullptr;            // seeded initial condition: RMS partial sums
  long long *d_step = nullptr;
  int *d_err = nullptr;
  // factors and tables
  owt::BandDev bv, bg, b1, b2;
  int *rhs_node_v = nullptr, *rb_col = nullptr, *b1_col = nullptr, *b2_col = nullptr, *rbv_col = nullptr;
  double *rbv_val = nullptr;
  double *rb_val = nullptr, *b1_val = nullptr, *b2_val = nullptr;
  // scratch
  double2 *sg = nullptr, *dg = nullptr, *yv = nullptr, *yg = nullptr, *sv = nullptr;
  double2 *mean_scratch = nullptr, *mean_dy1 = nullptr;
  double2 *bf = nullptr, *yscr = nullptr, *tmpA = nullptr, *tmpB = nullptr, *tmpC = nullptr, *stage = nullptr;
  void *zbuf = nullptr, *lbuf = nullptr;
  void *twx[2] = {nullptr, nullptr}, *twz[2] = {nullptr, nullptr};
  owt::FftPlan px{}, pz{};
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

  ~owt_handle();

  void check_launch(const char *what);

  // ---- setup -----------------------------------------------------------------
  size_t device_bytes = 0;
  std::string setup_report;  // wall time of the setup phases
  void setup(const owt_params &prm);

  // ---- kernel sequences --------------------------------------------------------
  void dapply(int order, const double2 *in, double2 *out);
  owt::XformArgs xform_args() const;
  owt::NLArgs nl_args(bool record_mean) const;
  // One time step.  Every argument is a fixed device pointer; which ring slot
  // is which history level is read from the device step counter, so the same
  // launch sequence (or its CUDA graph) serves every step.
  // The mean mode runs on a second stream beside the mode kernel (they touch
  // disjoint data); both read the counter before it advances.
  // after_modes: recorded on the stream right after the mode kernel (the new
  // v and omega_y are final from then on), when given
  void enqueue_step(cudaEvent_t after_modes = nullptr);
  void step_begin();   // the mean mode forked beside the mode kernel
  void step_finish();  // join, counter, Lamb vector, nonlinear source
  void stage_modes();
  bool modes_sparse() const { return sparse_v && !force_dense; }
  owt::ModeArgs mode_args() const;
  void stage_mean(bool pre_advance = false, cudaStream_t s = nullptr);
  owt::MeanArgs mean_args(bool pre_advance) const;

  void run_steps(int64_t n);
  int64_t per_step_launches = 0;
  bool force_dense = false;  // testing aid: always sweep the full band
  bool fft_stockham = false; // FP32 transforms: shared-memory Stockham kernels instead of register ones
  bool mean_split = true;    // mixed precision: the mean-flow terms of the Lamb vector mode by mode beside the transforms
  int host_chunks = 0;       // owt_time_integration_host: chunks of modes (0: the default)
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
  void ensure_tuned();
  void autotune_modes();

  void drop_graph();

  // DY2 v for history levels whose v was replaced from the host (one launch).
  void recompute_dirty_q(cudaStream_t on = nullptr);  // on: another stream than the handle's

  void copy_ring(double2 *ring, size_t n, int from, int to);
  // column of mode 0 of a device-layout field -> contiguous NY vector
  void mode0_column(double2 *dst, const double2 *field);

  void get_vor_from_vel();
  void lamb_vec(bool explicit_shift);
  void nonlinear_source(bool record_mean);
  void friction(int shift);

  void init_prologue();
  void init_fields(const double *hu, const double *hv, const double *hw);
  // The seeded laminar + random divergence-free state, generated on the
  // device (seeded_ic.cu); the Chebyshev coefficients live in the transform
  // buffer zbuf and omega_y in tmpC until the velocity is complete.
  void init_seeded(uint64_t seed, double rms);
  void init_from_velocity();

  // ---- host <-> device in the reference layout ---------------------------------
  void to_device(const double *host, double2 *dst);
  void to_host(const double2 *src, double *host);
  double2 *field_ptr(int f, bool for_write);
  // The reference's stand-alone dealiased transforms of one field, FP64:
  // spectral [z][x][y] complex128 <-> physical [z][x][y] doubles on the 3/2
  // grid (src/FFT.cpp:49-194); temporary device buffers for the physical field.
  void fourier2physical(const double *spec, double *phys);
  // One step on a state held by the caller on the host (owt_time_integration_host):
  // 12 history fields, 12 mean vectors, 6 friction values in; new v, omega_y
  // and the friction histories out; copies overlapped with the device work.
  struct HostStep {
    bool ready = false;
    // H2D copies; layout transposes (high priority); DY2 v; D2H transposes
    // and copies (high priority)
    cudaStream_t up = nullptr, tx = nullptr, aux = nullptr, down = nullptr;
    // chunks of Fourier modes the uploads and the mode kernel pipeline over:
    // at most kChunks, kDefaultChunks unless set (two measured fastest at
    // 384x257x384, 6% ahead of one and of four; with eight the DY2 v
    // re-derivations compete with the mode kernel, 25% slower)
    static constexpr int kChunks = 8, kDefaultChunks = 2;
    double2 *stage[12] = {}, *dstage[2] = {nullptr, nullptr};
    // pinned host staging of the six friction values in and out, so that
    // their copies are asynchronous like the uploads around them
    double *fric_pin = nullptr;
    cudaEvent_t landed[kChunks] = {}, v_done[kChunks] = {}, q_done[kChunks] = {}, tx_done[kChunks] = {};
    cudaEvent_t up_done = nullptr, after_modes = nullptr, down_done = nullptr;
  } hs;
  void host_step_prepare();
  void step_host(const double *const *hist, const double *means, const double *fric, double *v_out, double *g_out,
                 double *fric_out);
  void physical2fourier(const double *phys, double *spec);
  double2 *mean_ptr(int which);
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

  void free_owned(void *q);
  void d2d(void *dst, const void *src, size_t bytes);
  size_t image_values() const { return 15 * fs + 12 * (size_t)NY + 3; }
  // full state: the five 3-slot rings, the four mean rings, the friction rings
  void save_image(double2 *img, int64_t &step_out);
  void load_image(const double2 *img, int64_t step);

  double drag_forward(int64_t n, int64_t interval);

  void adj_alloc();

  void adjoint_step(const double2 *tp, double wgt);

  void drag_backward(double gJ, double *grad_bottom, double *grad_top);

  void sync_and_check();
};

namespace owt {

// Run f for a C entry point on handle h: status code and h's message.
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

}  // namespace owt

/*
 * owt_gpu.h -- C ABI of the GB300 channel-DNS time step.
 *
 * Drop-in boundary for the reference solver's per-step entry points.  The
 * reference keeps its state in C++ inline globals (src/setup.hpp:22-79) and
 * exposes free functions (src/setup.hpp:84-114) called from its driver loop
 * (src/main.cpp:63-87).  This library keeps the same state on one GPU behind an
 * opaque handle; every function below names the reference routine or global it
 * replaces.  Only plain pointers, sizes and integers cross this interface.
 *
 * Conventions
 *  - Host arrays are in the reference Field layout [z][x][y] (src/linalg.hpp:
 *    695-745): NZ * (NX/2) * NY complex values, complex128 stored as
 *    interleaved (re, im) doubles.  Mean-mode vectors are NY complex128.
 *  - Every call returns an int status: OWT_OK (0) on success.  On failure
 *    owt_last_error() returns a message (the reference throws
 *    std::runtime_error in the same places, src/linalg.hpp:519,643).
 *  - The caller owns host buffers; the library owns device memory and its
 *    CUDA stream.  Calls on one handle must not overlap (the reference is
 *    single-threaded per rank); separate handles are independent.
 *  - Get/set calls are synchronous: when they return, the host buffer has
 *    been read or written.
 */
#ifndef OWT_GPU_H
#define OWT_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define OWT_OK 0
#define OWT_ERR_INVALID 1   /* bad argument or size (src/parallel.cpp:40-44 analogue) */
#define OWT_ERR_CUDA 2      /* CUDA runtime error */
#define OWT_ERR_NUMERIC 3   /* singular factorization or non-finite state */
#define OWT_ERR_STATE 4     /* call made in the wrong order */
#define OWT_ERR_NOMEM 5     /* device allocation failed */

/* arithmetic of the x/z transforms and physical-space products */
#define OWT_PREC_FP64 0     /* everything in FP64, as the reference */
#define OWT_PREC_MIXED 1    /* transforms + products in FP32; solves, factors,
                               mean mode and friction stay FP64 */

typedef struct owt_handle owt_handle;

/* Case parameters: the TOML keys read by load_params (src/IO.cpp:14-25).
 * PX, PZ, NT and save_interval concern the driver, not the step. */
typedef struct owt_params {
  double dt;          /* time step */
  double dkx, dkz;    /* fundamental wavenumbers: Lx = 2 pi/dkx, Lz = 2 pi/dkz */
  double alpha_mesh;  /* tanh stretching factor, y = tanh(alpha s)/tanh(alpha) */
  double nu;          /* kinematic viscosity */
  int64_t NX, NY, NZ; /* modes: NX/2 kx, NZ kz, NY wall-normal points */
  int32_t precision;  /* OWT_PREC_FP64 or OWT_PREC_MIXED */
  int32_t device;     /* CUDA device ordinal */
  /* Interior order of the compact finite differences.  0 or 8: the
   * reference's schemes (src/compdiff.hpp, 8th order for D1-D3, 6th for D4);
   * 6: sixth-order tridiagonal interior schemes for D1-D3 (D4 and every
   * boundary closure unchanged).  Zero-initialising the struct selects the
   * reference's operators. */
  int32_t fd_order;
} owt_params;

/* Spectral fields, the reference globals of the same names
 * (src/setup.hpp:58-67).  On the device vely/vory/Hv/Hg share storage with
 * vely_0/vory_0/Hv_0/Hg_0: the reference makes them equal at the end of every
 * step (src/solver.cpp:612-626) and after init_fields (:383-397). */
enum owt_field {
  OWT_VELX = 0, OWT_VELY, OWT_VELZ,
  OWT_VORX, OWT_VORY, OWT_VORZ,
  OWT_LMBX, OWT_LMBY, OWT_LMBZ,
  OWT_HV, OWT_HG,
  OWT_VELY_0, OWT_VELY_1, OWT_VELY_2,
  OWT_VORY_0, OWT_VORY_1, OWT_VORY_2,
  OWT_HV_0, OWT_HV_1, OWT_HV_2,
  OWT_HG_0, OWT_HG_1, OWT_HG_2,
  OWT_NUM_FIELDS
};

/* Mean-mode history vectors (src/setup.hpp:68-71). */
enum owt_mean {
  OWT_LMBX_MEAN_0 = 0, OWT_LMBX_MEAN_1, OWT_LMBX_MEAN_2,
  OWT_LMBZ_MEAN_0, OWT_LMBZ_MEAN_1, OWT_LMBZ_MEAN_2,
  OWT_VELX_MEAN_0, OWT_VELX_MEAN_1, OWT_VELX_MEAN_2,
  OWT_VELZ_MEAN_0, OWT_VELZ_MEAN_1, OWT_VELZ_MEAN_2,
  OWT_NUM_MEANS
};

/* Individual reference routines, run on the handle's state (owt_call). */
enum owt_routine {
  OWT_CALL_GET_VOR_FROM_VEL = 0, /* src/solver.cpp:218-238 */
  OWT_CALL_LAMB_VEC,             /* src/solver.cpp:262-304 (incl. mean-Lamb history shift) */
  OWT_CALL_NONLINEAR_SOURCE,     /* src/solver.cpp:240-260 */
  OWT_CALL_SOLVE_FRICTION_FORCE, /* src/solver.cpp:306-327 */
  OWT_CALL_TIME_INTEGRATION      /* src/solver.cpp:541-627 */
};

/* Create a handle: replaces allocate_var + init_mat + init_fft
 * (src/solver.cpp:15-216, src/FFT.cpp:11-34).  Builds the grid, metric,
 * compact-FD operators and the per-mode banded factorizations on the device. */
int owt_create(const owt_params *params, owt_handle **out);

/* Free everything (cleanup_fft, src/FFT.cpp:36-47, and the field storage). */
int owt_destroy(owt_handle *h);

/* Message of the last failed call on h; h == NULL gives the calling thread's
 * last failure of a call that takes no handle (owt_create, owt_dy1_noalloc).
 * Never NULL. */
const char *owt_last_error(const owt_handle *h);

/* init_fields (src/solver.cpp:329-426) with a caller-given velocity field in
 * place of the reference's built-in laminar + TS-wave one: vorticity from
 * velocity, Lamb vector, sources, history levels all equal, friction, mean
 * histories.  velx/vely/velz: [z][x][y] complex128. */
int owt_init_fields(owt_handle *h, const double *velx, const double *vely, const double *velz);

/* init_fields with a seeded velocity generated on the device (no counterpart
 * in the reference, whose initial conditions are laminar, laminar + TS wave,
 * or a restart): laminar Poiseuille flow 1.5 (1 - y^2) plus a divergence-free
 * perturbation with complex Gaussian Chebyshev amplitudes (degree 5) under a
 * k^-2 spectrum, v, dv/dy and omega_y zero at the walls, scaled to RMS `rms`
 * (Parseval, trapezoidal in y).  Random numbers: Philox4x32-10 keyed by the
 * seed and counted per mode, so a seed gives the same field on every call. */
int owt_init_seeded(owt_handle *h, uint64_t seed, double rms);

/* time_Integration (src/solver.cpp:541-627), nsteps times. Asynchronous on
 * the handle's stream; errors found on the device surface at the next
 * synchronizing call. */
int owt_time_integration(owt_handle *h, int64_t nsteps);

/* time_Integration (src/solver.cpp:541-627) on a state the caller holds on
 * the host, as the reference keeps it in its globals: uploads the history
 * fields, runs one step, and returns the new v and omega_y and the friction
 * histories.  The handle's device state becomes that of the step.
 *  - hist: 12 arrays [z][x][y] complex128, in the order vely_0, vely_1,
 *    vely_2, vory_0, vory_1, vory_2, Hv_0, Hv_1, Hv_2, Hg_0, Hg_1, Hg_2
 *    (src/setup.hpp:64-67);
 *  - means: the 12 mean-mode history vectors in enum owt_mean order, NY
 *    complex128 each, consecutive;
 *  - fric: fx_fric_0..2, fz_fric_0..2;
 *  - vely, vory: out, the step's new v and omega_y, [z][x][y] complex128;
 *    fric_out: out, the friction histories after the step.
 * Copies overlap the device work: the twelve host-to-device copies run back
 * to back into staging buffers of their own (the first call allocates them:
 * 12 + 2 fields of device memory, kept by the handle), each field's layout
 * transpose follows its copy, the DY2 v history of the v levels is
 * re-derived while the other fields arrive, with a quad-mapping mode kernel
 * the copies are pipelined with it over chunks of Fourier modes
 * (OWT_OPT_HOST_CHUNKS), and v and omega_y travel back while the step's
 * transforms run.  History arrays in pinned (page-locked) host memory whose
 * addresses are 16-byte aligned are read by the GPU's own loads at the full
 * host-link rate; other arrays go through the copy engines (pageable memory
 * at a fraction of that rate).
 * Synchronous: when it returns, the outputs are written. */
int owt_time_integration_host(owt_handle *h, const double *const *hist, const double *means, const double *fric,
                              double *vely, double *vory, double *fric_out);

/* Run one reference routine on the current state (enum owt_routine). */
int owt_call(owt_handle *h, int routine);

/* Wait for all work on the handle; reports device-side numeric failures. */
int owt_synchronize(owt_handle *h);

/* Copy a spectral field (enum owt_field) between host [z][x][y] complex128
 * and the device. */
int owt_get_field(owt_handle *h, int field, double *host);
int owt_set_field(owt_handle *h, int field, const double *host);

/* Mean-mode histories (enum owt_mean): NY complex128. */
int owt_get_mean(owt_handle *h, int which, double *host);
int owt_set_mean(owt_handle *h, int which, const double *host);

/* Friction-force histories (src/setup.hpp:77-79):
 * out[0..2] = fx_fric_0..2, out[3..5] = fz_fric_0..2. */
int owt_get_friction(owt_handle *h, double *out6);
int owt_set_friction(owt_handle *h, const double *in6);

/* Select the transform precision (OWT_PREC_FP64 / OWT_PREC_MIXED). */
int owt_set_precision(owt_handle *h, int precision);

/* Capture one step in a CUDA graph and replay it in owt_time_integration
 * (on = 1), or launch kernel by kernel (on = 0, the default). */
int owt_use_graph(owt_handle *h, int on);

/* Step counter since owt_init_fields (id_step in src/setup.hpp:34). */
int owt_get_step(const owt_handle *h, int64_t *step);

/* The handle's CUDA stream (a cudaStream_t), for ordering external work. */
int owt_get_stream(const owt_handle *h, void **stream);

/* Kernel launches issued by the library since the handle was created. */
int owt_get_launch_count(const owt_handle *h, int64_t *count);

/* Wall-normal grid y (src/solver.cpp:76) and DYn applied along y to every mode
 * of a field: out = DYn * in for n = 1 or 2 (src/solver.cpp:182,193, applied as
 * in src/linalg.hpp:434-453).  Arrays in the [z][x][y] layout. */
int owt_get_grid(const owt_handle *h, double *y);
int owt_dy_apply(owt_handle *h, int order, const double *in, double *out);

/* Fourier2Physical_dealiased (src/FFT.cpp:49-128) and
 * Physical2Fourier_dealiased (src/FFT.cpp:130-194) of one field, in FP64
 * whatever the handle's precision, with the step's own transform kernels:
 * spec is [z][x][y] complex128 (NZ * NX/2 * NY values), phys is the
 * reference's Field<double> on the 3/2 grid, [z][x][y] with z in [0, 3NZ/2),
 * x in [0, 3NX/2): 3NZ/2 * 3NX/2 * NY doubles.  The Nyquist-z row is dropped
 * on the way to physical space and kept on the way back, kx = 0 enters
 * through its real part, the forward result is scaled by 1/(NX2 NZ2), as
 * the reference does.  The handle's state is not changed; a temporary device
 * buffer of two physical fields is allocated for the call. */
int owt_fourier2physical(owt_handle *h, const double *spec, double *phys);
int owt_physical2fourier(owt_handle *h, const double *phys, double *spec);

/* Batches of independent channels (no counterpart in the reference, which runs
 * one channel per MPI job).  A batch step is one CUDA graph launch in which
 * every kernel of the time step runs once over all channels (one launch per
 * group of up to 64 channels sharing the kernel's block shape); the mode
 * kernel, which holds every per-mode banded solve of every channel, is a
 * persistent launch whose resident blocks take work items from a counter.
 * owt_batch_create times every mode-kernel variant on the batch (the handles'
 * state is put back afterwards) and keeps the fastest; the report lists the
 * timings.  Handles keep their own state, sizes and parameters (uneven sizes
 * are fine) and must outlive the batch; all must be on one device and
 * initialised, each at most once.  While a handle is in a batch, step it
 * through the batch only; results are bitwise those of stepping it alone.
 * Launch counts: all kernels launched by the batch, and those of one step. */
typedef struct owt_batch owt_batch;
int owt_batch_create(owt_handle *const *handles, int count, owt_batch **out);
int owt_batch_step(owt_batch *b, int64_t nsteps);
int owt_batch_synchronize(owt_batch *b);
int owt_batch_get_stream(const owt_batch *b, void **stream);
int owt_batch_get_launch_count(const owt_batch *b, int64_t *count);
int owt_batch_get_step_launches(const owt_batch *b, int64_t *count);
const char *owt_batch_tuning_report(const owt_batch *b);
int owt_batch_destroy(owt_batch *b);

/* Wall-normal statistics of the current velocity (no counterpart in the
 * reference, which computes none).  out[q * NY + j] for q = 0..6:
 * mean U, V, W (real parts of the (0,0) modes), RMS of u', v', w', and the
 * Reynolds shear stress <u'v'>, all as averages over x and z of the physical
 * fields the transforms produce (Parseval: kx > 0 modes count twice, the
 * kx = 0 column through its Hermitian part, the Nyquist kz row not at all). */
int owt_statistics(owt_handle *h, double *out7ny);

/* Full-state checkpoint for an exact restart (the reference has none,
 * README.md:11; its snapshots hold u, v, w only).  The image holds the
 * parameters, the step counter, every history level (v, omega_y, Hv, Hg and
 * the DY2 v history), the current u, w, omega_x, omega_z and Lamb vector, the
 * mean-mode and friction histories, in the device layout.  Restoring it and
 * stepping reproduces the uninterrupted run bit for bit. */
int owt_checkpoint_bytes(const owt_handle *h, int64_t *bytes);
int owt_checkpoint_save(owt_handle *h, void *host, int64_t bytes);
int owt_checkpoint_load(owt_handle *h, const void *host, int64_t bytes);

/* Keep a copy of the full state in device memory (one slot per handle, about
 * 15 fields) and return to it later: restart without a host round trip, e.g.
 * to repeat a run from the same state.  The step counter is restored too. */
int owt_state_keep(owt_handle *h);
int owt_state_restore(owt_handle *h);

/* Options and introspection (no counterpart in the reference).
 * OWT_OPT_FORCE_DENSE_BANDS: 1 = sweep the full band of the v-system in every
 *   column instead of skipping structurally-zero interior entries (the two
 *   give the same result; this exists to test that).
 * OWT_OPT_FFT_STOCKHAM: 1 = the mixed precision's FP32 transforms use the
 *   shared-memory Stockham kernels (one pass per radix-2/3/4/5 stage) even
 *   where register-transform kernels exist for the line length (the two
 *   agree to FP32 rounding; this exists to compare them).
 * OWT_OPT_MEAN_SPLIT: mixed precision only; 1 (the default) = the FP32
 *   transforms carry the fluctuations, and the mean-flow terms of the Lamb
 *   vector (mean velocity x fluctuating vorticity and back) are formed mode
 *   by mode beside them in FP32, each with a rounding of its own size (not of
 *   the largest value of a transformed plane); 0 = the FP32 transforms carry
 *   the whole fields.
 * OWT_OPT_HOST_CHUNKS: owt_time_integration_host pipelines its uploads with
 *   the mode kernel over this many chunks of Fourier modes (1 .. 8; 0 = the
 *   default, 2) when the mode kernel in use maps threads by quads.
 * OWT_INFO_SPARSE_SOLVE: 1 if the interior-sparse v-system solve is active.
 * OWT_INFO_PATTERN_VIOLATIONS: modes whose factors fell outside the sparse
 *   pattern at setup (any such mode selects the full-band solve).
 * OWT_INFO_DEVICE_BYTES: device memory held by the handle.
 * Autotuning: owt_create times every variant of the mode kernel (thread
 * mapping, block shape, register budget; bitwise-identical results) and keeps
 * the fastest.  OWT_INFO_MODES_VARIANT is the variant in use,
 * OWT_INFO_MODES_VARIANTS their number, OWT_OPT_MODES_VARIANT forces one
 * (-1 returns to the tuned choice), owt_tuning_report() lists the timings. */
#define OWT_OPT_FORCE_DENSE_BANDS 1
#define OWT_OPT_MODES_VARIANT 2
#define OWT_OPT_FFT_STOCKHAM 3
#define OWT_OPT_MEAN_SPLIT 4
#define OWT_OPT_HOST_CHUNKS 5
#define OWT_INFO_SPARSE_SOLVE 1
#define OWT_INFO_PATTERN_VIOLATIONS 2
#define OWT_INFO_DEVICE_BYTES 3
#define OWT_INFO_MODES_VARIANT 4
#define OWT_INFO_MODES_VARIANTS 5
int owt_set_option(owt_handle *h, int option, int64_t value);
int owt_get_info(const owt_handle *h, int what, int64_t *value);
const char *owt_tuning_report(const owt_handle *h);
/* Wall time of owt_create's phases (host operators, band factorizations,
 * pattern check, fields and tables, mode-kernel autotune), as text. */
const char *owt_setup_report(const owt_handle *h);

/* Testing aid: factor U random band systems (kl/ku as the library's: 15/13,
 * 6/6, 2/2) of n columns with both factorization kernels (thread per system;
 * warp per system, used when a channel has few modes), count the entries of
 * the factors, pivots and row scales that differ bitwise, and time each. */
int owt_band_factor_selftest(int kl, int ku, int n, int U, uint64_t seed, int64_t *mismatches, float *ms_thread,
                             float *ms_warp);

/* Testing aid, no counterpart in the reference: the FP64 -> FP32 conversion
 * of the mixed precision's mean-flow terms (integer instructions, instead of
 * the hardware conversion on the FP64 pipe) against the hardware's, on n
 * samples (edge values, then seeded random bit patterns).  counts[4]: results
 * equal to the hardware's round to nearest even; ties rounded away from zero
 * instead; subnormal results flushed to zero; any other result. */
int owt_convert_selftest(int64_t n, uint64_t seed, int64_t *counts);

/* Measurement aid, no counterpart in the reference: enqueue one stage of the
 * step on the handle's stream without advancing the step counter, so a caller
 * can time it with CUDA events on that stream.  The stage overwrites the
 * state it would produce in a step (use a handle whose state is disposable).
 *   0: mode kernel (RHS assembly, both implicit solves, solve_horizontal)
 *   1: mean mode (solve_mean + friction)
 *   2: transforms + products (Lamb vector, three kernels)
 *   3: nonlinear source
 *   4, 5, 6: the three transform kernels alone (z backward, x pass with the
 *            products, z forward)
 *   7: the mean-flow terms of the mixed-precision Lamb vector (FP32, mode by
 *      mode; nothing in FP64) */
#define OWT_STAGE_MODES 0
#define OWT_STAGE_MEAN 1
#define OWT_STAGE_LAMB 2
#define OWT_STAGE_NONLINEAR 3
#define OWT_STAGE_ZBACK 4
#define OWT_STAGE_XLAMB 5
#define OWT_STAGE_ZFWD 6
#define OWT_STAGE_MEAN_LAMB 7 /* mixed precision: the mean-flow terms of the Lamb vector */
int owt_enqueue_stage(owt_handle *h, int stage);

/* Wall blowing/suction.  The reference imposes v = 0 on both walls through
 * the boundary rows of the v-system (src/solver.cpp:581-596, source_v[0] and
 * source_v[NY-1] set to zero); these calls put prescribed values there
 * instead: v(y = -1) = vw_bottom, v(y = +1) = vw_top, each a spectral wall
 * field of NZ * NX/2 complex128 values (interleaved re, im) in the layout of
 * one y-line set of a Field, [kz index][kx index].  Mode (0, 0) should be zero
 * (no net mass flux).  Both NULL restores no-slip.  get returns zeros when
 * no wall velocity is set. */
int owt_set_wall_velocity(owt_handle *h, const double *vw_bottom, const double *vw_top);
int owt_get_wall_velocity(owt_handle *h, double *vw_bottom, double *vw_top);

/* Wall-drag objective and its discrete adjoint (no counterpart in the
 * reference).  J = (1/N) sum_{n=1..N} fx_n, the driving force fx of each of
 * N steps (solve_friction_force, src/solver.cpp:306-312), which is the wall
 * shear stress averaged over both walls.
 *  - owt_drag_forward runs N steps from the current state (as
 *    owt_time_integration would), keeping a device image of the full state
 *    every `interval` steps, and returns J.  FP64 precision only.
 *  - owt_drag_backward gives grad_objective * dJ/d(vw) for the wall velocity
 *    in force during the forward run, as d/dRe + i d/dIm per mode, same
 *    layout as owt_set_wall_velocity.  It recomputes each segment of
 *    `interval` steps from its image and runs the adjoint step kernels
 *    backwards through it; afterwards the state is again the state after the
 *    forward run.  OWT_ERR_STATE if the state or the wall velocity changed
 *    since owt_drag_forward.
 * Device memory: (N/interval + 1) state images of ~15 fields each, a tape of
 * 6 * interval fields, and ~45 fields of adjoint state and scratch. */
int owt_drag_forward(owt_handle *h, int64_t nsteps, int64_t interval, double *objective);
int owt_drag_backward(owt_handle *h, double grad_objective, double *grad_bottom, double *grad_top);

/* DY1 along y for device arrays the caller owns, allocating no device memory.
 * No counterpart in the reference: it is the compact first derivative of
 * owt_dy_apply (order 1), out = diag(c11) A1^-1 B1 in, for callers that cannot
 * call cudaMalloc: programs whose own pool allocator owns the device memory
 * and forbids allocations from elsewhere, and loops that cannot accept the
 * implicit device-wide synchronisation of cudaMalloc/cudaFree.  It needs no
 * handle (creating one allocates).
 *  - d_in, d_out: device pointers, 16-byte aligned, NY * nlines complex128
 *    (interleaved), line index fastest: [y][line] (a whole field in the
 *    library's device layout is nlines = NZ * NX/2).
 *  - Grid: y = tanh(alpha_mesh s)/tanh(alpha_mesh), NY points.
 *  - Scratch: a file-scope static device array of 256 KiB + 2 *
 *    OWT_NOALLOC_MAX_VALUES * 16 bytes (32.25 MiB), held on every GPU that
 *    loads the library until the process exits.  Requests beyond NY <=
 *    OWT_NOALLOC_MAX_NY or NY * nlines <= OWT_NOALLOC_MAX_VALUES are rejected
 *    with OWT_ERR_INVALID and a message in owt_last_error(NULL).
 *  - The first call on a device looks up that array's device address (once
 *    per device, with the device current) and keeps it; make that first call
 *    before any stream capture, and do not use the entry point across a
 *    cudaDeviceReset, which invalidates the kept address.
 *  - Every call rebuilds the operator tables it reads (then the scratch) for
 *    its own (NY, alpha_mesh) before using them; calls share the one array,
 *    so calls that can overlap on the GPU (different streams without
 *    ordering between them) race and give wrong results.
 *  - Asynchronous on `stream` (a cudaStream_t, NULL for the legacy default
 *    stream); errors of the launch are returned, device-side ones appear at
 *    the caller's next synchronisation. */
#define OWT_NOALLOC_MAX_NY 1025
#define OWT_NOALLOC_MAX_VALUES (1 << 20)
int owt_dy1_noalloc(int64_t NY, int64_t nlines, double alpha_mesh, const double *d_in, double *d_out,
                    void *stream);

#ifdef __cplusplus
}
#endif

#endif /* OWT_GPU_H */

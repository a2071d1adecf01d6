// Argument blocks and launchers of the per-mode kernels (solve.cu) and the
// transform kernels (transforms.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "batch.cuh"
#include "owt_device.cuh"

namespace owt {

// The dynamic shared-memory limit is an attribute of the kernel function on
// the current device, shared by every handle of the process.  Raise it to
// what a handle needs, never lower it: a smaller channel created after a
// larger one must not break the larger one's launches.
inline std::mutex &smem_attr_mutex() {
  static std::mutex mu;
  return mu;
}
template <typename F>
inline cudaError_t raise_smem_limit(F *func, size_t bytes) {
  std::lock_guard<std::mutex> lk(smem_attr_mutex());
  cudaFuncAttributes at;
  cudaError_t e = cudaFuncGetAttributes(&at, func);
  if (e != cudaSuccess) return e;
  if ((size_t)at.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
  return cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

struct ModeArgs {
  int NY, NZ, NXH, NZH, M, U;
  int u0, u1;  // quad mapping: unique modes u0 <= u < u1 only (0, U: all)
  double inv_dt, nu;
  const double *kx, *kz;
  double2 *v_ring, *g_ring, *hv_ring, *hg_ring, *q_ring;  // 3 slots each, [slot][y][mode]
  double2 *u_out, *w_out, *ox_out, *oz_out;
  const double *ab_v; const uint8_t *piv_v; int n_v;
  const double *ab_g; const uint8_t *piv_g; int n_g;
  const int *rhs_node_v;
  const int *rb_col; const double *rb_val;
  const double *inv_cg;
  const double *rs_v;   // inverse row scales [n][U]
  const double *rs_gi;  // inverse row scales of the omega_y-system times 1/cg of the mode [n][U]
  double2 *sg, *dg, *yv, *yg, *sv;  // scratch
  const long long *step;
  const double2 *vw;  // wall-normal velocity at the walls [2][M] (bottom, top), or null
  const int *rbv_col; const double *rbv_val;  // v-system rhs tables [n_v][4]
  // metric coefficients with the unscaling of the solved h d1, h^2 d2:
  // c11/h, c21/h, c22/h^2, nu c21/h, nu c22/h^2 [NY]
  const double *c11h, *c21h, *c22h, *nc21h, *nc22h;
};

struct MeanArgs {
  int NY, M, U, n_g;
  double inv_dt, nu, Ly, inv_cg0;
  const double *c11, *c21, *c22;
  const double *ab_g; const uint8_t *piv_g;
  const int *rb_col; const double *rb_val;
  const double *rs_g;
  double inv_h, inv_h2;
  double2 *U_ring, *W_ring, *lx_ring, *lz_ring;  // [3][NY]
  double *fx_ring, *fz_ring;                     // [3]
  double2 *u_field, *w_field, *ox_field, *oz_field;
  double2 *scratch;  // 2*NY + 2*n_g
  double2 *dy1;      // 2*NY
  const long long *step;
  int *err;
  int pre_advance;   // 1: launched before the step counter advances (concurrently with the mode kernel)
};

struct NLArgs {
  int NY, NZ, NXH, M;
  const double *kx, *kz, *c11;
  const double2 *lx, *ly, *lz;
  double2 *hv_ring, *hg_ring;
  const double *ab1; const uint8_t *piv1;
  const int *b1_col; const double *b1_val;
  double2 *fscr, *yscr;        // B1 operand and forward-sweep scratch [NY][M] each
  double2 *lx_mean, *lz_mean;  // rings [3][NY], or null
  const long long *step;
};

struct DApplyArgs {
  int NY, M;
  const double2 *in;
  double2 *out;
  const double *ab; const uint8_t *piv;
  const int *b_col; const double *b_val;
  double2 *bf, *yscr;
};

struct DY2Args {
  int NY, M, nf;  // nf fields (at most 3)
  int m0, mcount; // modes m0 .. m0 + mcount - 1 (0, M: all)
  const double2 *in[3];
  double2 *out[3], *scr[3];  // scr: one field of scratch each
  const double *ab1, *ab2; const uint8_t *piv1, *piv2;
  const int *b1_col, *b2_col; const double *b1_val, *b2_val;
  const double *c21, *c22;
};

struct VorArgs {
  int NY, NXH, M;
  const double *kx, *kz, *c11;
  const double2 *u, *v, *w, *d1u, *d1w;
  double2 *ox, *oy, *oz;
};

// Transform kernels: inputs for the inverse pass are six spectral fields
// (u, v, w, omega_x, omega_y, omega_z) in device layout; outputs three.
struct XformDims {
  int NY, NZ, NXH, NZH, NX2, NZ2;
};
struct XformArgs {
  XformDims d;
  // in[f] is a plain field, or (bit f of ring_mask set) the base of a
  // three-slot ring whose level-0 slot is chosen from the step counter.
  const double2 *in[6];
  int ring_mask;
  size_t fs;
  const long long *step;
  // mixed precision (FP32 transforms only): transform only the fluctuations
  // (mode (0,0) left out); k_mean_lamb writes the mean-flow interaction terms
  // (formed mode by mode, mean_flow.cuh) to lm and the z forward adds them
  int mean_split;
  float2 *lm[3];  // [NY][M] each
  double2 *out[3];
  void *zbuf;  // [6][NY][NZ2][NXH] complex<T>
  void *lbuf;  // [3][NY][NZ2][NXH] complex<T>
  FftPlan px, pz;
  const void *twx, *twz;  // tables of exp(-2 pi i k/L) in T precision
  double inv_nx2, inv_nz2;
  int stockham;  // FP32: 1 = the shared-memory Stockham kernels even where register ones exist
};

bool band_supported(int kl, int ku);
// d2f_bits against the hardware conversion on n samples (counts: see
// k_convert_check); 0 on success.
int convert_selftest(long long n, uint64_t seed, long long counts[4]);
int band_factor_selftest(int kl, int ku, int n, int U, uint64_t seed, long long *mismatches, float *ms_thread,
                         float *ms_warp);
// Band LU of U systems (dgbtf2 order, row equilibration when rscale is given).
// kernel: 1 thread per system, 2 one warp per system, 0 chosen by U.
constexpr int kBandFactorWarpBelow = 32768;
void launch_band_factor(int kl, int ku, double *ab, uint8_t *piv, int n, int U, const double *t0, const double *t1,
                        const double *t2, const double *s1, const double *s2, double *rscale, int *info,
                        cudaStream_t st, int kernel = 0);
void launch_modes(const ModeArgs &a, int klv, int kuv, int klg, int kug, bool sparse, int variant, cudaStream_t st);
int modes_pair_count();  // variants below this index use the pair mapping, the others the quad mapping
void launch_modes_sixth(const ModeArgs &a, cudaStream_t st);  // masked solve with the sixth-order fill
// dst[p U + u] = scale[u] src[p U + u], p < n
void launch_scale_by_mode(double *dst, const double *src, const double *scale, int n, int U, cudaStream_t st);
int modes_variant_count();        // single-channel launches: pair, quad, split mappings
int modes_batch_variant_count();  // batched launches: pair and quad mappings
bool modes_variant_is_quad(int v);
const char *modes_variant_name(int v);
void launch_check_pattern(int which, const double *ab, const uint8_t *piv, int n, int U, int *bad,
                          cudaStream_t st);
void launch_advance(long long *step, cudaStream_t st);
void launch_mean(const MeanArgs &a, bool smem, cudaStream_t st);
bool mean_prepare(int NY, int n_g);
void launch_nl(const NLArgs &a, cudaStream_t st);
void launch_dapply(const DApplyArgs &a, cudaStream_t st);
void launch_dy2(const DY2Args &a, cudaStream_t st);
void launch_combine_y(double2 *out, const double2 *A, const double *ca, const double2 *B, const double *cb, int NY,
                      int M, cudaStream_t st);
void launch_vor(const VorArgs &a, cudaStream_t st);
void launch_friction(const double2 *d1u, const double2 *d1w, const double *c11, int NY, int M, double nu, double Ly,
                     double *fx_ring, double *fz_ring, const long long *step, int shift, int *err, cudaStream_t st);
void launch_lamb_mean_shift(double2 *lx_ring, double2 *lz_ring, const double2 *lx, const double2 *lz, int NY, int M,
                            const long long *step, cudaStream_t st);
void launch_transpose(const double2 *in, double2 *out, int rows, int cols, cudaStream_t st);
// the same with the output rows ldo values apart: out[c * ldo + r] = in[r * cols + c]
void launch_transpose_ld(const double2 *in, double2 *out, int rows, int cols, int ldo, cudaStream_t st);
// the same for a rows x cols matrix of doubles
void launch_transpose_real(const double *in, double *out, int rows, int cols, cudaStream_t st);
// bytes (a multiple of 16) from device-addressable host memory, both
// addresses 16-byte aligned, copied by SM loads
void launch_host_load(const void *src, void *dst, size_t bytes, cudaStream_t st);
void launch_stats(const double2 *u, const double2 *v, const double2 *w, int NY, int NZ, int NXH, double *out,
                  cudaStream_t st);

// Lamb vector: z-backward (6 fields) -> x pass with products -> z-forward (3),
// in mixed precision with the FP64 mean-flow terms (part 3) before the z
// forward.  precision 0: FP64, 1: FP32 transforms and products.  Returns
// launches issued.
int launch_lamb(const XformArgs &a, int precision, cudaStream_t st);
cudaError_t lamb_prepare(const XformDims &d);
void launch_lamb_part(const XformArgs &a, int precision, int part, cudaStream_t st);
size_t lamb_zbuf_bytes(const XformDims &d, int precision);
// FP32 transform kernels with register-resident line transforms
// (transforms_reg.cu) for one line length: ok = false when the length has no
// two-pass factorisation there (the shared-memory Stockham kernels serve it).
struct RegXformKernels {
  bool ok = false;
  void (*zback)(XformArgs) = nullptr, (*xlamb)(XformArgs) = nullptr, (*zfwd)(XformArgs) = nullptr;
  void (*zback_b)(BatchTable<XformArgs>) = nullptr, (*xlamb_b)(BatchTable<XformArgs>) = nullptr,
      (*zfwd_b)(BatchTable<XformArgs>) = nullptr;
  int zthreads = 0, xthreads = 0, xlines = 0;  // xlines: (y, z) lines per x group
  int xgrid = 0;  // the x pass is persistent: launch at most this many blocks (the resident ones)
  size_t zsmem = 0, xsmem = 0;
};
RegXformKernels reg_xform_kernels(int L);
// Stand-alone FP64 dealiased transforms of one field (zbuf / lbuf field 0 in
// between): a.in[0] -> phys [y][z][x], and phys -> a.out[0].
cudaError_t phys_prepare(const XformDims &d);
void launch_fourier2physical(const XformArgs &a, double *phys, cudaStream_t st);
void launch_physical2fourier(const XformArgs &a, const double *phys, cudaStream_t st);
size_t lamb_lbuf_bytes(const XformDims &d, int precision);

// Seeded initial condition (seeded_ic.cu): Chebyshev coefficients per mode
// from a counter-based generator, v and omega_y, then u, w and the RMS scaling.
struct SeedArgs {
  int NY, NZ, NXH, NZH, M, degree;
  uint64_t seed;
  double kmin;
  const double *kx, *kz, *y, *c11, *wy;  // wy: trapezoidal weights in y, summing to 1
  double2 *coef;                          // [M][2][degree + 1]
};
size_t ic_coef_values(int M, int degree);
size_t ic_partial_values();
int launch_ic_fields(const SeedArgs &a, double2 *v, double2 *g, cudaStream_t st);
int launch_ic_velocity(const SeedArgs &a, const double2 *d1v_raw, const double2 *g, double2 *u, double2 *v,
                       double2 *w, double *partial, double rms, cudaStream_t st);

// Batch tables travel as kernel parameters, which are limited to 32764 bytes.
static_assert(sizeof(BatchTable<ModeArgs>) <= 32764, "mode-kernel batch table exceeds the kernel parameter limit");
static_assert(sizeof(BatchTable<XformArgs>) <= 32764, "transform batch table exceeds the kernel parameter limit");
static_assert(sizeof(BatchTable<MeanArgs>) <= 32764, "mean-mode batch table exceeds the kernel parameter limit");
static_assert(sizeof(BatchTable<NLArgs>) <= 32764, "nonlinear batch table exceeds the kernel parameter limit");

// Batched launches (one launch per kernel over the channels of a table).
// Mode kernel: work items of `block` threads, a persistent grid of resident
// blocks taking items from the counter pair `work` (zero before the first
// launch; each launch leaves it zero).  variant -1 is the full-band solve.
struct ModeBatchShape {
  int block;  // threads per work item
  bool quad;  // 4 threads per unique mode (else 2 per mode)
  int grid;   // resident blocks on the device
};
ModeBatchShape modes_batch_shape(int variant);
void launch_modes_batch(const BatchTable<ModeArgs> &t, int variant, int *work, int grid, cudaStream_t st);
cudaError_t mean_batch_prepare(size_t smem_bytes);
size_t mean_smem_bytes(int NY, int n_g);
void launch_mean_batch(const BatchTable<MeanArgs> &t, bool smem, size_t smem_bytes, cudaStream_t st);
void launch_advance_batch(const StepCounters &c, cudaStream_t st);
int nl_batch_blocks(const NLArgs &a);
void launch_nl_batch(const BatchTable<NLArgs> &t, cudaStream_t st);
// Transforms: part 0 z backward, 1 x pass, 2 z forward, 3 mean-flow terms
// (mixed precision).  The channels of a table share the precision, NZ2 (parts
// 0, 2) or NX2 (part 1).
int lamb_batch_blocks(const XformDims &d, int precision, int part, bool stockham);
cudaError_t lamb_batch_prepare(const XformDims &d, int precision);
void launch_lamb_batch(const BatchTable<XformArgs> &t, int precision, int part, cudaStream_t st);

}  // namespace owt

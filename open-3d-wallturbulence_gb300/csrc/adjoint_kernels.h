// Argument blocks and launchers of the discrete-adjoint step (adjoint.cu).
//
// The adjoint step runs the forward step's launches backwards: nonlinear
// source, Lamb vector (three transform kernels), mean mode, mode kernel.  Its
// state is the adjoint of the forward state: for each of v, omega_y, Hv, Hg
// and the DY2 v history three levels, plus the mean-mode histories (U, W, the
// mean Lamb vector) and the friction forces.  Level 0 of every history is the
// adjoint of the value the forward step produced; the kernels consume it and
// leave behind, in the same three buffers, the adjoints of the levels the
// forward step read (the caller rotates the buffer roles after each step).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "owt_device.cuh"
#include "solve_kernels.h"

namespace owt {

// Adjoint of nonlinear_source and of the mean-Lamb-vector record.
struct AdjNLArgs {
  int NY, NXH, M;
  const double *kx, *kz, *c11;
  const double2 *hvb, *hgb;      // adjoints of the new Hv, Hg [NY][M]
  const double2 *lxmb, *lzmb;    // adjoints of the new mean Lamb vectors [NY]
  double2 *lxb, *lyb, *lzb;      // out: adjoint of the Lamb vector [NY][M]
  const double *ab1; const uint8_t *piv1;    // band LU of A_1 (one system)
  const int *b1t_col; const double *b1t_val;  // B_1 transposed, (row, val) x 8 per column
  double2 *ys, *ws;              // scratch [NY][M]
};

// Adjoint of the Lamb vector: inputs are the step's six spectral fields and
// the adjoint Lamb vector, outputs the adjoints of the six fields.
struct AdjXformArgs {
  XformDims d;
  const double2 *st[6];   // u, v, w, omega_x, omega_y, omega_z of the step
  const double2 *lb[3];   // adjoint Lamb vector
  double2 *out[6];        // adjoints of u, v, w, omega_x, omega_y, omega_z
  double2 *zbuf;          // [9][NY][NZ2][NXH]
  double2 *lbuf;          // [6][NY][NZ2][NXH]
  FftPlan px, pz;
  const double2 *twx, *twz;
  double inv_n;           // 1 / (NX2 NZ2)
};

// Adjoint of solve_mean + solve_friction_force.
struct AdjMeanArgs {
  int NY, M, U, n_g;
  double inv_dt, nu, Ly, inv_cg0, inv_h, inv_h2;
  double weight;          // d objective / d fx of this step
  const double *c11, *c21, *c22;
  const double *ab_g; const uint8_t *piv_g; const int *rb_col; const double *rb_val; const double *rs_g;
  const double2 *ub, *wb, *oxb, *ozb;   // adjoint fields; the mean mode is column 0
  double2 *Ub[3], *Wb[3], *Lxb[3], *Lzb[3];  // [NY] each
  double *fxb[3], *fzb[3];
  double2 *scratch;       // 2 (3 NY + n_g)
};

// Adjoint of the mode kernel (both implicit solves and solve_horizontal).
struct AdjModeArgs {
  int NY, NZ, NXH, NZH, M, U;
  double inv_dt, nu, inv_h, inv_h2;
  const double *kx, *kz, *c11, *c21, *c22, *inv_cg;
  const double *ab_v; const uint8_t *piv_v; int n_v; const int *rhs_node_v; const double *rs_v;
  const int *rbv_col; const double *rbv_val;  // v-system rhs tables [n_v][4]
  const double *ab_g; const uint8_t *piv_g; int n_g; const int *rb_col; const double *rb_val; const double *rs_g;
  const double2 *ub, *vb, *wb, *oxb, *gb, *ozb;  // adjoint fields from the Lamb vector
  double2 *v[3], *g[3], *hv[3], *hg[3], *q[3];   // adjoint histories [NY][M]
  double2 *grad;          // [2][M] accumulated d objective / d v_w (bottom, top)
  double2 *yv, *yg;       // scratch [n_v][M], [n_g][M]
  double2 *xv0, *xv1, *xv2, *xg0, *xg1, *sgb, *svb;  // scratch [NY][M]
};

void launch_adj_nl(const AdjNLArgs &a, cudaStream_t st);
cudaError_t adj_lamb_prepare(const XformDims &d);
void launch_adj_lamb(const AdjXformArgs &a, cudaStream_t st);  // three launches
void launch_adj_mean(const AdjMeanArgs &a, cudaStream_t st);
// vmode: 0 full band, 1 / 2 the v-system's transposed solve inside the
// eighth- / sixth-order interior masks (only where the setup check passed)
void launch_adj_modes(const AdjModeArgs &a, int vmode, cudaStream_t st);
void launch_objective_add(const double *fx_ring, const long long *step, double weight, double *acc,
                          cudaStream_t st);
size_t adj_zbuf_values(const XformDims &d);
size_t adj_lbuf_values(const XformDims &d);

}  // namespace owt

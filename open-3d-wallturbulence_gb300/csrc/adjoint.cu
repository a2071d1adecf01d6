// Discrete adjoint of the time step (src/solver.cpp:541-627 with wall
// blowing/suction in the v boundary rows), in FP64.
//
// The forward step is, per mode, linear in the state except for the Lamb
// vector.  Its adjoint runs the step's stages backwards with the transposes of
// the same discrete operators:
//
//  k_adj_nl     nonlinear_source^T: lambda_bar from Hv_bar, Hg_bar, with
//               DY1^T = B_1^T A_1^-T diag(c11) (transposed band solve);
//               the adjoint of the mean-Lamb-vector record joins mode (0, 0).
//  k_zback_adj  } Lamb_vec^T.  The forward map is  lambda = F((B u) x (B om))
//  k_xlamb_adj  } with B the dealiased inverse transform (Hermitian extension
//  k_zfwd_adj   } in x, z-Nyquist row dropped) and F the truncating forward
//               transform (normalised, z-Nyquist row kept).  With the real
//               inner product, F^T = (1/N) B' where B' is B with weight 1/2 on
//               kx > 0 and the Nyquist row kept, and B^T = N F' where F' is F
//               with weight 2 on kx > 0 and the Nyquist row dropped.  So
//                 u_bar  = B^T (om_p x lambda_bar_p)
//                 om_bar = B^T (lambda_bar_p x u_p),  lambda_bar_p = F^T lambda_bar
//               with u_p, om_p the step's physical fields recomputed from its
//               spectral fields (the recompute tape).
//  k_adj_mean   solve_mean^T + solve_friction_force^T (one block).
//  k_adj_modes  mode kernel^T: solve_horizontal^T, then transposed solves of
//               the augmented v- and omega_y-systems on the forward factors,
//               and the source assembly^T into the three history levels.  The
//               transposed v solve also yields d objective / d v_w from the
//               two wall rows; it skips the entries outside the interior
//               fill masks where the forward's masked solves apply.
#include <cuda_runtime.h>

#include "adjoint_kernels.h"
#include "owt_device.cuh"
#include "setup_host.h"

namespace owt {

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_adj_nl(AdjNLArgs a) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= a.M) return;
  const int M = a.M, NY = a.NY;
  const int k = m / a.NXH, i = m - k * a.NXH;
  const double kx = a.kx[i], kz = a.kz[k];
  const double k2 = kx * kx + kz * kz;
  // w = A_1^-T (c11 .* Hv_bar)
  auto rhs = [&](int p) -> double2 {
    const double2 h = a.hvb[(size_t)p * M + m];
    const double c = a.c11[p];
    return make_double2(c * h.x, c * h.y);
  };
  auto ys = [&](int p, double2 y) { a.ys[(size_t)p * M + m] = y; };
  auto yl = [&](int p) -> double2 { return a.ys[(size_t)p * M + m]; };
  auto out = [&](int c, double2 x) { a.ws[(size_t)c * M + m] = x; };
  band_solve_t<2, 2>(a.ab1, a.piv1, NY, 1, 0, rhs, ys, yl, out);
  for (int j = 0; j < NY; ++j) {
    // q = B_1^T w  (so that the adjoint of f = i kx lx + i kz lz is -q)
    double2 q = make_double2(0.0, 0.0);
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const double b = a.b1t_val[j * 8 + e];
      if (b != 0.0) {
        const double2 x = a.ws[(size_t)a.b1t_col[j * 8 + e] * M + m];
        q.x += b * x.x;
        q.y += b * x.y;
      }
    }
    const size_t at = (size_t)j * M + m;
    const double2 hg = a.hgb[at], hv = a.hvb[at];
    // lx_bar = -i kz Hg_bar + i kx q ; ly_bar = -k^2 Hv_bar ; lz_bar = i kx Hg_bar + i kz q
    double2 bx = make_double2(kz * hg.y - kx * q.y, -kz * hg.x + kx * q.x);
    double2 bz = make_double2(-kx * hg.y - kz * q.y, kx * hg.x + kz * q.x);
    if (m == 0) {
      bx.x += a.lxmb[j].x; bx.y += a.lxmb[j].y;
      bz.x += a.lzmb[j].x; bz.y += a.lzmb[j].y;
    }
    a.lxb[at] = bx;
    a.lyb[at] = make_double2(-k2 * hv.x, -k2 * hv.y);
    a.lzb[at] = bz;
  }
}

void launch_adj_nl(const AdjNLArgs &a, cudaStream_t st) {
  k_adj_nl<<<(a.M + 127) / 128, 128, 0, st>>>(a);
}

// ---------------------------------------------------------------------------
// Lamb vector adjoint.  Tile shapes as the FP64 forward transforms: ATX kx
// lines per z block, AP (y, z) lines per x block.
constexpr int ATX = 6, AP = 2, ANPAIR = 5;

// R5: the lines have a radix-5 stage (the butterfly is compiled in only then).
template <bool R5>
__global__ void __launch_bounds__(1024) k_zback_adj(AdjXformArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const XformDims d = a.d;
  const int ls = d.NZ2 + 1;
  double2 *bufa = reinterpret_cast<double2 *>(smraw);
  double2 *bufb = bufa + ATX * ls;
  const int i0 = blockIdx.x * ATX, j = blockIdx.y, f = blockIdx.z;
  const int M = d.NZ * d.NXH;
  const bool adj = f >= 6;  // fields 6..8: lambda_bar (F^T), else the step's fields (B)
  const double2 *src = (adj ? a.lb[f - 6] : a.st[f]) + (size_t)j * M;
  for (int idx = threadIdx.x; idx < ATX * ls; idx += blockDim.x) bufa[idx] = make_double2(0.0, 0.0);
  __syncthreads();
  for (int idx = threadIdx.x; idx < d.NZ * ATX; idx += blockDim.x) {
    const int kz = idx / ATX, c = idx - kz * ATX, i = i0 + c;
    if (i < d.NXH && (adj || kz != d.NZH)) {
      const int slot = kz < d.NZH ? kz : kz + d.NZH;
      double2 v = src[(size_t)kz * d.NXH + i];
      if (adj) {
        const double s = i == 0 ? a.inv_n : 0.5 * a.inv_n;
        v.x *= s;
        v.y *= s;
      }
      bufa[c * ls + slot] = v;
    }
  }
  __syncthreads();
  const double2 *r = fft_lines<double, true, R5>(bufa, bufb, ATX, ls, a.pz, a.twz);
  double2 *dst = a.zbuf + ((size_t)f * d.NY + j) * d.NZ2 * d.NXH;
  for (int idx = threadIdx.x; idx < d.NZ2 * ATX; idx += blockDim.x) {
    const int z = idx / ATX, c = idx - z * ATX;
    if (i0 + c < d.NXH) dst[(size_t)z * d.NXH + i0 + c] = r[c * ls + z];
  }
}

template <bool R5>
__global__ void __launch_bounds__(1024) k_xlamb_adj(AdjXformArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const XformDims d = a.d;
  const int ls = d.NX2 + 1;
  double2 *bufa = reinterpret_cast<double2 *>(smraw);
  double2 *bufb = bufa + ANPAIR * AP * ls;
  const size_t nlines = (size_t)d.NY * d.NZ2;
  const size_t line0 = (size_t)blockIdx.x * AP;
  const size_t fstride = nlines * d.NXH;
  // 1. pack (u,v) (w,ox) (oy,oz) (lbx,lby) (lbz,0) with the Hermitian extension
  for (int idx = threadIdx.x; idx < ANPAIR * AP * d.NX2; idx += blockDim.x) {
    const int q = idx / d.NX2, mm = idx - q * d.NX2;
    const int pair = q / AP, l = q - pair * AP;
    const size_t line = line0 + l;
    double2 z = make_double2(0.0, 0.0);
    if (line < nlines) {
      const double2 *A = a.zbuf + (size_t)(2 * pair) * fstride + line * d.NXH;
      const double2 *B = (2 * pair + 1 < 9) ? A + fstride : nullptr;
      if (mm == 0) {
        z = make_double2(A[0].x, B ? B[0].x : 0.0);
      } else if (mm < d.NXH) {
        const double2 x = A[mm], y = B ? B[mm] : make_double2(0.0, 0.0);
        z = make_double2(x.x - y.y, x.y + y.x);
      } else if (mm > d.NX2 - d.NXH) {
        const int mp = d.NX2 - mm;
        const double2 x = A[mp], y = B ? B[mp] : make_double2(0.0, 0.0);
        z = make_double2(x.x + y.y, y.x - x.y);
      }
    }
    bufa[q * ls + mm] = z;
  }
  __syncthreads();
  double2 *r = fft_lines<double, true, R5>(bufa, bufb, ANPAIR * AP, ls, a.px, a.twx);
  double2 *o = (r == bufa) ? bufb : bufa;
  // 2. u_bar = om x lb, om_bar = lb x u, packed (ub,vb) (wb,oxb) (oyb,ozb)
  for (int idx = threadIdx.x; idx < AP * d.NX2; idx += blockDim.x) {
    const int l = idx / d.NX2, x = idx - l * d.NX2;
    const double2 uv = r[(0 * AP + l) * ls + x], wox = r[(1 * AP + l) * ls + x], oyz = r[(2 * AP + l) * ls + x];
    const double2 bxy = r[(3 * AP + l) * ls + x], bz0 = r[(4 * AP + l) * ls + x];
    const double u = uv.x, v = uv.y, w = wox.x, ox = wox.y, oy = oyz.x, oz = oyz.y;
    const double bx = bxy.x, by = bxy.y, bz = bz0.x;
    o[(0 * AP + l) * ls + x] = make_double2(oy * bz - oz * by, oz * bx - ox * bz);
    o[(1 * AP + l) * ls + x] = make_double2(ox * by - oy * bx, by * w - bz * v);
    o[(2 * AP + l) * ls + x] = make_double2(bz * u - bx * w, bx * v - by * u);
  }
  __syncthreads();
  const double2 *fo = fft_lines<double, false, R5>(o, r, 3 * AP, ls, a.px, a.twx);
  // 3. unpack the real-pair spectra, keep kx < NXH, weight 1 (kx = 0) or 2
  for (int idx = threadIdx.x; idx < AP * d.NXH; idx += blockDim.x) {
    const int l = idx / d.NXH, mm = idx - l * d.NXH;
    const size_t line = line0 + l;
    if (line >= nlines) continue;
    const int mc = (mm == 0) ? 0 : d.NX2 - mm;
    const double hw = mm == 0 ? 0.5 : 1.0;
#pragma unroll
    for (int pair = 0; pair < 3; ++pair) {
      const double2 zm = fo[(pair * AP + l) * ls + mm], zc = fo[(pair * AP + l) * ls + mc];
      a.lbuf[(size_t)(2 * pair) * fstride + line * d.NXH + mm] =
          make_double2((zm.x + zc.x) * hw, (zm.y - zc.y) * hw);
      a.lbuf[(size_t)(2 * pair + 1) * fstride + line * d.NXH + mm] =
          make_double2((zm.y + zc.y) * hw, (zc.x - zm.x) * hw);
    }
  }
}

template <bool R5>
__global__ void __launch_bounds__(1024) k_zfwd_adj(AdjXformArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const XformDims d = a.d;
  const int ls = d.NZ2 + 1;
  double2 *bufa = reinterpret_cast<double2 *>(smraw);
  double2 *bufb = bufa + ATX * ls;
  const int i0 = blockIdx.x * ATX, j = blockIdx.y, f = blockIdx.z;
  const double2 *src = a.lbuf + ((size_t)f * d.NY + j) * d.NZ2 * d.NXH;
  for (int idx = threadIdx.x; idx < d.NZ2 * ATX; idx += blockDim.x) {
    const int z = idx / ATX, c = idx - z * ATX;
    bufa[c * ls + z] = (i0 + c < d.NXH) ? src[(size_t)z * d.NXH + i0 + c] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  const double2 *r = fft_lines<double, false, R5>(bufa, bufb, ATX, ls, a.pz, a.twz);
  double2 *dst = a.out[f] + (size_t)j * d.NZ * d.NXH;
  for (int idx = threadIdx.x; idx < d.NZ * ATX; idx += blockDim.x) {
    const int kz = idx / ATX, c = idx - kz * ATX;
    if (i0 + c < d.NXH) {
      const int slot = kz < d.NZH ? kz : kz + d.NZH;
      dst[(size_t)kz * d.NXH + i0 + c] = kz == d.NZH ? make_double2(0.0, 0.0) : r[c * ls + slot];
    }
  }
}

static size_t adj_smem_z(const XformDims &d) { return 2 * (size_t)ATX * (d.NZ2 + 1) * sizeof(double2); }
static size_t adj_smem_x(const XformDims &d) { return 2 * (size_t)ANPAIR * AP * (d.NX2 + 1) * sizeof(double2); }
size_t adj_zbuf_values(const XformDims &d) { return 9 * (size_t)d.NY * d.NZ2 * d.NXH; }
size_t adj_lbuf_values(const XformDims &d) { return 6 * (size_t)d.NY * d.NZ2 * d.NXH; }

// the instances for the channel's line lengths
struct AdjXformKernels {
  void (*zback)(AdjXformArgs), (*xlamb)(AdjXformArgs), (*zfwd)(AdjXformArgs);
};
static AdjXformKernels adj_kernels(const XformDims &d) {
  const bool z5 = d.NZ2 % 5 == 0, x5 = d.NX2 % 5 == 0;
  return {z5 ? k_zback_adj<true> : k_zback_adj<false>, x5 ? k_xlamb_adj<true> : k_xlamb_adj<false>,
          z5 ? k_zfwd_adj<true> : k_zfwd_adj<false>};
}

cudaError_t adj_lamb_prepare(const XformDims &d) {
  const AdjXformKernels k = adj_kernels(d);
  cudaError_t e = raise_smem_limit(k.zback, adj_smem_z(d));
  if (e == cudaSuccess) e = raise_smem_limit(k.zfwd, adj_smem_z(d));
  if (e == cudaSuccess) e = raise_smem_limit(k.xlamb, adj_smem_x(d));
  return e;
}

void launch_adj_lamb(const AdjXformArgs &a, cudaStream_t st) {
  const XformDims &d = a.d;
  const AdjXformKernels k = adj_kernels(d);
  dim3 gz((d.NXH + ATX - 1) / ATX, d.NY, 9);
  k.zback<<<gz, d.NZ2, adj_smem_z(d), st>>>(a);
  const size_t nl = (size_t)d.NY * d.NZ2;
  k.xlamb<<<(unsigned)((nl + AP - 1) / AP), d.NX2, adj_smem_x(d), st>>>(a);
  dim3 gf((d.NXH + ATX - 1) / ATX, d.NY, 6);
  k.zfwd<<<gf, d.NZ2, adj_smem_z(d), st>>>(a);
}

// ---------------------------------------------------------------------------
// Mean mode.  Thread 0: U (with fx), thread 1: W (with fz).  Forward:
//   s_j = sum_l beta_l (L_l,j + f_l) + sum_l alpha_l U_l,j / dt   (interior j)
//   U = solve(s) by the omega_y-system of mode (0, 0), dU = c11 d1
//   f = -nu/Ly (dU_NY-1 - dU_0).re ;  u(0,0) = U ;  om_z(0,0) = -dU
//   (W: om_x(0,0) = +dW)
// ---------------------------------------------------------------------------
__global__ void k_adj_mean(AdjMeanArgs a) {
  const int t = threadIdx.x;
  if (t >= 2) return;
  const int NY = a.NY, n = a.n_g, M = a.M;
  const double icg = a.inv_cg0, nu = a.nu;
  double2 *sc = a.scratch + (size_t)t * (3 * NY + n);
  double2 *ubar = sc, *dbar = sc + NY, *sb = sc + 2 * NY, *yy = sc + 3 * NY;
  double2 *X0 = t == 0 ? a.Ub[0] : a.Wb[0];
  double2 *X1 = t == 0 ? a.Ub[1] : a.Wb[1];
  double2 *X2 = t == 0 ? a.Ub[2] : a.Wb[2];
  double2 *L0 = t == 0 ? a.Lxb[0] : a.Lzb[0];
  double2 *L1 = t == 0 ? a.Lxb[1] : a.Lzb[1];
  double2 *L2 = t == 0 ? a.Lxb[2] : a.Lzb[2];
  double *F0 = t == 0 ? a.fxb[0] : a.fzb[0];
  double *F1 = t == 0 ? a.fxb[1] : a.fzb[1];
  double *F2 = t == 0 ? a.fxb[2] : a.fzb[2];
  const double2 *fld = t == 0 ? a.ub : a.wb;
  for (int j = 0; j < NY; ++j) {
    const double2 x = X0[j], y = fld[(size_t)j * M];
    ubar[j] = make_double2(x.x + y.x, x.y + y.y);
    const double2 o = t == 0 ? a.ozb[(size_t)j * M] : a.oxb[(size_t)j * M];
    dbar[j] = t == 0 ? make_double2(-o.x, -o.y) : o;
  }
  const double fbar = *F0 + (t == 0 ? a.weight : 0.0);
  dbar[NY - 1].x += -nu / a.Ly * fbar;
  dbar[0].x += nu / a.Ly * fbar;
  for (int j = 0; j < NY; ++j) {
    const bool in = j != 0 && j != NY - 1;
    sb[j] = in ? make_double2(icg * ubar[j].x, icg * ubar[j].y) : make_double2(0.0, 0.0);
  }
  auto rhs = [&](int c) -> double2 {
    const int jn = c >> 1;
    const bool in = jn != 0 && jn != NY - 1;
    if (c & 1) {
      const double w = in ? a.inv_h2 * nu * a.c22[jn] * icg : 0.0;
      return make_double2(w * ubar[jn].x, w * ubar[jn].y);
    }
    const double w = in ? nu * a.c21[jn] * icg : 0.0, c1 = a.c11[jn];
    return make_double2(a.inv_h * (c1 * dbar[jn].x + w * ubar[jn].x), a.inv_h * (c1 * dbar[jn].y + w * ubar[jn].y));
  };
  auto ys = [&](int p, double2 y) { yy[p] = y; };
  auto yl = [&](int p) -> double2 { return yy[p]; };
  auto out = [&](int p, double2 z) {
    const double s = icg * a.rs_g[(size_t)p * a.U];
    for (int e = 0; e < 5; ++e) {
      const double b = a.rb_val[p * 5 + e];
      if (b != 0.0) {
        double2 &d = sb[a.rb_col[p * 5 + e]];
        d.x += b * s * z.x;
        d.y += b * s * z.y;
      }
    }
  };
  band_solve_t<6, 6>(a.ab_g, a.piv_g, n, a.U, 0, rhs, ys, yl, out);
  const double al0 = 3.0, al1 = -1.5, al2 = 1.0 / 3.0, be0 = 3.0, be1 = -3.0, be2 = 1.0;
  double fsum = 0.0;
  for (int j = 0; j < NY; ++j) {
    const double2 s = sb[j];
    fsum += s.x;
    L1[j].x += be0 * s.x; L1[j].y += be0 * s.y;
    L2[j].x += be1 * s.x; L2[j].y += be1 * s.y;
    L0[j] = make_double2(be2 * s.x, be2 * s.y);
    const double q0 = al0 * a.inv_dt, q1 = al1 * a.inv_dt, q2 = al2 * a.inv_dt;
    X1[j].x += q0 * s.x; X1[j].y += q0 * s.y;
    X2[j].x += q1 * s.x; X2[j].y += q1 * s.y;
    X0[j] = make_double2(q2 * s.x, q2 * s.y);
  }
  *F1 += be0 * fsum;
  *F2 += be1 * fsum;
  *F0 = be2 * fsum;
}

void launch_adj_mean(const AdjMeanArgs &a, cudaStream_t st) { k_adj_mean<<<1, 32, 0, st>>>(a); }

// ---------------------------------------------------------------------------
// Mode kernel adjoint, two threads per real component of a mode (one per system).
// ---------------------------------------------------------------------------
// VMODE: the v-system's transposed solve over the full band (0) or inside
// the interior masks the setup check admitted (1: VMasks, 2: VMasks6).
// Blocks of two warps serve 16 modes (both real components): warp 0 the
// v-system's part (its inputs from solve_horizontal^T, the transposed v
// solve, the v, DY2 v and Hv histories), warp 1 the omega_y-system's (its
// inputs, the transposed omega_y solve, the g and Hg histories).  The two
// parts read and write disjoint data, so they need no synchronisation, and
// each value comes from the same operations as in one thread doing both.
template <int KLV, int KUV, int KLG, int KUG, int VMODE>
__global__ void __launch_bounds__(64) k_adj_modes(AdjModeArgs a) {
  const int role = threadIdx.x >> 5;  // 0: v-system, 1: omega_y-system
  const int tid = blockIdx.x * 32 + (threadIdx.x & 31);
  const int m = tid >> 1, comp = tid & 1;
  if (m >= a.M) return;
  const int M = a.M, NY = a.NY;
  const int k = m / a.NXH, i = m - k * a.NXH;
  const int kabs = (k <= a.NZH) ? k : a.NZ - k;
  const int u = kabs * a.NXH + i;
  const double kx = a.kx[i], kz = a.kz[k];
  const double k2 = kx * kx + kz * kz;
  const bool horiz = !(k2 < 1.e-8);
  const double ik2 = horiz ? 1.0 / k2 : 0.0;
  const double ax = kx * ik2, az = kz * ik2;
  const double icg = a.inv_cg[u], nu = a.nu, idt = a.inv_dt;
  const double al0 = 3.0, al1 = -1.5, al2 = 1.0 / 3.0, be0 = 3.0, be1 = -3.0, be2 = 1.0;
  auto E = [&](int j) { return 2 * ((size_t)j * M + m) + comp; };
  auto D = [](double2 *p) { return reinterpret_cast<double *>(p); };
  auto cmp = [&](double2 v) { return comp ? v.y : v.x; };
  // level 1 += c0 s, level 2 += c1 s, level 0 = c2 s
  auto upd = [&](double2 *const *f, int j, double s, double c0, double c1, double c2) {
    const size_t e = E(j);
    D(f[1])[e] += c0 * s;
    D(f[2])[e] += c1 * s;
    D(f[0])[e] = c2 * s;
  };

  // 1. solve_horizontal^T and the adjoints of the solves' outputs per node:
  //    v, D1 v (through DY1 v = c11 d1, DY2 v = c21 d1 + c22 d2), g, D1 g
  //    (each warp the part its system reads)
  for (int j = 0; j < NY; ++j) {
    const bool in = j != 0 && j != NY - 1;
    const size_t at = (size_t)j * M + m;
    const double c11 = a.c11[j], c21 = a.c21[j], c22 = a.c22[j];
    const size_t e = E(j);
    if (role == 0) {
      double2 vt = a.v[0][at], qt = a.q[0][at];
      const double2 vf = a.vb[at];
      vt.x += vf.x; vt.y += vf.y;
      double2 dv = make_double2(0.0, 0.0);
      if (horiz) {
        const double2 ub = a.ub[at], wb = a.wb[at], oxb = a.oxb[at], ozb = a.ozb[at];
        // adjoints of u = i ax DY1v - i az g, w = i ax g + i az DY1v,
        // om_x = i/k2 (kx DY1g + kz DY2v) - i kz v, om_z = i/k2 (kz DY1g - kx DY2v) + i kx v
        dv = make_double2(ax * ub.y + az * wb.y, -ax * ub.x - az * wb.x);
        qt.x += az * oxb.y - ax * ozb.y;
        qt.y += -az * oxb.x + ax * ozb.x;
        vt.x += -kz * oxb.y + kx * ozb.y;
        vt.y += kz * oxb.x - kx * ozb.x;
      }
      const double v_ = cmp(vt), q_ = cmp(qt), dv_ = cmp(dv);
      D(a.xv0)[e] = v_;
      D(a.xv1)[e] = a.inv_h * (c11 * dv_ + c21 * q_);
      D(a.xv2)[e] = a.inv_h2 * c22 * q_;
    } else {
      double2 gt = a.g[0][at];
      const double2 gf = a.gb[at];
      gt.x += gf.x; gt.y += gf.y;
      double2 dg = make_double2(0.0, 0.0);
      if (horiz) {
        const double2 ub = a.ub[at], wb = a.wb[at], oxb = a.oxb[at], ozb = a.ozb[at];
        gt.x += -az * ub.y + ax * wb.y;
        gt.y += az * ub.x - ax * wb.x;
        dg = make_double2(ax * oxb.y + az * ozb.y, -ax * oxb.x - az * ozb.x);
      }
      const double g_ = cmp(gt), dg_ = cmp(dg);
      D(a.xg0)[e] = a.inv_h * (c11 * dg_ + (in ? nu * c21 * icg * g_ : 0.0));
      D(a.xg1)[e] = in ? a.inv_h2 * nu * c22 * icg * g_ : 0.0;
      D(a.sgb)[e] = in ? icg * g_ : 0.0;
    }
  }

  // 2. v-system^T: the source adjoint is scattered through the rows' rhs
  //    tables, then feeds Hv, v, DY2 v of the three levels; the two wall
  //    rows give the wall-velocity gradient
  if (role == 0) {
    for (int j = 0; j < NY; ++j) D(a.svb)[E(j)] = 0.0;
    auto rhs = [&](int c) -> double {
      int t, jn;
      vcol_split(c, NY, t, jn);
      if (t == 0) return D(a.xv0)[E(jn)];
      if (t == 1) return D(a.xv1)[E(jn)];
      if (t == 2) return D(a.xv2)[E(jn)];
      return 0.0;
    };
    auto ys = [&](int p, double y) { D(a.yv)[E(p)] = y; };
    auto yl = [&](int p) -> double { return D(a.yv)[E(p)]; };
    auto out = [&](int p, double z) {
      const double r = z * a.rs_v[(size_t)p * a.U + u];
      const int tag = a.rhs_node_v[p];
      if (tag == kRhsTable) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const double b = a.rbv_val[p * 4 + q];
          if (b != 0.0) D(a.svb)[E(a.rbv_col[p * 4 + q])] += b * r;
        }
      } else if (tag == kRhsWallBottom) {
        D(a.grad)[2 * (size_t)m + comp] += r;
      } else if (tag == kRhsWallTop) {
        D(a.grad)[2 * ((size_t)M + m) + comp] += r;
      }
    };
    if constexpr (VMODE == 1)
      band_solve_t_masked<KLV, KUV, 4, 2, VMasks>(a.ab_v, a.piv_v, a.n_v, a.U, u, rhs, ys, yl, out);
    else if constexpr (VMODE == 2)
      band_solve_t_masked<KLV, KUV, 4, 2, VMasks6>(a.ab_v, a.piv_v, a.n_v, a.U, u, rhs, ys, yl, out);
    else
      band_solve_t<KLV, KUV>(a.ab_v, a.piv_v, a.n_v, a.U, u, rhs, ys, yl, out);
    // source_v = sum beta Hv_l - k^2/dt sum alpha v_l + sum alpha q_l / dt on
    // nodes 2..NY-3; the tables reference no other node, so svb is zero there
    for (int j = 0; j < NY; ++j) {
      const double r = D(a.svb)[E(j)];
      upd(a.hv, j, r, be0, be1, be2);
      upd(a.v, j, -k2 * idt * r, al0, al1, al2);
      upd(a.q, j, idt * r, al0, al1, al2);
    }
  }

  // 3. omega_y-system^T: source adjoint scattered through the B rows
  else {
    auto rhs = [&](int c) -> double { return (c & 1) ? D(a.xg1)[E(c >> 1)] : D(a.xg0)[E(c >> 1)]; };
    auto ys = [&](int p, double y) { D(a.yg)[E(p)] = y; };
    auto yl = [&](int p) -> double { return D(a.yg)[E(p)]; };
    auto out = [&](int p, double z) {
      const double r = z * icg * a.rs_g[(size_t)p * a.U + u];
#pragma unroll
      for (int e = 0; e < 5; ++e) {
        const double b = a.rb_val[p * 5 + e];
        if (b != 0.0) D(a.sgb)[E(a.rb_col[p * 5 + e])] += b * r;
      }
    };
    band_solve_t<KLG, KUG>(a.ab_g, a.piv_g, a.n_g, a.U, u, rhs, ys, yl, out);
    for (int j = 0; j < NY; ++j) {
      const double s = D(a.sgb)[E(j)];
      upd(a.hg, j, s, be0, be1, be2);
      upd(a.g, j, idt * s, al0, al1, al2);
    }
  }
}

void launch_adj_modes(const AdjModeArgs &a, int vmode, cudaStream_t st) {
  const int grid = (2 * a.M + 31) / 32;  // 16 modes (32 real components) a block of two warps
  if (vmode == 1) k_adj_modes<kVKL, kVKU, 6, 6, 1><<<grid, 64, 0, st>>>(a);
  else if (vmode == 2) k_adj_modes<kVKL, kVKU, 6, 6, 2><<<grid, 64, 0, st>>>(a);
  else k_adj_modes<kVKL, kVKU, 6, 6, 0><<<grid, 64, 0, st>>>(a);
}

// ---------------------------------------------------------------------------
__global__ void k_objective_add(const double *fx_ring, const long long *step, double weight, double *acc) {
  *acc += weight * fx_ring[ring_head(*step)];
}

void launch_objective_add(const double *fx_ring, const long long *step, double weight, double *acc,
                          cudaStream_t st) {
  k_objective_add<<<1, 1, 0, st>>>(fx_ring, step, weight, acc);
}

}  // namespace owt

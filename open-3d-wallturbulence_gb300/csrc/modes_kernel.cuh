// The mode kernel (RHS assembly, both implicit solves, solve_horizontal's
// components) as a template; instantiated by modes_pair.cu / modes_quad.cu.
#pragma once
#include <cuda_runtime.h>

#include "owt_device.cuh"
#include "setup_host.h"
#include "solve_kernels.h"

namespace owt {

// ---------------------------------------------------------------------------
// Mode kernel: two threads per Fourier mode (one per real component).  For
// mode (kz, kx):
//  1. source_g = sum beta Hg_l + sum alpha g_l / dt      (solver.cpp:573-574)
//  2. omega_y-system: g and DY1 g                         (solver.cpp:578, 603)
//  3. source_v = sum beta Hv_l - k^2/dt sum alpha v_l + DY2(sum alpha v_l)/dt
//     with DY2 v_l kept as a history of its own (q_l)    (solver.cpp:569-571)
//  4. v-system: v, D1 v, D2 v                             (solver.cpp:577, 602)
//     with v = v_w on the walls when blowing/suction is set; its rows carry
//     combinations of source_v (the fourth-derivative rows into which the
//     interior equations were substituted)
//  5. solve_horizontal's velocity/vorticity from v, g    (solver.cpp:532-536)
//
// ROLE 0: one thread does all of it.  ROLE 1 and 2 (the split mapping, pair
// lanes only): a warp of ROLE 1 does steps 1 and 2 for 16 modes and a warp
// of ROLE 2 steps 1, 3-5 for the same modes; the v-system's forward sweep
// runs beside the omega_y solve, and named barrier `bar` (the two warps, 64
// threads; every thread of both arrives exactly once, active or not) orders
// the omega_y results before the backward sweep that reads them.  Each value
// is computed by the same operations as in ROLE 0.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void named_bar_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}
__device__ __forceinline__ void named_bar_arrive(int id, int nthreads) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

template <int KLV, int KUV, int KLG, int KUG, bool SPARSE, bool QUAD, class VM = VMasks, int ROLE = 0>
__device__ __forceinline__ void mode_body(const ModeArgs &a, const int tid, const int bar = 0) {
  static_assert(ROLE == 0 || (!QUAD && SPARSE), "the split mapping pairs lanes and runs the masked solves");
  // One thread per real component of a mode (the band systems are real).
  // Pair mapping: lanes 2m, 2m+1 are Re, Im of mode m.  Quad mapping: lanes
  // 4u..4u+3 are (Re, Im) of the two modes +kz, -kz of unique mode u, which
  // share one factorization, so four adjacent lanes read the same factors.
  int m, comp, k, i, kabs;
  const bool active = QUAD || (tid >> 1) < a.M;
  if (QUAD) {
    const int uq = a.u0 + (tid >> 2), r = tid & 3, sgn = r >> 1;
    comp = r & 1;
    if (uq >= a.u1) return;
    kabs = uq / a.NXH;
    i = uq - kabs * a.NXH;
    if (sgn == 1 && (kabs == 0 || kabs == a.NZH)) return;  // these have no -kz partner
    k = sgn == 0 ? kabs : a.NZ - kabs;
    m = k * a.NXH + i;
  } else {
    m = tid >> 1;
    comp = tid & 1;
    if (m >= a.M) {
      if (ROLE == 0) return;
      m = 0;  // an idle lane of the split mapping: no work, but it arrives at the barrier
    }
    k = m / a.NXH;
    i = m - k * a.NXH;
    kabs = (k <= a.NZH) ? k : a.NZ - k;
  }
  const int M = a.M, NY = a.NY;
  const int u = kabs * a.NXH + i;
  const double kx = a.kx[i], kz = a.kz[k];
  const double k2 = kx * kx + kz * kz;
  const long long s = *a.step;
  const int h = ring_head(s);
  const size_t fs2 = 2 * (size_t)NY * M;  // doubles per field
  auto lvl = [&](const double2 *ring, int l) {
    return reinterpret_cast<const double *>(ring) + (size_t)((h + l) % 3) * fs2 + comp;
  };
  const double *v0 = lvl(a.v_ring, 0), *v1 = lvl(a.v_ring, 1), *v2 = lvl(a.v_ring, 2);
  const double *g0 = lvl(a.g_ring, 0), *g1 = lvl(a.g_ring, 1), *g2 = lvl(a.g_ring, 2);
  const double *hv0 = lvl(a.hv_ring, 0), *hv1 = lvl(a.hv_ring, 1), *hv2 = lvl(a.hv_ring, 2);
  const double *hg0 = lvl(a.hg_ring, 0), *hg1 = lvl(a.hg_ring, 1), *hg2 = lvl(a.hg_ring, 2);
  const double *q0 = lvl(a.q_ring, 0), *q1 = lvl(a.q_ring, 1), *q2 = lvl(a.q_ring, 2);
  const int hn = (h + 2) % 3;  // slot of the new level 0
  double *vn = reinterpret_cast<double *>(a.v_ring) + (size_t)hn * fs2 + comp;
  double *gn = reinterpret_cast<double *>(a.g_ring) + (size_t)hn * fs2 + comp;
  double *qn = reinterpret_cast<double *>(a.q_ring) + (size_t)hn * fs2 + comp;
  double *sg = reinterpret_cast<double *>(a.sg) + comp;
  double *sv = reinterpret_cast<double *>(a.sv) + comp;
  double *dg = reinterpret_cast<double *>(a.dg) + comp;
  double *yv = reinterpret_cast<double *>(a.yv) + comp;
  double *yg = reinterpret_cast<double *>(a.yg) + comp;
  auto E = [&](int j) { return 2 * ((size_t)j * M + m); };  // offset of (j, m) in doubles
  // (be1 = -be0 and be2 = 1 are used in the form of step 1)
  const double al0 = 3.0, al1 = -1.5, al2 = 1.0 / 3.0, be0 = 3.0;
  const double idt = a.inv_dt;

  // 1. source_g, walls zero (solver.cpp:573-574, 598-599), and source_v on
  //    the nodes with an interior equation (solver.cpp:569-571, 590-596).
  //    The beta sum 3 H0 - 3 H1 + H2 is formed as 3 (H0 - H1) + H2, and 1/dt
  //    (and -k^2/dt for v) is folded into the alpha weights: two and three
  //    FP64 operations fewer per node than the sums as written.
  {
    const double k2dt = k2 * idt;
    const double ag0 = al0 * idt, ag1 = al1 * idt, ag2 = al2 * idt;
    const double av0 = -k2dt * al0, av1 = -k2dt * al1, av2 = -k2dt * al2;
    for (int j = 0; j < NY && active; ++j) {
      const size_t e = E(j);
      if (ROLE != 2) {
        double r = 0.0;
        if (j != 0 && j != NY - 1)
          r = fma(g2[e], ag2, fma(g1[e], ag1, fma(g0[e], ag0, fma(hg0[e] - hg1[e], be0, hg2[e]))));
        sg[e] = r;
      }
      if (ROLE != 1) {
        double rv = 0.0;
        if (j >= 2 && j <= NY - 3) {
          rv = fma(hv0[e] - hv1[e], be0, hv2[e]);
          rv = fma(v0[e], av0, rv);
          rv = fma(v1[e], av1, rv);
          rv = fma(v2[e], av2, rv);
          rv = fma(q0[e], ag0, rv);
          rv = fma(q1[e], ag1, rv);
          rv = fma(q2[e], ag2, rv);
        }
        sv[e] = rv;
      }
    }
  }

  // 2. omega_y-system: g and DY1 g.  The solve gives h DY1 g and h^2 DY2 g;
  //    the tables c11h, nc21h, nc22h carry the 1/h, 1/h^2 of the metric
  //    coefficients, and rs_gi the 1/cg of the row scales.
  if (ROLE != 2 && active) {
    const double icg = a.inv_cg[u];
    double d2 = 0.0;
    auto rhs = [&](int p) -> double {
      double acc = 0.0;
#pragma unroll
      for (int q = 0; q < 5; ++q) acc += a.rb_val[p * 5 + q] * sg[E(a.rb_col[p * 5 + q])];
      return acc * a.rs_gi[(size_t)p * a.U + u];
    };
    auto ys = [&](int p, double y) { yg[E(p)] = y; };
    auto yl = [&](int p) -> double { return yg[E(p)]; };
    auto out = [&](int c, double x) {
      const int jn = c >> 1;
      if (c & 1) {
        d2 = x;
      } else {
        const size_t e = E(jn);
        double g = 0.0;
        if (jn != 0 && jn != NY - 1) g = fma(a.nc22h[jn], d2, fma(a.nc21h[jn], x, sg[e])) * icg;
        gn[e] = g;
        dg[e] = a.c11h[jn] * x;
      }
    };
    if (SPARSE) band_solve_g_sparse(a.ab_g, a.piv_g, a.n_g, a.U, u, rhs, ys, yl, out);
    else band_solve<KLG, KUG>(a.ab_g, a.piv_g, a.n_g, a.U, u, rhs, ys, yl, out);
  }
  if (ROLE == 0) __syncwarp(__activemask());  // the partner's g, DY1 g are read below
  if (ROLE == 1) {
    __threadfence_block();  // g, DY1 g before the v warp's backward sweep reads them
    named_bar_arrive(bar, 64);
    return;
  }

  // 3-5. v-system, then solve_horizontal's components
  {
    const bool horiz = !(k2 < 1.e-8);
    const double ik2 = horiz ? 1.0 / k2 : 0.0;
    const double sgn = comp ? 1.0 : -1.0;
    const double sax = sgn * kx * ik2, saz = sgn * kz * ik2, skx = sgn * kx, skz = sgn * kz;
    double xv = 0.0, d1 = 0.0, d2 = 0.0;  // v, h DY1 v, h^2 DY2 v of the node being finished
    auto rhs = [&](int p) -> double {
      const int tag = a.rhs_node_v[p];
      if (tag == kRhsTable) {
        double acc = 0.0;
#pragma unroll
        for (int q = 0; q < 4; ++q) acc += a.rbv_val[p * 4 + q] * sv[E(a.rbv_col[p * 4 + q])];
        return acc * a.rs_v[(size_t)p * a.U + u];
      }
      // wall rows: v = v_w (blowing/suction) or 0 (solver.cpp:593-596)
      if (tag == kRhsNone || !a.vw) return 0.0;
      const double *vw = reinterpret_cast<const double *>(a.vw) + (tag == kRhsWallBottom ? 0 : 2 * (size_t)M);
      return vw[2 * m + comp] * a.rs_v[(size_t)p * a.U + u];
    };
    auto ys = [&](int p, double y) { yv[E(p)] = y; };
    auto yl = [&](int p) -> double { return yv[E(p)]; };
    auto out = [&](int c, double x) {
      int t, jn;
      vcol_split(c, NY, t, jn);
      // the backward sweep gives a node's unknowns in falling column order:
      // at the four wall nodes d2, d1, then v; at interior nodes (reversed
      // order) v, d1, then d2.  The node is finished with the last of the three.
      const bool wall = jn < 2 || jn >= NY - 2;
      bool last = false;
      if (t == 2) {
        d2 = x;
        last = !wall;
      } else if (t == 1) {
        d1 = x;
      } else if (t == 0) {
        xv = x;
        last = wall;
      }
      if (last) {
        x = xv;
        const size_t e = E(jn);
        vn[e] = x;
        const double q = fma(a.c22h[jn], d2, a.c21h[jn] * d1);
        qn[e] = q;
        if (horiz) {
          const double dv = a.c11h[jn] * d1;
          const unsigned mask = __activemask();
          // the partner lane's component of v, DY1 v, DY2 v; of g, DY1 g from memory
          const double xo = __shfl_xor_sync(mask, x, 1), dvo = __shfl_xor_sync(mask, dv, 1),
                       qo = __shfl_xor_sync(mask, q, 1);
          const double go = gn[e + 1 - 2 * comp], dgo = dg[e + 1 - 2 * comp];
          // u = i kx/k2 DY1v - i kz/k2 g ; w = i kx/k2 g + i kz/k2 DY1v
          // omega_x = i/k2 (kx DY1g + kz DY2v) - i kz v ; omega_z = i/k2 (kz DY1g - kx DY2v) + i kx v
          // component c of i z is (2c - 1) times the other component of z
          double *uo = reinterpret_cast<double *>(a.u_out), *wo = reinterpret_cast<double *>(a.w_out);
          double *oxo = reinterpret_cast<double *>(a.ox_out), *ozo = reinterpret_cast<double *>(a.oz_out);
          uo[e + comp] = sax * dvo - saz * go;
          wo[e + comp] = sax * go + saz * dvo;
          oxo[e + comp] = fma(-skz, xo, fma(saz, qo, sax * dgo));
          ozo[e + comp] = fma(skx, xo, fma(-sax, qo, saz * dgo));
        }
      }
    };
    if (SPARSE) {
      if (active) band_forward_v_sparse<VM>(a.ab_v, a.piv_v, a.n_v, a.U, u, rhs, ys);
      if (ROLE == 2) named_bar_sync(bar, 64);
      if (active) band_backward_v_sparse<VM>(a.ab_v, a.n_v, a.U, u, yl, ys, out);
    } else {
      band_solve<KLV, KUV>(a.ab_v, a.piv_v, a.n_v, a.U, u, rhs, ys, yl, out);
    }
  }
}

// One channel: thread tid of the grid is thread tid of the mapping.
template <int KLV, int KUV, int KLG, int KUG, bool SPARSE, bool QUAD, int BLOCK, int MINB, class VM = VMasks>
__global__ void __launch_bounds__(BLOCK, MINB) k_modes(const __grid_constant__ ModeArgs a) {
  mode_body<KLV, KUV, KLG, KUG, SPARSE, QUAD, VM>(a, blockIdx.x * BLOCK + threadIdx.x);
}

// The split mapping: warp pairs (omega_y warp, v warp) over the pair
// mapping's lanes; BLOCK/64 pairs per block, barrier ids 1 .. BLOCK/64.
template <int KLV, int KUV, int KLG, int KUG, int BLOCK, int MINB, class VM = VMasks>
__global__ void __launch_bounds__(BLOCK, MINB) k_modes_split(const __grid_constant__ ModeArgs a) {
  static_assert(BLOCK % 64 == 0 && BLOCK / 64 <= 15, "warp pairs and named barriers");
  const int w = threadIdx.x >> 5, pair = w >> 1;
  const int tid = blockIdx.x * (BLOCK / 2) + pair * 32 + (threadIdx.x & 31);
  if (w & 1) mode_body<KLV, KUV, KLG, KUG, true, false, VM, 2>(a, tid, 1 + pair);
  else mode_body<KLV, KUV, KLG, KUG, true, false, VM, 1>(a, tid, 1 + pair);
}

// Every channel of a batch in one persistent launch.  Work items are the
// BLOCK-thread slices of each channel's mapping, numbered channel by channel
// in the table's order (the host lists the channels with the longest systems
// first); resident blocks take items from an atomic counter until none are
// left, so channels of uneven sizes share the SMs without a tail per channel.
// The last block to finish resets the counter for the next launch.
template <int KLV, int KUV, int KLG, int KUG, bool SPARSE, bool QUAD, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB)
    k_modes_batch(const __grid_constant__ BatchTable<ModeArgs> t, int *work) {
  __shared__ int item;
  const int total = t.start[t.n];
  for (;;) {
    if (threadIdx.x == 0) item = atomicAdd(work, 1);
    __syncthreads();
    const int it = item;
    __syncthreads();  // every thread has read item before it is overwritten
    if (it >= total) break;
    const int c = batch_channel(t.start, t.n, it);
    mode_body<KLV, KUV, KLG, KUG, SPARSE, QUAD>(t.a[c], (it - t.start[c]) * BLOCK + threadIdx.x);
  }
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(work + 1, 1) == (int)gridDim.x - 1) {
      work[0] = 0;
      work[1] = 0;
    }
  }
}


int modes_pair_count();
const char *modes_pair_name(int v);
void modes_pair_launch(int v, const ModeArgs &a, cudaStream_t st);
void modes_dense_launch(const ModeArgs &a, cudaStream_t st);
void modes_sixth_launch(const ModeArgs &a, cudaStream_t st);  // the sixth-order masks
int modes_split_count();
const char *modes_split_name(int v);
void modes_split_launch(int v, const ModeArgs &a, cudaStream_t st);
bool modes_split_is_quad(int v);
int modes_quad_count();
const char *modes_quad_name(int v);
void modes_quad_launch(int v, const ModeArgs &a, cudaStream_t st);

// Batched launches: the work-item geometry of a variant and the persistent launch.
ModeBatchShape modes_pair_batch_shape(int v);
ModeBatchShape modes_quad_batch_shape(int v);
ModeBatchShape modes_dense_batch_shape();
void modes_pair_batch_launch(int v, const BatchTable<ModeArgs> &t, int *work, int grid, cudaStream_t st);
void modes_quad_batch_launch(int v, const BatchTable<ModeArgs> &t, int *work, int grid, cudaStream_t st);
void modes_dense_batch_launch(const BatchTable<ModeArgs> &t, int *work, int grid, cudaStream_t st);

}  // namespace owt

// DY1 along y for caller-owned device arrays, without any device allocation.
//
// Some callers cannot call cudaMalloc: code that runs while a CUDA graph is
// being captured (allocation is not a stream operation), host programs that
// hand the whole device memory to their own pool allocator and forbid other
// allocations, and tight loops where cudaMalloc's implicit device-wide
// synchronisation is not acceptable.  owt_dy1_noalloc serves them: it needs no
// handle (creating one allocates) and keeps its scratch in a file-scope
// static __device__ array of fixed size.  That array is reserved on every GPU
// that loads this library, for the life of the process.
//
// What it computes is the handle-based DY1 (owt_dy_apply with order 1):
// out = diag(c11) A1^-1 B1 in along y, for every line, with the compact first
// derivative of src/compdiff.hpp:11-69 and c11 = 1/(dy/ds) of
// src/solver.cpp:77,94 on the grid y = tanh(alpha s)/tanh(alpha).  Each call
// first rebuilds the A1 band factors, B1 rows and c11 for its (NY, alpha) in
// the static array (one small kernel), then runs the derivative kernel.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "owt_device.cuh"
#include "owt_gpu.h"

namespace owt {

// Layout of the static array: [setup region][bf: MAX values][yscr: MAX values]
constexpr size_t NOALLOC_SETUP_BYTES = 256 * 1024;
constexpr size_t NOALLOC_SCRATCH_BYTES =
    NOALLOC_SETUP_BYTES + 2 * (size_t)OWT_NOALLOC_MAX_VALUES * sizeof(double2);

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

struct NoallocSetup {
  // all inside the setup region; NY <= OWT_NOALLOC_MAX_NY
  double *ab;      // 7 x NY band (kl = ku = 2, LAPACK factorization layout)
  uint8_t *piv;    // NY
  double *c11;     // NY
  int *bcol;       // NY x 5
  double *bval;    // NY x 5
};

__host__ __device__ inline NoallocSetup noalloc_layout(unsigned char *base, int NY) {
  NoallocSetup s;
  const int nmax = OWT_NOALLOC_MAX_NY;
  s.ab = reinterpret_cast<double *>(base);
  s.c11 = s.ab + 7 * nmax;
  s.bval = s.c11 + nmax;
  s.bcol = reinterpret_cast<int *>(s.bval + 5 * nmax);
  s.piv = reinterpret_cast<uint8_t *>(s.bcol + 5 * nmax);
  (void)NY;
  return s;
}

// One thread: grid metric, B1 rows, A1 band assembled and factored with
// partial pivoting (the dgbtf2 order used by the handle's factorization).
// Everything the derivative kernel reads is rewritten here, band fill rows
// cleared, so nothing depends on what an earlier call left in the array.
__global__ void k_noalloc_setup(unsigned char *base, int NY, double alpha) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  NoallocSetup s = noalloc_layout(base, NY);
  const double h = 2.0 / (NY - 1.0);
  const double coth_ap = 1.0 / tanh(alpha);
  for (int i = 0; i < NY; ++i) {
    const double si = 2 * i / (NY - 1.0) - 1.0;
    const double sech = 1.0 / cosh(alpha * si);
    s.c11[i] = 1.0 / (alpha * coth_ap * sech * sech);
  }
  // B1 rows (col, val) x 5, zero-padded
  for (int e = 0; e < 5 * NY; ++e) { s.bcol[e] = 0; s.bval[e] = 0.0; }
  auto put = [&](int row, int k, int col, double v) { s.bcol[row * 5 + k] = col; s.bval[row * 5 + k] = v; };
  const double a2 = 40.0 / 27.0, b2 = 25.0 / 54.0;
  for (int i = 2; i < NY - 2; ++i) {
    put(i, 0, i - 2, -b2 / (4 * h)); put(i, 1, i - 1, -a2 / (2 * h));
    put(i, 2, i + 1, a2 / (2 * h)); put(i, 3, i + 2, b2 / (4 * h));
  }
  for (int i : {1, NY - 2}) { put(i, 0, i - 1, -1.5 / (2 * h)); put(i, 1, i + 1, 1.5 / (2 * h)); }
  const double a0 = -17.0 / 6.0, b0 = 1.5, c0 = 1.5, d0 = -1.0 / 6.0;
  put(0, 0, 0, a0 / h); put(0, 1, 1, b0 / h); put(0, 2, 2, c0 / h); put(0, 3, 3, d0 / h);
  put(NY - 1, 0, NY - 1, -a0 / h); put(NY - 1, 1, NY - 2, -b0 / h);
  put(NY - 1, 2, NY - 3, -c0 / h); put(NY - 1, 3, NY - 4, -d0 / h);
  // A1 band, rows b = KV + i - j with KV = 4 (kl = ku = 2)
  constexpr int KL = 2, KU = 2, KV = KL + KU, NB = 2 * KL + KU + 1;
  for (int e = 0; e < NB * NY; ++e) s.ab[e] = 0.0;
  auto A = [&](int i, int j) -> double & { return s.ab[(KV + i - j) * NY + j]; };
  for (int i = 2; i < NY - 2; ++i) {
    A(i, i - 2) = 1.0 / 36.0; A(i, i - 1) = 4.0 / 9.0; A(i, i) = 1.0; A(i, i + 1) = 4.0 / 9.0; A(i, i + 2) = 1.0 / 36.0;
  }
  for (int i : {1, NY - 2}) { A(i, i - 1) = 0.25; A(i, i) = 1.0; A(i, i + 1) = 0.25; }
  A(0, 0) = 1.0; A(0, 1) = 3.0; A(NY - 1, NY - 1) = 1.0; A(NY - 1, NY - 2) = 3.0;
  auto AB = [&](int b, int c) -> double & { return s.ab[b * NY + c]; };
  int ju = 0;
  for (int j = 0; j < NY; ++j) {
    const int km = min(KL, NY - 1 - j);
    int jp = 0;
    double best = fabs(AB(KV, j));
    for (int i = 1; i <= km; ++i) {
      const double v = fabs(AB(KV + i, j));
      if (v > best) { best = v; jp = i; }
    }
    s.piv[j] = (uint8_t)jp;
    ju = max(ju, min(j + KU + jp, NY - 1));
    if (jp != 0)
      for (int c = j; c <= ju; ++c) {
        const double t = AB(KV + jp - (c - j), c);
        AB(KV + jp - (c - j), c) = AB(KV - (c - j), c);
        AB(KV - (c - j), c) = t;
      }
    const double rp = 1.0 / AB(KV, j);
    for (int i = 1; i <= km; ++i) AB(KV + i, j) *= rp;
    for (int c = j + 1; c <= ju; ++c) {
      const double t = AB(KV - (c - j), c);
      if (t != 0.0)
        for (int i = 1; i <= km; ++i) AB(KV + i - (c - j), c) -= AB(KV + i, j) * t;
    }
  }
  for (int j = 0; j < NY; ++j) AB(KV, j) = 1.0 / AB(KV, j);
}

// One thread per line: bf = B1 f, band solve with A1, out = c11 * d.
__global__ void __launch_bounds__(128) k_dy1_noalloc(unsigned char *base, int NY, int nlines,
                                                     const double2 *__restrict__ in, double2 *__restrict__ out) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nlines) return;
  NoallocSetup s = noalloc_layout(base, NY);
  double2 *bf = reinterpret_cast<double2 *>(base + NOALLOC_SETUP_BYTES);
  double2 *yscr = bf + OWT_NOALLOC_MAX_VALUES;
  const int M = nlines;
  for (int j = 0; j < NY; ++j) {
    double2 acc = make_double2(0.0, 0.0);
#pragma unroll
    for (int e = 0; e < 5; ++e) {
      const double b = s.bval[j * 5 + e];
      if (b != 0.0) {
        const double2 f = in[(size_t)s.bcol[j * 5 + e] * M + m];
        acc.x += b * f.x;
        acc.y += b * f.y;
      }
    }
    bf[(size_t)j * M + m] = acc;
  }
  auto rhs = [&](int p) -> double2 { return bf[(size_t)p * M + m]; };
  auto ys = [&](int p, double2 y) { yscr[(size_t)p * M + m] = y; };
  auto yl = [&](int p) -> double2 { return yscr[(size_t)p * M + m]; };
  auto outf = [&](int c, double2 d) { out[(size_t)c * M + m] = make_double2(s.c11[c] * d.x, s.c11[c] * d.y); };
  band_solve<2, 2>(s.ab, s.piv, NY, 1, 0, rhs, ys, yl, outf);
}

}  // namespace owt

// capi.cu: the calling thread's message for owt_last_error(NULL)
void owt_set_thread_error(const std::string &m);

namespace {
std::mutex g_noalloc_mu;
unsigned char *g_noalloc_ptr[256] = {nullptr};  // device address of the static array, per device
}  // namespace

extern "C" int owt_dy1_noalloc(int64_t NY, int64_t nlines, double alpha_mesh, const double *d_in, double *d_out,
                               void *stream) {
  using namespace owt;
  auto fail = [&](int code, const std::string &m) {
    owt_set_thread_error(m);
    return code;
  };
  if (NY < 7 || NY > OWT_NOALLOC_MAX_NY)
    return fail(OWT_ERR_INVALID, "NY must be within [7, " + std::to_string(OWT_NOALLOC_MAX_NY) + "]");
  if (nlines < 1 || NY * nlines > (int64_t)OWT_NOALLOC_MAX_VALUES)
    return fail(OWT_ERR_INVALID, "NY * nlines must be within [1, " + std::to_string(OWT_NOALLOC_MAX_VALUES) +
                                     "] complex values (the static scratch holds that many)");
  if (!(alpha_mesh > 0)) return fail(OWT_ERR_INVALID, "alpha_mesh must be positive");
  if (!d_in || !d_out || ((uintptr_t)d_in % 16) || ((uintptr_t)d_out % 16))
    return fail(OWT_ERR_INVALID, "d_in and d_out must be 16-byte aligned device pointers");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 256) return fail(OWT_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  unsigned char *base = nullptr;
  {
    // once per device, with that device current: the device address of the
    // static array (its host-side name is only a stand-in)
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      void *p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) return fail(OWT_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_noalloc_ptr[dev] = static_cast<unsigned char *>(p);
    }
    base = g_noalloc_ptr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_noalloc_setup<<<1, 32, 0, st>>>(base, (int)NY, alpha_mesh);
  k_dy1_noalloc<<<(unsigned)((nlines + 127) / 128), 128, 0, st>>>(
      base, (int)NY, (int)nlines, reinterpret_cast<const double2 *>(d_in), reinterpret_cast<double2 *>(d_out));
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(OWT_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return OWT_OK;
}

// DY1 along y for caller-owned device arrays, without any device allocation.
//
// Some callers cannot call cudaMalloc: programs that hand the whole device
// memory to their own pool allocator and forbid allocations from elsewhere,
// and tight loops that cannot accept the implicit device-wide
// synchronisation cudaMalloc and cudaFree bring.  owt_dy1_noalloc serves
// them: it needs no handle (creating one allocates) and keeps its scratch in
// a file-scope static __device__ array of fixed size.  That array is reserved
// on every GPU that loads this library, for the life of the process.
//
// What it computes is the handle-based DY1 (owt_dy_apply with order 1):
// out = diag(c11) A1^-1 B1 in along y, for every line, with the compact first
// derivative of src/compdiff.hpp:11-69 and c11 = 1/(dy/ds) of
// src/solver.cpp:77,94 on the grid y = tanh(alpha s)/tanh(alpha).  Each call
// first rebuilds the A1 band factors, B1 rows and c11 for its (NY, alpha) in
// the static array (one small kernel, noalloc_setup.h), then runs the
// derivative kernel.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "noalloc_setup.h"
#include "owt_device.cuh"
#include "owt_gpu.h"

namespace owt {

// Layout of the static array: [setup region][bf: MAX values][yscr: MAX values]
constexpr size_t NOALLOC_SETUP_BYTES = 256 * 1024;
static_assert(noalloc_setup_bytes() <= NOALLOC_SETUP_BYTES, "setup tables exceed their region");
static_assert(kNoallocMaxNY == OWT_NOALLOC_MAX_NY, "table layout and the entry point's limit disagree");
constexpr size_t NOALLOC_SCRATCH_BYTES =
    NOALLOC_SETUP_BYTES + 2 * (size_t)OWT_NOALLOC_MAX_VALUES * sizeof(double2);

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// One thread builds the operator tables for (NY, alpha) in the array.
__global__ void k_noalloc_setup(unsigned char *base, int NY, double alpha) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const NoallocSetup s = noalloc_layout(base);
  noalloc_assemble(s, NY, alpha);
  noalloc_factor(s, NY);
}

// One thread per line: bf = B1 f, band solve with A1, out = c11 * d.
__global__ void __launch_bounds__(128) k_dy1_noalloc(unsigned char *base, int NY, int nlines,
                                                     const double2 *__restrict__ in, double2 *__restrict__ out) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nlines) return;
  const NoallocSetup s = noalloc_layout(base);
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
// Device address of the static array, looked up once per device on the first
// call with that device current.  It belongs to the device's primary context:
// after cudaDeviceReset it would be stale, so this entry point must not be
// used across a device reset.
std::mutex g_noalloc_mu;
unsigned char *g_noalloc_ptr[256] = {nullptr};
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

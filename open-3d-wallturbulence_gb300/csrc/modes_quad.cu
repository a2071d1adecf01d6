// Mode-kernel variants with the quad thread mapping (see modes_kernel.cuh).
#include "modes_kernel.cuh"

namespace owt {

namespace {
struct Variant {
  const char *name;
  int block;
  void (*kernel)(ModeArgs);
  void (*batch)(BatchTable<ModeArgs>, int *);
};
const Variant kVariants[] = {
    {"quad/128/r166", 128, k_modes<kVKL, kVKU, 6, 6, true, true, 128, 3>, k_modes_batch<kVKL, kVKU, 6, 6, true, true, 128, 3>},
    {"quad/128/r128", 128, k_modes<kVKL, kVKU, 6, 6, true, true, 128, 4>, k_modes_batch<kVKL, kVKU, 6, 6, true, true, 128, 4>},
    {"quad/256/r128", 256, k_modes<kVKL, kVKU, 6, 6, true, true, 256, 2>, k_modes_batch<kVKL, kVKU, 6, 6, true, true, 256, 2>},
};

int resident(void (*kernel)(BatchTable<ModeArgs>, int *), int block) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, 0);
  return (per > 0 ? per : 1) * (sms > 0 ? sms : 1);
}
}  // namespace

int modes_quad_count() { return (int)(sizeof(kVariants) / sizeof(kVariants[0])); }
const char *modes_quad_name(int v) { return kVariants[v].name; }
void modes_quad_launch(int v, const ModeArgs &a, cudaStream_t st) {
  const Variant &x = kVariants[v];
  const long long threads = 4 * (long long)(a.u1 - a.u0);
  x.kernel<<<(unsigned)((threads + x.block - 1) / x.block), x.block, 0, st>>>(a);
}

ModeBatchShape modes_quad_batch_shape(int v) {
  const Variant &x = kVariants[v];
  return {x.block, true, resident(x.batch, x.block)};
}
void modes_quad_batch_launch(int v, const BatchTable<ModeArgs> &t, int *work, int grid, cudaStream_t st) {
  const Variant &x = kVariants[v];
  x.batch<<<grid, x.block, 0, st>>>(t, work);
}

}  // namespace owt

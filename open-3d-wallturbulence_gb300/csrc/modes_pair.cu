// Mode-kernel variants with the pair thread mapping (see modes_kernel.cuh).
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
    {"pair/128/r166", 128, k_modes<kVKL, kVKU, 6, 6, true, false, 128, 3>, k_modes_batch<kVKL, kVKU, 6, 6, true, false, 128, 3>},
    {"pair/128/r128", 128, k_modes<kVKL, kVKU, 6, 6, true, false, 128, 4>, k_modes_batch<kVKL, kVKU, 6, 6, true, false, 128, 4>},
    {"pair/256/r128", 256, k_modes<kVKL, kVKU, 6, 6, true, false, 256, 2>, k_modes_batch<kVKL, kVKU, 6, 6, true, false, 256, 2>},
};

// resident blocks of a batched kernel on the current device
int resident(void (*kernel)(BatchTable<ModeArgs>, int *), int block) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, 0);
  return (per > 0 ? per : 1) * (sms > 0 ? sms : 1);
}
}  // namespace

int modes_pair_count() { return (int)(sizeof(kVariants) / sizeof(kVariants[0])); }
const char *modes_pair_name(int v) { return kVariants[v].name; }
void modes_pair_launch(int v, const ModeArgs &a, cudaStream_t st) {
  const Variant &x = kVariants[v];
  const long long threads = 2 * (long long)a.M;
  x.kernel<<<(unsigned)((threads + x.block - 1) / x.block), x.block, 0, st>>>(a);
}

// full-band solve (used when a factorization falls outside the sparse masks)
void modes_dense_launch(const ModeArgs &a, cudaStream_t st) {
  const int bs = 128;
  k_modes<kVKL, kVKU, 6, 6, false, false, 128, 3><<<(unsigned)((2 * (long long)a.M + bs - 1) / bs), bs, 0, st>>>(a);
}

// masked solve with the sixth-order fill (one variant: the sixth-order option
// is not autotuned)
void modes_sixth_launch(const ModeArgs &a, cudaStream_t st) {
  const int bs = 128;
  k_modes<kVKL, kVKU, 6, 6, true, false, 128, 3, VMasks6><<<(unsigned)((2 * (long long)a.M + bs - 1) / bs), bs, 0, st>>>(a);
}

ModeBatchShape modes_pair_batch_shape(int v) {
  const Variant &x = kVariants[v];
  return {x.block, false, resident(x.batch, x.block)};
}
void modes_pair_batch_launch(int v, const BatchTable<ModeArgs> &t, int *work, int grid, cudaStream_t st) {
  const Variant &x = kVariants[v];
  x.batch<<<grid, x.block, 0, st>>>(t, work);
}

ModeBatchShape modes_dense_batch_shape() {
  return {128, false, resident(k_modes_batch<kVKL, kVKU, 6, 6, false, false, 128, 3>, 128)};
}
void modes_dense_batch_launch(const BatchTable<ModeArgs> &t, int *work, int grid, cudaStream_t st) {
  k_modes_batch<kVKL, kVKU, 6, 6, false, false, 128, 3><<<grid, 128, 0, st>>>(t, work);
}

}  // namespace owt

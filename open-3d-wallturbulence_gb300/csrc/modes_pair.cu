// Mode-kernel variants with the pair thread mapping (see modes_kernel.cuh).
#include "modes_kernel.cuh"

namespace owt {

namespace {
struct Variant {
  const char *name;
  int block;
  void (*kernel)(ModeArgs);
};
const Variant kVariants[] = {
    {"pair/128/r166", 128, k_modes<15, 13, 6, 6, true, false, 128, 3>},
    {"pair/128/r128", 128, k_modes<15, 13, 6, 6, true, false, 128, 4>},
    {"pair/256/r128", 256, k_modes<15, 13, 6, 6, true, false, 256, 2>},
};
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
  k_modes<15, 13, 6, 6, false, false, 128, 3><<<(unsigned)((2 * (long long)a.M + bs - 1) / bs), bs, 0, st>>>(a);
}

}  // namespace owt

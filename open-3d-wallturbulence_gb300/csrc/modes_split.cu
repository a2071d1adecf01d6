// Mode-kernel variants with the split mapping (see modes_kernel.cuh): an
// omega_y warp and a v warp per 16 modes, so that the v-system's forward
// sweep runs beside the omega_y solve.  Twice the threads of the pair
// mapping, each with a shorter sequential path: it pays where the modes are
// too few to fill the GPU (small channels), not where the FP64 pipe is full.
#include "modes_kernel.cuh"

namespace owt {

namespace {
struct Variant {
  const char *name;
  int block;
  void (*kernel)(ModeArgs);
};
const Variant kVariants[] = {
    {"split/64/r128", 64, k_modes_split<kVKL, kVKU, 6, 6, 64, 8>},
    {"split/128/r128", 128, k_modes_split<kVKL, kVKU, 6, 6, 128, 4>},
    {"split/64/r166", 64, k_modes_split<kVKL, kVKU, 6, 6, 64, 6>},
};
}  // namespace

int modes_split_count() { return (int)(sizeof(kVariants) / sizeof(kVariants[0])); }
const char *modes_split_name(int v) { return kVariants[v].name; }
void modes_split_launch(int v, const ModeArgs &a, cudaStream_t st) {
  const Variant &x = kVariants[v];
  const long long lanes = 2 * (long long)a.M;  // pair-mapping lanes; each has an omega_y and a v thread
  const int per_block = x.block / 2;
  x.kernel<<<(unsigned)((lanes + per_block - 1) / per_block), x.block, 0, st>>>(a);
}

}  // namespace owt

// Mode-kernel variants for single-channel launches only (batches choose
// among the pair and quad variants):
//  - the split mapping (see modes_kernel.cuh): an omega_y warp and a v warp
//    per 16 modes, so that the v-system's forward sweep runs beside the
//    omega_y solve.  Twice the threads of the pair mapping, each with a
//    shorter sequential path: it pays where the modes are too few to fill
//    the GPU (small channels), not where the FP64 pipe is full.
// (Measured and not kept: the pair and quad mappings in 224-thread blocks at
// 144 registers, about twice the time of the 128-register variants at
// 384x257x384.)
#include "modes_kernel.cuh"

namespace owt {

namespace {
enum Mapping { kSplit, kPair, kQuad };
struct Variant {
  const char *name;
  int block;
  Mapping mapping;
  void (*kernel)(ModeArgs);
};
const Variant kVariants[] = {
    {"split/64/r128", 64, kSplit, k_modes_split<kVKL, kVKU, 6, 6, 64, 8>},
    {"split/128/r128", 128, kSplit, k_modes_split<kVKL, kVKU, 6, 6, 128, 4>},
    {"split/64/r166", 64, kSplit, k_modes_split<kVKL, kVKU, 6, 6, 64, 6>},
};
}  // namespace

int modes_split_count() { return (int)(sizeof(kVariants) / sizeof(kVariants[0])); }
const char *modes_split_name(int v) { return kVariants[v].name; }
bool modes_split_is_quad(int v) { return kVariants[v].mapping == kQuad; }
void modes_split_launch(int v, const ModeArgs &a, cudaStream_t st) {
  const Variant &x = kVariants[v];
  long long threads;
  if (x.mapping == kSplit) threads = 2 * (2 * (long long)a.M);  // an omega_y and a v thread per pair-mapping lane
  else if (x.mapping == kPair) threads = 2 * (long long)a.M;
  else threads = 4 * (long long)(a.u1 - a.u0);
  x.kernel<<<(unsigned)((threads + x.block - 1) / x.block), x.block, 0, st>>>(a);
}

}  // namespace owt

// Mode-kernel variants with the quad thread mapping (see modes_kernel.cuh).
#include "modes_kernel.cuh"

namespace owt {

namespace {
struct Variant {
  const char *name;
  int block;
  void (*kernel)(ModeArgs);
};
const Variant kVariants[] = {
    {"quad/128/r166", 128, k_modes<15, 13, 6, 6, true, true, 128, 3>},
    {"quad/128/r128", 128, k_modes<15, 13, 6, 6, true, true, 128, 4>},
    {"quad/256/r128", 256, k_modes<15, 13, 6, 6, true, true, 256, 2>},
};
}  // namespace

int modes_quad_count() { return (int)(sizeof(kVariants) / sizeof(kVariants[0])); }
const char *modes_quad_name(int v) { return kVariants[v].name; }
void modes_quad_launch(int v, const ModeArgs &a, cudaStream_t st) {
  const Variant &x = kVariants[v];
  const long long threads = 4 * (long long)a.U;
  x.kernel<<<(unsigned)((threads + x.block - 1) / x.block), x.block, 0, st>>>(a);
}

}  // namespace owt

// Argument tables of the batched launches.  In a batch step every kernel of
// the time step covers all channels of a group in one launch: block b belongs
// to channel c with start[c] <= b < start[c + 1] and runs that channel's
// per-block body with the local block index b - start[c].  The table travels
// as a __grid_constant__ kernel parameter (read-only, no per-thread copy), so
// it is read through the constant cache with a block-uniform index.
#pragma once
#include <cuda_runtime.h>

namespace owt {

constexpr int kBatchChannels = 64;  // channels per launch (kernel parameters stay below 32 KB)

template <class A>
struct BatchTable {
  int n;                          // channels in this launch
  int start[kBatchChannels + 1];  // first block of each channel; start[n] = blocks in total
  A a[kBatchChannels];
};

// channel of block b: the last c with start[c] <= b (start is increasing)
__device__ __forceinline__ int batch_channel(const int *start, int n, int b) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Step counters of every channel of a batch (one thread each).
struct StepCounters {
  int n;
  long long *p[kBatchChannels];
};

}  // namespace owt

// gas_grid.cuh -- helpers of the persistent cooperative kernels (the small-
// graph BFS, the push tail): a grid barrier whose wait is bounded, and warp-
// aggregated counters.  Not installed.
#ifndef GAS_GRID_CUH_
#define GAS_GRID_CUH_

#include <cuda_runtime.h>

namespace gasgrid {

// x 64 ns back-off: a wait gives up after about a second
constexpr long long kMaxSpins = 1LL << 24;

// The barrier's state (zeroed before the launch).  err != 0 makes every CTA
// leave: 1 is written here when a wait gives up.
struct Barrier {
  unsigned int count;
  unsigned int gen;
  int err;
  int pad;
};

// Every CTA of a cooperative launch calls it; one atomic per CTA.  Returns
// false once err is set, and the caller leaves the kernel.  err is read
// after the release, so a CTA still leaving one barrier sees a value that
// another CTA wrote after passing it: write err only to end the kernel
// with an error, never as a signal the kernel goes on from (an iteration
// cap, say).
__device__ __forceinline__ bool barrier(Barrier *b) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int *gen = &b->gen;
    const unsigned int g = *gen;
    __threadfence();
    if (atomicAdd(&b->count, 1u) == gridDim.x - 1) {
      b->count = 0;
      __threadfence();
      atomicAdd(&b->gen, 1u);
    } else {
      long long spins = 0;
      while (*gen == g) {
        if (++spins > kMaxSpins) {
          atomicExch(&b->err, 1);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *(volatile int *)&b->err == 0;
}

__device__ __forceinline__ long long warp_sum(long long v) {
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
  return v;
}

__device__ __forceinline__ int warp_incl_sum(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int o = __shfl_up_sync(0xffffffffu, v, d);
    if (lane >= d) v += o;
  }
  return v;
}

// Adds a per-thread count to *dst, one atomic per warp (all lanes call).
__device__ __forceinline__ void warp_add(long long v, long long *dst) {
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0 && v)
    atomicAdd((unsigned long long *)dst, (unsigned long long)v);
}

}  // namespace gasgrid

#endif  // GAS_GRID_CUH_

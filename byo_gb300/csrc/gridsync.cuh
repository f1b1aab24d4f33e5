// gridsync.cuh -- a bounded grid barrier for cooperative (co-resident) launches.
//
// Blocks count in with an atomic; the last one resets the count and bumps a
// generation word the others spin on.  A wait that lasts longer than the
// barrier's limit (limit_ms, 0 = kBarrierNs) or finds the error word set by
// another block sets the error word and returns false, so every block leaves
// instead of spinning forever.  `extra` raises the number of arrivals the
// barrier waits for beyond the blocks launched: a test sets it to 1 (with a
// short limit) so that the wait runs out and the error path is exercised.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace byo {

constexpr uint64_t kBarrierNs = 4000000000ull;  // 4 s

struct GridBar {
  unsigned int count, gen, err;
  unsigned int limit_ms;  // 0: kBarrierNs
  unsigned int extra;     // arrivals awaited beyond the launched blocks (tests only)
  unsigned int pad[3];
};

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool grid_sync(GridBar *b, unsigned int nblocks) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    volatile unsigned int *gen = &b->gen;
    const unsigned int g = *gen;
    __threadfence();
    const unsigned int need = nblocks + b->extra;
    const uint64_t limit = b->limit_ms ? (uint64_t)b->limit_ms * 1000000ull : kBarrierNs;
    if (atomicAdd(&b->count, 1u) == need - 1) {
      b->count = 0;
      __threadfence();
      atomicAdd(&b->gen, 1u);
    } else {
      const uint64_t t0 = globaltimer_ns();
      while (*gen == g) {
        if (*(volatile unsigned int *)&b->err || globaltimer_ns() - t0 > limit) {
          atomicOr(&b->err, 1u);
          ok = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

}  // namespace byo

// device.cuh -- small device-side building blocks shared by the kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace byo {

constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_inclusive_scan(T v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T t = __shfl_up_sync(kFull, v, o);
    if (lane_id() >= (unsigned)o) v += t;
  }
  return v;
}

// Exclusive block scan of one value per thread; returns the prefix and the
// block total.  smem must hold blockDim.x/32 + 1 elements.  All threads call.
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T *smem, T *total) {
  const unsigned w = threadIdx.x >> 5, l = lane_id(), nw = blockDim.x >> 5;
  T inc = warp_inclusive_scan(v);
  if (l == 31) smem[w] = inc;
  __syncthreads();
  if (w == 0) {
    T s = (l < nw) ? smem[l] : T(0);
    T si = warp_inclusive_scan(s);
    if (l < nw) smem[l] = si - s;
    if (l == nw - 1) smem[nw] = si;
  }
  __syncthreads();
  T res = smem[w] + inc - v;
  *total = smem[nw];
  __syncthreads();
  return res;
}

template <typename T>
__device__ __forceinline__ T block_sum(T v, T *smem) {
  const unsigned w = threadIdx.x >> 5, l = lane_id(), nw = blockDim.x >> 5;
  v = warp_sum(v);
  if (l == 0) smem[w] = v;
  __syncthreads();
  T r = T(0);
  if (w == 0) {
    r = (l < nw) ? smem[l] : T(0);
    r = warp_sum(r);
  }
  __syncthreads();
  return r;  // valid in thread 0
}

// Warp-aggregated append of `pred` items to a global list; returns the slot
// for this lane (undefined when !pred).
__device__ __forceinline__ uint64_t warp_append(bool pred, unsigned long long *counter) {
  unsigned mask = __ballot_sync(kFull, pred);
  if (!mask) return 0;
  unsigned leader = __ffs(mask) - 1;
  unsigned long long base = 0;
  if (lane_id() == leader) base = atomicAdd(counter, (unsigned long long)__popc(mask));
  base = __shfl_sync(kFull, base, leader);
  return base + __popc(mask & lanemask_lt());
}

__device__ __forceinline__ bool test_bit(const uint32_t *bits, uint32_t v) {
  return (__ldg(bits + (v >> 5)) >> (v & 31)) & 1u;
}
// Bit test that may read a stale bitmap written by an earlier launch only.
__device__ __forceinline__ bool test_bit_cg(const uint32_t *bits, uint32_t v) {
  return (__ldcg(bits + (v >> 5)) >> (v & 31)) & 1u;
}

// Bitonic sort of R*32 keys held by a warp in registers: element r*32 + lane
// lives in register r of that lane; strides below 32 exchange through
// shuffles, larger strides swap registers inside a lane.
template <int R>
__device__ __forceinline__ void warp_bitonic(uint64_t (&v)[R]) {
  const unsigned lane = lane_id();
#pragma unroll
  for (int size = 2; size <= R * 32; size <<= 1) {
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      if (stride >= 32) {
        const int rs = stride / 32;
#pragma unroll
        for (int r = 0; r < R; r++) {
          if ((r & rs) == 0) {
            const bool up = ((r * 32) & size) == 0;
            const uint64_t x = v[r], y = v[r ^ rs];
            if ((x > y) == up) {
              v[r] = y;
              v[r ^ rs] = x;
            }
          }
        }
      } else {
#pragma unroll
        for (int r = 0; r < R; r++) {
          const unsigned i = r * 32 + lane;
          const uint64_t x = v[r];
          const uint64_t y = __shfl_xor_sync(kFull, x, stride);
          const bool up = (i & size) == 0, lower = (lane & stride) == 0;
          const uint64_t lo = x < y ? x : y, hi = x < y ? y : x;
          v[r] = (lower == up) ? lo : hi;
        }
      }
    }
  }
}

}  // namespace byo

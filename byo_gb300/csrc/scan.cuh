// scan.cuh -- tiled device-wide exclusive scan with a pluggable input and
// output, used for frontier degree prefixes, stream compaction and radix-sort
// digit offsets (the roles parlay::scan / parlay::pack play in the reference,
// gbbs/bridge.h:208-313).
//
// Three launches: per-tile sums, one block scanning the tile sums, per-tile
// scan that hands (index, exclusive prefix, value) to the output functor.
// Tiles are SCAN_TILE items; loads go through shared memory so global reads
// stay coalesced while each thread scans a contiguous run.
#pragma once

#include "device.cuh"
#include "internal.h"

namespace byo {

constexpr int SCAN_BLOCK = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

template <class In>
__global__ void __launch_bounds__(SCAN_BLOCK) k_scan_reduce(In in, uint64_t count, uint64_t *partial) {
  __shared__ uint64_t sm[SCAN_BLOCK / 32 + 1];
  const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
  uint64_t s = 0;
#pragma unroll 4
  for (int k = 0; k < SCAN_ITEMS; k++) {
    uint64_t i = base + (uint64_t)k * SCAN_BLOCK + threadIdx.x;
    if (i < count) s += in(i);
  }
  s = block_sum(s, sm);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// Exclusive scan of partial[0..nt) in place; partial[nt] = total.  One block
// of 1024 threads, each owning a contiguous run.
template <int kUnused = 0>
__global__ void __launch_bounds__(1024) k_scan_partials(uint64_t *partial, uint64_t nt) {
  __shared__ uint64_t sm[1024 / 32 + 1];
  const uint64_t per = (nt + blockDim.x - 1) / blockDim.x;
  const uint64_t lo = threadIdx.x * per;
  const uint64_t hi = lo + per < nt ? lo + per : nt;
  uint64_t s = 0;
  for (uint64_t i = lo; i < hi; i++) s += partial[i];
  uint64_t tot;
  uint64_t pre = block_exclusive_scan(s, sm, &tot);
  for (uint64_t i = lo; i < hi; i++) {
    uint64_t t = partial[i];
    partial[i] = pre;
    pre += t;
  }
  if (threadIdx.x == 0) partial[nt] = tot;
}

template <class In, class Out>
__global__ void __launch_bounds__(SCAN_BLOCK) k_scan_apply(In in, Out out, uint64_t count,
                                                           const uint64_t *partial) {
  __shared__ uint64_t items[SCAN_TILE + SCAN_TILE / 32];
  __shared__ uint64_t sm[SCAN_BLOCK / 32 + 1];
  const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
#pragma unroll 4
  for (int k = 0; k < SCAN_ITEMS; k++) {
    uint32_t j = k * SCAN_BLOCK + threadIdx.x;
    uint64_t i = base + j;
    items[j + (j >> 5)] = i < count ? in(i) : 0;
  }
  __syncthreads();
  uint64_t v[SCAN_ITEMS];
  uint64_t s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    uint32_t j = threadIdx.x * SCAN_ITEMS + k;
    v[k] = items[j + (j >> 5)];
    s += v[k];
  }
  uint64_t tot;
  uint64_t pre = block_exclusive_scan(s, sm, &tot) + partial[blockIdx.x];
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    uint64_t i = base + (uint64_t)threadIdx.x * SCAN_ITEMS + k;
    if (i < count) out(i, pre, v[k]);
    pre += v[k];
  }
}

// Runs the scan; the total ends up in device memory at *d_total_slot (the
// last entry of the partial array, returned through d_total).
template <class In, class Out>
int scan_apply(byo_ctx *ctx, uint64_t count, In in, Out out, const uint64_t **d_total) {
  uint64_t nt = (count + SCAN_TILE - 1) / SCAN_TILE;
  if (nt == 0) nt = 1;
  uint64_t *partial = nullptr;
  BYO_TRY(scratch(ctx, 7, nt + 1, &partial));
  if (count > 0) {
    launch(ctx, k_scan_reduce<In>, dim3((unsigned)nt), dim3(SCAN_BLOCK), 0, in, count, partial);
    launch(ctx, k_scan_partials<0>, dim3(1), dim3(1024), 0, partial, nt);
    launch(ctx, k_scan_apply<In, Out>, dim3((unsigned)nt), dim3(SCAN_BLOCK), 0, in, out, count,
           (const uint64_t *)partial);
  } else {
    BYO_CU(ctx, cudaMemsetAsync(partial, 0, 2 * sizeof(uint64_t), ctx->stream));
    nt = 0;
  }
  if (d_total) *d_total = partial + nt;
  return check_launch(ctx, "scan");
}

// ---------------------------------------------------------------- functors
struct InU32 {
  const uint32_t *p;
  __device__ uint64_t operator()(uint64_t i) const { return p[i]; }
};
struct InU64 {
  const uint64_t *p;
  __device__ uint64_t operator()(uint64_t i) const { return p[i]; }
};
struct InDegOfList {
  const uint32_t *deg;
  const uint32_t *list;
  __device__ uint64_t operator()(uint64_t i) const { return deg[list[i]]; }
};
struct InRangeOfList {
  const uint64_t *off;
  const uint32_t *list;
  __device__ uint64_t operator()(uint64_t i) const {
    uint32_t v = list[i];
    return off[v + 1] - off[v];
  }
};
struct OutPrefix {
  uint64_t *out;
  __device__ void operator()(uint64_t i, uint64_t pre, uint64_t) const { out[i] = pre; }
};

}  // namespace byo

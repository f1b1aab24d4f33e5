// map.cu -- the neighbour-map benchmarks of run_all.
//
//   Test_Map (benchmarks/Map/Base/Map.h:8-18): the sum over every edge
//     (u, v) of v.
//   Test_Map_Remote (benchmarks/Map/RemoteRead/Map.h:21-33, run by
//     Map_Remote_runner<G, W>, benchmarks/run_unweighted.h:50-126): the sum
//     over every edge (u, v) of remote[v] for an n-entry array of W-byte
//     elements (W = 0: std::vector<bool>; 16, 32: wide_int<size_t, W>, a
//     size_t padded to W bytes).
//
// Both scan the container's own slot array -- the CSR's ids, or the PMA's
// leaves with their gaps -- which is what the reference times: how fast a
// container maps its neighbours.  The ids stream once with 16-byte loads
// (evict-first); the remote reads are the gathers.  Integer sums, so the
// result does not depend on the order of the block partials.
#include "device.cuh"
#include "internal.h"

namespace byo {

// Element v of the remote array; kId: v itself (Test_Map).
template <int W>
__device__ __forceinline__ uint64_t remote_value(uint32_t v, const unsigned char *__restrict__ r) {
  if (v == kSentinel) return 0;
  if constexpr (W < 0) {
    return v;
  } else if constexpr (W == 0) {  // bit v of 64-bit word v / 64, least significant bit first
    return (__ldg(reinterpret_cast<const unsigned long long *>(r) + (v >> 6)) >> (v & 63)) & 1ull;
  } else if constexpr (W == 1) {
    return __ldg(r + v);
  } else if constexpr (W == 2) {
    return __ldg(reinterpret_cast<const unsigned short *>(r) + v);
  } else if constexpr (W == 4) {
    return __ldg(reinterpret_cast<const unsigned int *>(r) + v);
  } else {  // 8, 16, 32: an unsigned 64-bit value at the start of the element
    return __ldg(reinterpret_cast<const unsigned long long *>(r + (uint64_t)v * W));
  }
}

template <int W>
__global__ void __launch_bounds__(256) k_map_sum(const uint32_t *__restrict__ slots, uint64_t nslots,
                                                 const unsigned char *__restrict__ remote,
                                                 unsigned long long *out) {
  __shared__ unsigned long long sm[9];
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  const uint64_t nthr = (uint64_t)gridDim.x * blockDim.x;
  unsigned long long acc = 0;
  const uint64_t n4 = nslots / 4;
  const uint4 *s4 = reinterpret_cast<const uint4 *>(slots);
  for (uint64_t i = tid; i < n4; i += nthr) {
    const uint4 q = __ldcs(s4 + i);
    acc += remote_value<W>(q.x, remote) + remote_value<W>(q.y, remote) + remote_value<W>(q.z, remote) +
           remote_value<W>(q.w, remote);
  }
  for (uint64_t i = 4 * n4 + tid; i < nslots; i += nthr) acc += remote_value<W>(slots[i], remote);
  acc = block_sum(acc, sm);
  if (threadIdx.x == 0 && acc) atomicAdd(out, acc);
}

// Random 4-byte gathers from a table of `words` uint32: each thread draws
// kGatherBatch independent indices per round from a counter-based hash and
// keeps every loaded value in its sum, so all loads are live.  The rate this
// sustains is the ceiling of a kernel whose time goes to one-word random
// gathers from an L2-resident array (PageRank's pull).
constexpr int kGatherBatch = 16;
__device__ __forceinline__ uint32_t gather_hash(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return (uint32_t)x;
}

__global__ void __launch_bounds__(256) k_gather_roof(const uint32_t *__restrict__ table, uint64_t words,
                                                     uint32_t rounds, unsigned long long *out) {
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  unsigned long long acc = 0;
  for (uint32_t r = 0; r < rounds; r++) {
    uint32_t v[kGatherBatch];
#pragma unroll
    for (int q = 0; q < kGatherBatch; q++)
      v[q] = __ldg(table + gather_hash((tid * rounds + r) * kGatherBatch + q) % words);
#pragma unroll
    for (int q = 0; q < kGatherBatch; q++) acc += v[q];
  }
  if (acc == 0x5eedull) out[0] = acc;  // keeps the loads alive
}

int gather_roof(byo_ctx *ctx, uint64_t table_bytes, double *gathers_per_s) {
  const uint64_t words = table_bytes / 4;
  if (words < 1024) return set_error(ctx, BYO_EINVAL, "gather roof: table of at least 4 KiB");
  uint32_t *table = nullptr;
  unsigned long long *out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = BYO_OK;
  if (cudaMalloc(&table, words * 4) != cudaSuccess || cudaMalloc(&out, 8) != cudaSuccess) {
    cudaGetLastError();
    rc = set_error(ctx, BYO_ENOMEM, "gather roof: table");
  }
  if (rc == BYO_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
    rc = set_error(ctx, BYO_EDEVICE, "gather roof: events");
  if (rc == BYO_OK && cudaMemsetAsync(table, 1, words * 4, ctx->stream) != cudaSuccess)
    rc = set_error(ctx, BYO_EDEVICE, "gather roof: table fill");
  if (rc == BYO_OK) {
    const dim3 grid(ctx->num_sms * 8), block(256);
    const uint32_t rounds = 64;
    const double gathers = (double)grid.x * block.x * rounds * kGatherBatch;
    launch(ctx, k_gather_roof, grid, block, 0, (const uint32_t *)table, words, rounds, out);  // warm
    float best = 1e30f;
    for (int rep = 0; rep < 5 && rc == BYO_OK; rep++) {
      cudaEventRecord(e0, ctx->stream);
      launch(ctx, k_gather_roof, grid, block, 0, (const uint32_t *)table, words, rounds, out);
      cudaEventRecord(e1, ctx->stream);
      float ms = 0.f;
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
        rc = set_error(ctx, BYO_EDEVICE, "gather roof: timing");
      else if (ms < best)
        best = ms;
    }
    if (rc == BYO_OK) *gathers_per_s = gathers / (best / 1e3);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamSynchronize(ctx->stream);
  if (table) cudaFree(table);
  if (out) cudaFree(out);
  return rc == BYO_OK ? check_launch(ctx, "gather roof") : rc;
}

uint64_t map_remote_bytes(uint64_t n, uint32_t width) {
  return width == 0 ? (n + 63) / 64 * 8 : n * width;
}

// width: -1 for Test_Map, else a Test_Map_Remote element width.
int map_run(byo_graph *g, int width, const void *d_remote, uint64_t *sum) {
  byo_ctx *ctx = g->ctx;
  *sum = 0;
  if (!g->nslots) return BYO_OK;
  unsigned long long *acc = nullptr;
  BYO_TRY(ws(g, WS_MISC, 1, (uint64_t **)&acc));
  BYO_CU(ctx, cudaMemsetAsync(acc, 0, 8, ctx->stream));
  const dim3 grid(grid_for(ctx, (g->nslots + 3) / 4, 256, 8)), block(256);
  const unsigned char *r = static_cast<const unsigned char *>(d_remote);
  const uint32_t *s = g->d_slots;
  switch (width) {
    case -1: launch_t(ctx, "map", k_map_sum<-1>, grid, block, 0, s, g->nslots, r, acc); break;
    case 0: launch_t(ctx, "map", k_map_sum<0>, grid, block, 0, s, g->nslots, r, acc); break;
    case 1: launch_t(ctx, "map", k_map_sum<1>, grid, block, 0, s, g->nslots, r, acc); break;
    case 2: launch_t(ctx, "map", k_map_sum<2>, grid, block, 0, s, g->nslots, r, acc); break;
    case 4: launch_t(ctx, "map", k_map_sum<4>, grid, block, 0, s, g->nslots, r, acc); break;
    case 8: launch_t(ctx, "map", k_map_sum<8>, grid, block, 0, s, g->nslots, r, acc); break;
    case 16: launch_t(ctx, "map", k_map_sum<16>, grid, block, 0, s, g->nslots, r, acc); break;
    case 32: launch_t(ctx, "map", k_map_sum<32>, grid, block, 0, s, g->nslots, r, acc); break;
    default: return set_error(ctx, BYO_EINVAL, "map: remote width must be 0, 1, 2, 4, 8, 16 or 32");
  }
  uint64_t *h = nullptr;
  BYO_TRY(pinned(ctx, 4096, (void **)&h));
  BYO_CU(ctx, cudaMemcpyAsync(h, acc, 8, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  *sum = h[0];
  return check_launch(ctx, "map");
}

}  // namespace byo

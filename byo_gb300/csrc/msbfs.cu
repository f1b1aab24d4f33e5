// msbfs.cu -- 64-source BFS packed into bit lanes, run by one persistent
// cooperative kernel.
//
// Each vertex carries three 64-bit masks: seen (sources that reached it),
// F (sources whose frontier holds it this round) and N (next round).  A round
// is a pull over every vertex that still misses some source: OR the F masks of
// its neighbours, stopping once every missing bit is found; the new bits go to
// N and seen, and the round number is written as the level of each new
// (source, vertex) pair.  BFS levels do not depend on the order of these ORs,
// so every source's levels equal those of a single-source BFS (BFS.h:47-64)
// from it.  Rounds are separated by a grid barrier of the project's own
// (bounded spin: a barrier that does not complete sets an error flag and every
// block leaves), so one launch runs the whole traversal without returning to
// the host.
#include <algorithm>
#include <vector>

#include "device.cuh"
#include "internal.h"

namespace byo {

constexpr int kMsBlock = 256;
constexpr uint32_t kBarrierSpins = 1u << 22;

struct GridBarrier {
  unsigned int count;
  unsigned int gen;
  unsigned int err;
  unsigned int changed[2];
  unsigned int rounds;
};

// Sense-counting barrier across all blocks of a cooperative launch.  Returns
// false (and sets gb->err) when the other blocks did not arrive in time.
__device__ __forceinline__ bool grid_sync(GridBarrier *gb, unsigned int nblocks) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    volatile unsigned int *gen = &gb->gen;
    const unsigned int g = *gen;
    __threadfence();
    const unsigned int arrived = atomicAdd(&gb->count, 1u);
    if (arrived == nblocks - 1) {
      gb->count = 0;
      __threadfence();
      atomicAdd(&gb->gen, 1u);
    } else {
      uint32_t spins = 0;
      while (*gen == g) {
        if (++spins > kBarrierSpins || *(volatile unsigned int *)&gb->err) {
          atomicOr(&gb->err, 1u);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

__global__ void k_ms_init(uint64_t *seen, uint64_t *F, uint64_t *N, uint16_t *lvl, uint64_t n,
                          const uint32_t *__restrict__ srcs, uint32_t k, GridBarrier *gb) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n * 64;
       i += (uint64_t)gridDim.x * blockDim.x) {
    lvl[i] = 0xFFFF;
    if (i < n) {
      seen[i] = 0;
      F[i] = 0;
      N[i] = 0;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    gb->count = 0;
    gb->gen = 0;
    gb->err = 0;
    gb->changed[0] = gb->changed[1] = 0;
  }
}

__global__ void k_ms_seed(uint64_t *seen, uint64_t *F, uint16_t *lvl, const uint32_t *__restrict__ srcs, uint32_t k) {
  // one thread: sources may repeat
  if (blockIdx.x == 0 && threadIdx.x == 0)
    for (uint32_t s = 0; s < k; s++) {
      seen[srcs[s]] |= 1ull << s;
      F[srcs[s]] |= 1ull << s;
      lvl[(uint64_t)srcs[s] * 64 + s] = 0;
    }
}

__global__ void __launch_bounds__(kMsBlock) k_ms_bfs(const uint64_t *__restrict__ off,
                                                     const uint32_t *__restrict__ slots, uint64_t n,
                                                     uint64_t full, uint64_t *seen, uint64_t *Fa, uint64_t *Fb,
                                                     uint16_t *lvl, GridBarrier *gb, uint32_t max_rounds,
                                                     uint32_t *rounds_out) {
  const unsigned int nblocks = gridDim.x;
  uint64_t *F = Fa, *N = Fb;
  uint32_t r = 1;
  for (; r <= max_rounds; r++) {
    unsigned int any = 0;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
      const uint64_t sv = seen[v];
      const uint64_t need = full & ~sv;
      uint64_t got = 0;
      if (need) {
        const uint64_t b = off[v], e = off[v + 1];
        for (uint64_t j = b; j < e; j++) {
          const uint32_t u = slots[j];
          if (u == kSentinel) continue;
          got |= __ldcg(F + u);
          if ((got & need) == need) break;
        }
        got &= need;
      }
      N[v] = got;
      if (got) {
        seen[v] = sv | got;
        any = 1;
        uint64_t bits = got;
        while (bits) {
          const int s = __ffsll((long long)bits) - 1;
          bits &= bits - 1;
          lvl[v * 64 + s] = (uint16_t)r;
        }
      }
    }
    if (__syncthreads_or(any) && threadIdx.x == 0) atomicOr(&gb->changed[r & 1], 1u);
    if (!grid_sync(gb, nblocks)) return;
    const unsigned int changed = *(volatile unsigned int *)&gb->changed[r & 1];
    if (blockIdx.x == 0 && threadIdx.x == 0) gb->changed[(r + 1) & 1] = 0;
    if (!changed) break;
    uint64_t *t = F;
    F = N;
    N = t;
    if (!grid_sync(gb, nblocks)) return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *rounds_out = r;
}

// lvl (vertex-major, uint16) -> levels[s * n + v] (uint32, BYO_NONE unreached)
__global__ void k_ms_levels(const uint16_t *__restrict__ lvl, uint64_t n, uint32_t k, uint32_t *levels) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n * k; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t s = i / n, v = i % n;
    const uint16_t x = lvl[v * 64 + s];
    levels[i] = x == 0xFFFF ? kSentinel : (uint32_t)x;
  }
}

int bfs_multi_run(byo_graph *g, const uint32_t *h_srcs, uint32_t k, uint32_t *d_levels, uint32_t *rounds) {
  byo_ctx *ctx = g->ctx;
  const uint64_t n = g->n;
  if (k == 0 || k > 64) return set_error(ctx, BYO_EINVAL, "bfs_multi: 1 <= k <= 64 sources");
  for (uint32_t s = 0; s < k; s++)
    if (h_srcs[s] >= n) return set_error(ctx, BYO_EINVAL, "bfs_multi: source >= n");
  uint64_t *seen, *Fa, *Fb;
  uint16_t *lvl;
  uint32_t *srcs;
  GridBarrier *gb;
  BYO_TRY(ws(g, WS_LP, 3 * n + 2, &seen));  // seen | Fa | Fb
  Fa = seen + n;
  Fb = Fa + n;
  BYO_TRY(ws(g, WS_PR_A, n * 64 / 2 + 2, (uint32_t **)&lvl));
  BYO_TRY(ws(g, WS_MISC, 64 + sizeof(GridBarrier) / 4 + 4, &srcs));  // sources, then the barrier
  gb = (GridBarrier *)(srcs + 64);
  BYO_CU(ctx, cudaMemcpyAsync(srcs, h_srcs, k * 4, cudaMemcpyHostToDevice, ctx->stream));
  launch(ctx, k_ms_init, dim3(grid_for(ctx, n * 64, 256, 16)), dim3(256), 0, seen, Fa, Fb, lvl, n,
         (const uint32_t *)srcs, k, gb);
  launch(ctx, k_ms_seed, dim3(1), dim3(32), 0, seen, Fa, lvl, (const uint32_t *)srcs, k);
  // co-resident grid for the cooperative launch
  int per_sm = 0;
  BYO_CU(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ms_bfs, kMsBlock, 0));
  if (per_sm < 1) return set_error(ctx, BYO_EDEVICE, "bfs_multi: kernel cannot be resident");
  const unsigned int grid = (unsigned int)std::min<uint64_t>((uint64_t)per_sm * ctx->num_sms,
                                                            (n + kMsBlock - 1) / kMsBlock);
  uint64_t full = k == 64 ? ~0ull : ((1ull << k) - 1);
  uint32_t max_rounds = 0xFFFE;  // levels are stored in 16 bits
  uint32_t *d_rounds = &gb->rounds;
  const uint64_t *off = g->d_off;
  const uint32_t *slots = g->d_slots;
  void *args[] = {(void *)&off, (void *)&slots, (void *)&n, (void *)&full, (void *)&seen, (void *)&Fa, (void *)&Fb,
                  (void *)&lvl, (void *)&gb, (void *)&max_rounds, (void *)&d_rounds};
  BYO_CU(ctx, cudaLaunchCooperativeKernel((const void *)k_ms_bfs, dim3(grid), dim3(kMsBlock), args, 0, ctx->stream));
  ctx->launches++;
  unsigned int h[2] = {0, 0};
  BYO_CU(ctx, cudaMemcpyAsync(&h[0], &gb->err, 4, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaMemcpyAsync(&h[1], d_rounds, 4, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  if (h[0]) return set_error(ctx, BYO_ETIMEDOUT, "bfs_multi: grid barrier timed out");
  if (rounds) *rounds = h[1];
  launch(ctx, k_ms_levels, dim3(grid_for(ctx, n * k, 256, 16)), dim3(256), 0, (const uint16_t *)lvl, n, k, d_levels);
  return check_launch(ctx, "bfs_multi");
}

}  // namespace byo

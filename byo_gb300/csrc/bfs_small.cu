// bfs_small.cu -- consecutive small push rounds of a BFS in one persistent
// cooperative kernel.
//
// A push round over a frontier of a few thousand edges takes a few
// microseconds of GPU work, but driving it from the host (launches, a copy of
// the round statistics, a stream synchronisation) costs several times that.
// On graphs of high diameter (grids, road-like graphs) nearly every round is
// like that.  This kernel runs such rounds back to back, separated by a grid
// barrier, with the same visit rule as the push kernels (BFS_F's
// updateAtomic keeping the smallest (level, parent), BFS.h:30-45), so the
// result does not depend on which rounds it ran.  It leaves as soon as the
// next frontier is empty, grows past `limit` edges or holds a vertex of
// degree >= 4^5 (the round kernels give such vertices whole CTAs, and the
// learned policy inspects such frontiers), and hands the host the frontier in
// the engine's form (list + bitmap, its size, out-degree and degree sketch),
// so the round loop continues from there.
#include <algorithm>
#include <cstring>
#include <vector>

#include "device.cuh"
#include "engine.h"
#include "gridsync.cuh"
#include "internal.h"

namespace byo {

constexpr int kSmallBlock = 256;
constexpr uint32_t kSmallLog = 1u << 16;  // rounds one launch may run (and log)

struct SmallCtl {
  GridBar bar;
  unsigned long long cnt[2], outdeg[2], hist[2][8];
  unsigned int hub[2];
  unsigned int rounds, final_idx;
};

struct SmallArgs {
  const uint64_t *off;
  const uint32_t *slots;
  const uint32_t *deg;
  uint64_t *lp;
  uint32_t *visited;
  uint32_t *list[2];
  uint32_t *bits[2];
  uint64_t limit;
  uint32_t round0;
  int gate_hub;
  SmallCtl *ctl;
  unsigned long long *log;  // per round: |F| and its out-degree, 2 words
};

__device__ __forceinline__ int small_bin(uint32_t d) {
  int b = d ? (31 - __clz(d)) / 2 : 0;
  return b > 7 ? 7 : b;
}

__global__ void __launch_bounds__(kSmallBlock) k_bfs_small(SmallArgs a) {
  SmallCtl *c = a.ctl;
  const unsigned nb = gridDim.x;
  const unsigned lane = threadIdx.x & 31;
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t nthr = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t warp = tid >> 5, nwarps = nthr >> 5;
  int cur = 0;
  uint64_t f = *(volatile unsigned long long *)&c->cnt[0];
  uint32_t *const L0 = a.list[0], *const L1 = a.list[1], *const B0 = a.bits[0], *const B1 = a.bits[1];
  for (uint32_t r = 0; r < kSmallLog; r++) {
    const int nxt = cur ^ 1;
    uint32_t *const Lc = cur ? L1 : L0, *const Ln = cur ? L0 : L1;
    uint32_t *const Bc = cur ? B1 : B0, *const Bn = cur ? B0 : B1;
    const uint64_t lvl = (uint64_t)(a.round0 + r) << 32;
    // push: a warp per frontier vertex
    uint64_t dsum = 0;
    for (uint64_t i = warp; i < f; i += nwarps) {
      const uint32_t u = __ldcg(Lc + i);
      const uint64_t b = a.off[u], e = a.off[u + 1];
      for (uint64_t base = b; base < e; base += 32) {
        const uint64_t j = base + lane;
        bool first = false;
        uint32_t v = kSentinel;
        if (j < e) {
          v = a.slots[j];
          if (v != kSentinel && !((__ldcg(a.visited + (v >> 5)) >> (v & 31)) & 1u))
            first = atomicMin((unsigned long long *)(a.lp + v), (unsigned long long)(lvl | u)) == kNone64;
        }
        const uint64_t at = warp_append(first, &c->cnt[nxt]);
        uint32_t d = 0;
        if (first) {
          Ln[at] = v;
          atomicOr(Bn + (v >> 5), 1u << (v & 31));
          d = a.deg[v];
          dsum += d;
        }
        const unsigned any = __ballot_sync(kFull, first);
        if (any) {
          const int bin = small_bin(d);
#pragma unroll
          for (int q = 0; q < 8; q++) {
            const unsigned m = __ballot_sync(kFull, first && bin == q);
            if (m && lane == 0) atomicAdd(&c->hist[nxt][q], (unsigned long long)__popc(m));
          }
          if (__ballot_sync(kFull, first && bin >= 5) && lane == 0) atomicOr(&c->hub[nxt], 1u);
        }
      }
    }
    dsum = warp_sum(dsum);
    if (lane == 0 && dsum) atomicAdd(&c->outdeg[nxt], (unsigned long long)dsum);
    if (!grid_sync(&c->bar, nb)) return;
    // the new frontier becomes visited; the old one's bitmap is cleared (its
    // set bits all belong to its list) so the buffer can take a frontier again
    const uint64_t fn = *(volatile unsigned long long *)&c->cnt[nxt];
    const uint64_t dn = *(volatile unsigned long long *)&c->outdeg[nxt];
    const unsigned hub = *(volatile unsigned int *)&c->hub[nxt];
    for (uint64_t i = tid; i < fn; i += nthr) {
      const uint32_t v = __ldcg(Ln + i);
      atomicOr(a.visited + (v >> 5), 1u << (v & 31));
    }
    for (uint64_t i = tid; i < f; i += nthr) Bc[__ldcg(Lc + i) >> 5] = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.log[2 * r] = f;
      a.log[2 * r + 1] = dn;
      c->cnt[cur] = 0;
      c->outdeg[cur] = 0;
      c->hub[cur] = 0;
      for (int q = 0; q < 8; q++) c->hist[cur][q] = 0;
      c->rounds = r + 1;
      c->final_idx = (unsigned)nxt;
    }
    if (!grid_sync(&c->bar, nb)) return;
    if (fn == 0 || fn + dn > a.limit || (a.gate_hub && hub)) return;
    cur = nxt;
    f = fn;
  }
}

int bfs_small_rounds(byo_graph *g, TravState &st, Frontier *&cur, Frontier *&nxt, uint64_t limit, bool gate_hub,
                     RoundStats *d_st, uint32_t *rounds_run) {
  byo_ctx *ctx = g->ctx;
  *rounds_run = 0;
  SmallCtl *c = nullptr;
  BYO_TRY(ws(g, WS_MISC, sizeof(SmallCtl) / 8 + 2, (uint64_t **)&c));
  unsigned long long *logb = nullptr;
  BYO_TRY(ws(g, WS_BUCKETS, 2ull * kSmallLog, (uint64_t **)&logb));
  // the current frontier's counts seed slot 0; the bitmap of `nxt` is clean
  SmallCtl *h = nullptr;
  BYO_TRY(pinned(ctx, std::max<size_t>(sizeof(SmallCtl), 4096), (void **)&h));
  std::memset(h, 0, sizeof(SmallCtl));
  h->cnt[0] = cur->size;
  h->outdeg[0] = cur->outdeg;
  h->bar.limit_ms = ctx->bar_limit_ms;
  h->bar.extra = ctx->bar_extra;
  BYO_CU(ctx, cudaMemcpyAsync(c, h, sizeof(SmallCtl), cudaMemcpyHostToDevice, ctx->stream));
  SmallArgs a;
  a.off = g->d_off;
  a.slots = g->d_slots;
  a.deg = g->d_deg;
  a.lp = st.lp;
  a.visited = st.visited;
  a.list[0] = cur->list;
  a.list[1] = nxt->list;
  a.bits[0] = cur->bits;
  a.bits[1] = nxt->bits;
  a.limit = limit;
  a.round0 = st.round;
  a.gate_hub = gate_hub ? 1 : 0;
  a.ctl = c;
  a.log = logb;
  int per_sm = 0;
  BYO_CU(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bfs_small, kSmallBlock, 0));
  if (per_sm < 1) return set_error(ctx, BYO_EDEVICE, "bfs: persistent kernel cannot be resident");
  // a small grid: the frontiers are small, and barriers over fewer blocks are cheaper
  const unsigned grid = (unsigned)std::min<uint64_t>((uint64_t)per_sm * ctx->num_sms, ctx->num_sms * 2ull);
  void *args[] = {(void *)&a};
  BYO_CU(ctx, cudaLaunchCooperativeKernel((const void *)k_bfs_small, dim3(grid), dim3(kSmallBlock), args, 0,
                                          ctx->stream));
  ctx->launches++;
  BYO_CU(ctx, cudaMemcpyAsync(h, c, sizeof(SmallCtl), cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  if (h->bar.err) return set_error(ctx, BYO_ETIMEDOUT, "bfs: grid barrier timed out");
  const uint32_t R = h->rounds;
  const int fi = (int)h->final_idx;
  std::vector<unsigned long long> lg(2ull * R);
  if (R) {
    BYO_CU(ctx, cudaMemcpyAsync(lg.data(), logb, 16ull * R, cudaMemcpyDeviceToHost, ctx->stream));
    BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  }
  for (uint32_t r = 0; r < R; r++) {
    byo_round_log e{};
    e.round = st.round + r;
    e.mode = MODE_PUSH;
    e.frontier = lg[2 * r];
    e.frontier_deg = r == 0 ? cur->outdeg : lg[2 * (r - 1) + 1];
    e.unvisited = 0;
    ctx->rounds.push_back(e);
  }
  // the frontier the kernel ended with, in the engine's form
  Frontier *fin = fi == 0 ? cur : nxt;
  Frontier *other = fi == 0 ? nxt : cur;
  fin->size = h->cnt[fi];
  fin->outdeg = h->outdeg[fi];
  for (int q = 0; q < 8; q++) fin->hist[q] = h->hist[fi][q];
  fin->dense = false;
  fin->has_list = fin->has_bits = true;
  other->size = 0;
  other->has_list = true;
  other->has_bits = true;
  uint64_t reached = 0;
  for (uint32_t r = 0; r < R; r++) reached += r + 1 < R ? lg[2 * (r + 1)] : fin->size;
  st.reached += reached;
  st.round += R;
  cur = fin;
  nxt = other;
  if (d_st) {
    // the statistics the policy reads for the round after (a pageable source:
    // the copy has consumed it when the call returns)
    RoundStats rs{};
    rs.count = fin->size;
    rs.outdeg = fin->outdeg;
    for (int q = 0; q < 8; q++) rs.hist[q] = fin->hist[q];
    BYO_CU(ctx, cudaMemcpyAsync(d_st, &rs, sizeof(RoundStats), cudaMemcpyHostToDevice, ctx->stream));
  }
  *rounds_run = R;
  return check_launch(ctx, "bfs_small");
}

}  // namespace byo

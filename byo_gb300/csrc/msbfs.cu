// msbfs.cu -- 64-source BFS packed into bit lanes, run by one persistent
// cooperative kernel.
//
// Each vertex carries 64-bit masks: seen (sources that reached it), and the
// frontier masks of two consecutive rounds, F (read) and N (written).  BFS
// levels do not depend on the order in which a round's ORs happen, so every
// source's levels equal those of a single-source BFS (BFS.h:47-64) from it.
// The union frontier of all lanes chooses the direction of each round, as
// edgeMapData does for one source (edge_map_data.h:254-307):
//
//   push  every frontier vertex u ORs F[u] & ~seen[v] into an accumulator
//         X[v] of each neighbour; the first writer of X[v] appends v to a
//         touched list, and a second phase turns the touched vertices into
//         the next frontier and its list.  A frontier vertex takes a warp;
//         hubs (more than hub_deg slots) are cut into chunks of hub_deg
//         slots, a warp per chunk.
//   pull  every vertex that still misses some source ORs the F masks of its
//         neighbours, stopping once every missing bit is found.  Up to
//         heavy_deg slots a thread takes the vertex, up to hub_deg a warp;
//         above that its slots are cut into chunks, a warp each, whose ORs
//         meet in X[v] and are settled after a grid barrier.  A pull round
//         writes every N[v] and keeps only the frontier's size and slot sum,
//         reduced per block, so no single counter is contended.
//
// A push round needs the list of its input frontier: it has one when the
// previous round was a push, otherwise it first collects it from F.  It also
// needs N free of the entries of two rounds before, which it clears from that
// round's list, or wholesale when that round was a pull.  Levels are kept as
// bit planes: when round r reaches sources `got` at v, got is ORed into
// plane b of v for every bit b of r (16 planes, rounds below 2^16; later
// rounds write their levels straight to the output).  A last kernel turns
// each vertex's planes into its 64 levels and writes them source-major, a
// warp storing 32 consecutive words per source, with BYO_NONE for pairs never
// reached; the traversal itself makes no scattered output stores.  Rounds are
// separated by a grid
// barrier of the project's own whose wait is bounded in time: a barrier that
// does not complete sets an error flag and every block leaves.
#include <algorithm>
#include <vector>

#include "msbfs.cuh"

namespace byo {

__global__ void __launch_bounds__(kMsBlock, 5) k_ms_bfs(MsArgs a) { ms_bfs_body(a, &a.ctl->bar); }

__global__ void __launch_bounds__(256) k_ms_levels(const MsArgs a) {
  if (a.ctl->bar.err) return;
  ms_levels_body(a, blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, (uint64_t)gridDim.x * blockDim.x);
}

int ms_args_setup(byo_graph *g, uint32_t k, MsArgs *out) {
  const uint64_t n = g->n;
  const byo_tuning t = effective_tuning(g);
  MsArgs a = {};
  a.off = g->d_off;
  a.slots = g->d_slots;
  a.n = n;
  a.nslots = g->nslots;
  a.full = k == 64 ? ~0ull : ((1ull << k) - 1);
  a.k = k;
  a.max_rounds = 0xFFFFFFF0u;
  a.heavy_deg = t.ms_heavy_deg;
  a.hub_deg = t.ms_hub_deg;
  a.push_div = t.ms_push_div;
  // chunks of a set of distinct vertices above hub_deg: sum of ceil(d / hub_deg) <= 2 * slots / hub_deg
  const uint64_t nchunks = 2 * g->nslots / a.hub_deg + 64;
  a.ccap = nchunks;
  uint64_t *masks;
  BYO_TRY(ws(g, WS_LP, 4 * n + 4, &masks));  // seen | A | B | X
  a.seen = masks;
  a.A = masks + n;
  a.B = masks + 2 * n;
  a.X = masks + 3 * n;
  uint32_t *lists;
  BYO_TRY(ws(g, WS_FRONT_LIST_A, 3 * n + 4, &lists));
  for (int i = 0; i < 3; i++) a.L[i] = lists + i * n;
  uint32_t *th;
  BYO_TRY(ws(g, WS_FRONT_LIST_B, 2 * n + 4, &th));
  a.T = th;
  a.H = th + n;
  uint64_t *chunks;
  BYO_TRY(ws(g, WS_DEFER, 3 * nchunks, &chunks));
  a.C[0] = chunks;
  a.C[1] = chunks + nchunks;
  a.MC = chunks + 2 * nchunks;
  BYO_TRY(ws(g, WS_MS_LEVELS, (size_t)kLevelBits * n, &a.planes));
  *out = a;
  return BYO_OK;
}

int bfs_multi_run(byo_graph *g, const uint32_t *h_srcs, uint32_t k, uint32_t *d_levels, uint32_t *rounds) {
  byo_ctx *ctx = g->ctx;
  const uint64_t n = g->n;
  if (k == 0 || k > 64) return set_error(ctx, BYO_EINVAL, "bfs_multi: 1 <= k <= 64 sources");
  for (uint32_t s = 0; s < k; s++)
    if (h_srcs[s] >= n) return set_error(ctx, BYO_EINVAL, "bfs_multi: source >= n");
  if (n >= (1ull << 32) - 1) return set_error(ctx, BYO_EINVAL, "bfs_multi: n too large");
  MsArgs a = {};
  BYO_TRY(ms_args_setup(g, k, &a));
  uint32_t *misc;
  BYO_TRY(ws(g, WS_MISC, 64 + sizeof(MsCtl) / 4 + 8, &misc));  // sources, then the control block
  a.srcs = misc;
  a.ctl = (MsCtl *)(misc + 64);
  a.levels = d_levels;
  BYO_CU(ctx, cudaMemcpyAsync(misc, h_srcs, k * 4, cudaMemcpyHostToDevice, ctx->stream));
  BYO_CU(ctx, cudaMemsetAsync(a.ctl, 0, sizeof(MsCtl), ctx->stream));
  if (ctx->bar_limit_ms || ctx->bar_extra) {  // the barrier test hook
    const unsigned int hb[2] = {ctx->bar_limit_ms, ctx->bar_extra};
    BYO_CU(ctx, cudaMemcpyAsync(&a.ctl->bar.limit_ms, hb, sizeof(hb), cudaMemcpyHostToDevice, ctx->stream));
    BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));  // hb is on the stack
  }
  // co-resident grid for the cooperative launch
  int per_sm = 0;
  BYO_CU(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ms_bfs, kMsBlock, 0));
  if (per_sm < 1) return set_error(ctx, BYO_EDEVICE, "bfs_multi: kernel cannot be resident");
  const unsigned int grid = (unsigned int)std::max<uint64_t>(
      1, std::min<uint64_t>((uint64_t)per_sm * ctx->num_sms, (n + kMsBlock - 1) / kMsBlock));
  void *args[] = {(void *)&a};
  const bool timed = !ctx->ktag.empty() && ktimer_begin(ctx, "bfs_multi");
  BYO_CU(ctx, cudaLaunchCooperativeKernel((const void *)k_ms_bfs, dim3(grid), dim3(kMsBlock), args, 0, ctx->stream));
  launch(ctx, k_ms_levels, dim3(grid_for(ctx, n, 256)), dim3(256), 0, a);
  ctx->launches++;
  if (timed) ktimer_end(ctx);
  MsCtl *h = nullptr;
  BYO_TRY(pinned(ctx, sizeof(MsCtl), (void **)&h));
  BYO_CU(ctx, cudaMemcpyAsync(h, a.ctl, sizeof(MsCtl), cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  if (h->bar.err & 2u) return set_error(ctx, BYO_EDEVICE, "bfs_multi: hub chunk list overflow");
  if (h->bar.err) return set_error(ctx, BYO_ETIMEDOUT, "bfs_multi: grid barrier timed out");
  if (rounds) *rounds = h->rounds;
  ctx->rounds.clear();
  uint64_t prev = h->t0;
  for (uint32_t r = 0; r < h->rounds && r < (uint32_t)kMsLog; r++) {
    byo_round_log e = {};
    e.round = r + 1;
    e.mode = h->rlog[r][1] ? 0 : 1;
    e.frontier = h->rlog[r][2];
    e.frontier_deg = h->rlog[r][3];
    e.ms = (float)((double)(h->rlog[r][0] - prev) * 1e-6);
    prev = h->rlog[r][0];
    ctx->rounds.push_back(e);
  }
  return check_launch(ctx, "bfs_multi");
}

}  // namespace byo

// autotune.cu -- picks a graph's traversal launch shapes by timing them.
//
// The fields of byo_tuning are degree-bucket boundaries (where the work for
// one vertex moves from a thread to a lane group, a warp, chunks of warps or a
// CTA) and tile sizes.  None of them changes a result, so the tuner is free
// to try each: coordinate descent, one field at a time over a short candidate
// list with the other fields at their best so far, scoring a candidate by the
// summed device time of BFS runs from a fixed set of seeded sources.
#include <algorithm>
#include <vector>

#include "internal.h"

namespace byo {

namespace {

struct Timer {
  cudaEvent_t a = nullptr, b = nullptr;
  ~Timer() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};

// Sources with at least one neighbour, from a fixed counter-based sequence.
int pick_sources(byo_graph *g, uint32_t count, std::vector<uint32_t> &out) {
  std::vector<uint32_t> deg(g->n);
  BYO_CU(g->ctx, cudaMemcpyAsync(deg.data(), g->d_deg, g->n * 4, cudaMemcpyDeviceToHost, g->ctx->stream));
  BYO_CU(g->ctx, cudaStreamSynchronize(g->ctx->stream));
  uint64_t x = 0x243F6A8885A308D3ull;
  for (uint64_t tries = 0; out.size() < count && tries < 64ull * count + 1024; tries++) {
    x += 0x9E3779B97F4A7C15ull;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const uint32_t v = (uint32_t)(z % g->n);
    if (deg[v]) out.push_back(v);
  }
  if (out.empty()) out.push_back(0);
  return BYO_OK;
}

}  // namespace

int autotune(byo_graph *g, uint32_t what, uint32_t trials) {
  byo_ctx *ctx = g->ctx;
  if (!g->n) return BYO_OK;
  if (trials == 0) trials = 3;
  if (trials > 64) trials = 64;
  std::vector<uint32_t> srcs;
  BYO_TRY(pick_sources(g, (what & BYO_TUNE_MULTI) ? std::max<uint32_t>(trials, 64) : trials, srcs));
  Timer t;
  BYO_CU(ctx, cudaEventCreate(&t.a));
  BYO_CU(ctx, cudaEventCreate(&t.b));
  uint32_t *d_parent = nullptr, *d_levels = nullptr;
  BYO_TRY(ws(g, WS_LABEL, 2 * g->n + 2, &d_parent));
  const uint32_t kq = (uint32_t)std::min<size_t>(64, srcs.size());
  if (what & BYO_TUNE_MULTI) BYO_TRY(ws(g, WS_TC_NBR, (uint64_t)kq * g->n + 1, &d_levels));

  // score of the current g->tune for one kernel family, in ms
  auto score = [&](bool multi, int policy, float *ms) -> int {
    byo_graph *tg = nullptr;
    BYO_TRY(traversal_view(g, &tg));  // carries g->tune
    float total = 0;
    const uint32_t runs = multi ? std::max<uint32_t>(1, trials / 2) : trials;
    for (uint32_t i = 0; i < runs; i++) {
      BYO_CU(ctx, cudaEventRecord(t.a, ctx->stream));
      if (multi) {
        // rotate the 64-source set so each run starts from different sources
        std::vector<uint32_t> q(kq);
        for (uint32_t s = 0; s < kq; s++) q[s] = srcs[(s + i * 7) % srcs.size()];
        BYO_TRY(bfs_multi_run(tg, q.data(), kq, d_levels, nullptr));
      } else {
        BYO_TRY(bfs_run(tg, srcs[i % srcs.size()], d_parent, nullptr, policy, nullptr));
      }
      BYO_CU(ctx, cudaEventRecord(t.b, ctx->stream));
      BYO_CU(ctx, cudaEventSynchronize(t.b));
      float x = 0;
      BYO_CU(ctx, cudaEventElapsedTime(&x, t.a, t.b));
      total += x;
    }
    *ms = total;
    return BYO_OK;
  };

  struct Field {
    uint32_t byo_tuning::*f;
    std::vector<uint32_t> cand;
    bool multi;
    int policy;
  };
  std::vector<Field> fields;
  if (what & BYO_TUNE_BFS) {
    fields.push_back({&byo_tuning::push_group, {4, 8, 16, 32}, false, BYO_POLICY_M20});
    fields.push_back({&byo_tuning::hub_min, {1024, 4096, 16384}, false, BYO_POLICY_M20});
    fields.push_back({&byo_tuning::pull_cap, {8, 16, 32, 64, 128}, false, BYO_POLICY_M20});
    fields.push_back({&byo_tuning::blocked_tile, {512, 2048, 8192}, false, BYO_POLICY_M20_BLOCKED});
    fields.push_back({&byo_tuning::pull_stage_words, {8192, 16384, 32768}, false, BYO_POLICY_M20});
  }
  if (what & BYO_TUNE_MULTI) {
    fields.push_back({&byo_tuning::ms_heavy_deg, {8, 16, 32, 64, 128, 256}, true, 0});
    fields.push_back({&byo_tuning::ms_hub_deg, {512, 2048, 8192}, true, 0});
    fields.push_back({&byo_tuning::ms_push_div, {5, 10, 20, 40, 80}, true, 0});
  }
  // start from what is in effect; warm the workspaces once per family
  g->tune = effective_tuning(g);
  float warm = 0;
  if (what & BYO_TUNE_BFS) BYO_TRY(score(false, BYO_POLICY_M20, &warm));
  if (what & BYO_TUNE_MULTI) BYO_TRY(score(true, 0, &warm));
  for (const Field &fd : fields) {
    uint32_t best = g->tune.*(fd.f);
    float best_ms = 0;
    BYO_TRY(score(fd.multi, fd.policy, &best_ms));
    for (uint32_t c : fd.cand) {
      if (c == best) continue;
      const uint32_t keep = g->tune.*(fd.f);
      g->tune.*(fd.f) = c;
      float ms = 0;
      BYO_TRY(score(fd.multi, fd.policy, &ms));
      if (ms < best_ms) {
        best_ms = ms;
        best = c;
      } else {
        g->tune.*(fd.f) = keep;
      }
    }
    g->tune.*(fd.f) = best;
  }
  return BYO_OK;
}

}  // namespace byo

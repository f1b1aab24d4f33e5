// engine.cu -- edgeMap rounds (push / blocked / pull) and the BFS driver.
// See engine.h for the design.  Algorithmic bytes of one BFS traversal:
// 4 B per adjacency entry of every reached vertex + 8 B offsets per vertex
// + 8 B lp written per reached vertex (parent/level split is 8 B more).
#include <algorithm>
#include <cstring>

#include "device.cuh"
#include "engine.h"
#include "policy.cuh"
#include "internal.h"
#include "scan.cuh"

namespace byo {

__host__ __device__ __forceinline__ int log4_bin(uint32_t d) {
#ifdef __CUDA_ARCH__
  int b = d ? (31 - __clz(d)) / 2 : 0;  // 0:[0,4) 1:[4,16) ...
#else
  int b = d ? (31 - __builtin_clz(d)) / 2 : 0;
#endif
  return b > 7 ? 7 : b;
}

// The degree sketch of the next frontier is counted per block in shared
// memory (a warp adds one count per bin it holds) and added to the round's
// statistics once per block, so no global counter sees one atomic per vertex.
__device__ __forceinline__ void hist_init(unsigned long long *sh) {
  if (threadIdx.x < 8) sh[threadIdx.x] = 0;
  __syncthreads();
}
__device__ __forceinline__ void hist_warp_add(unsigned long long *sh, bool has, uint32_t d) {
  if (!__ballot_sync(kFull, has)) return;
  const int bin = log4_bin(d);
#pragma unroll
  for (int b = 0; b < 8; b++) {
    const unsigned m = __ballot_sync(kFull, has && bin == b);
    if (m && lane_id() == 0) atomicAdd(sh + b, (unsigned long long)__popc(m));
  }
}
__device__ __forceinline__ void hist_flush(unsigned long long *sh, RoundStats *st) {
  __syncthreads();
  if (threadIdx.x < 8 && sh[threadIdx.x]) atomicAdd(&st->hist[threadIdx.x], sh[threadIdx.x]);
}

// Emits v (if `emit`) to the next frontier list and bitmap; accumulates its
// degree for the round statistics.  Warp-collective.
__device__ __forceinline__ void emit_next(bool emit, uint32_t v, uint32_t *out_list,
                                          uint32_t *out_bits, RoundStats *st,
                                          const uint32_t *__restrict__ deg, uint64_t &dsum,
                                          bool set_bits, unsigned long long *sh) {
  uint64_t slot = warp_append(emit, &st->count);
  uint32_t d = 0;
  if (emit) {
    out_list[slot] = v;
    if (set_bits) atomicOr(out_bits + (v >> 5), 1u << (v & 31));
    d = deg[v];
    dsum += d;
  }
  hist_warp_add(sh, emit, d);
}

__device__ __forceinline__ void flush_dsum(uint64_t dsum, RoundStats *st) {
  dsum = warp_sum(dsum);
  if (lane_id() == 0 && dsum) atomicAdd(&st->outdeg, (unsigned long long)dsum);
}

// Visits edge u->v for BFS_F: cond(v) = not visited before this round;
// updateAtomic keeps the smallest (level, parent); the first writer emits.
__device__ __forceinline__ bool visit(uint32_t u, uint32_t v, uint64_t lvl, uint64_t *lp,
                                      const uint32_t *__restrict__ visited) {
  if (v == kSentinel) return false;
  if (test_bit_cg(visited, v)) return false;
  unsigned long long old = atomicMin((unsigned long long *)(lp + v), (unsigned long long)(lvl | u));
  return old == kNone64;
}

// ---------------------------------------------------------------- push
template <int GS>
__global__ void __launch_bounds__(256) k_push(const uint64_t *__restrict__ off,
                                              const uint32_t *__restrict__ slots,
                                              const uint32_t *__restrict__ deg,
                                              const uint32_t *__restrict__ F, uint64_t fsize,
                                              uint64_t *lp, const uint32_t *__restrict__ visited,
                                              uint32_t *out_list, uint32_t *out_bits,
                                              RoundStats *st, uint64_t lvl, uint32_t *hubs,
                                              uint32_t hub_min) {
  __shared__ unsigned long long s_hist[8];
  hist_init(s_hist);
  constexpr int PER_WARP = 32 / GS;
  const unsigned lane = lane_id(), g = lane / GS, gl = lane % GS;
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  uint64_t dsum = 0;
  for (uint64_t i0 = gw * PER_WARP; i0 < fsize; i0 += nw * PER_WARP) {
    uint64_t i = i0 + g;
    uint32_t u = 0;
    uint64_t b = 0, e = 0;
    if (i < fsize) {
      u = F[i];
      b = off[u];
      e = off[u + 1];
      if (e - b >= hub_min) {
        if (gl == 0) hubs[atomicAdd(&st->ndefer, 1ull)] = u;
        e = b;
      }
    }
    uint64_t chunks = (e - b + GS - 1) / GS;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      uint64_t t = __shfl_xor_sync(kFull, chunks, o);
      chunks = t > chunks ? t : chunks;
    }
    for (uint64_t c = 0; c < chunks; c++) {
      uint64_t j = b + c * GS + gl;
      bool em = false;
      uint32_t v = kSentinel;
      if (j < e) {
        v = slots[j];
        em = visit(u, v, lvl, lp, visited);
      }
      emit_next(em, v, out_list, out_bits, st, deg, dsum, true, s_hist);
    }
  }
  hist_flush(s_hist, st);
  flush_dsum(dsum, st);
}

// edgeMapDenseForward (edge_map_data.h:180-247): every vertex of a dense
// frontier pushes to its neighbours; a warp takes a 32-vertex bitmap word and
// walks the adjacency of each of its set bits with all lanes.
__global__ void __launch_bounds__(256) k_push_dense_fwd(const uint64_t *__restrict__ off,
                                                        const uint32_t *__restrict__ slots,
                                                        const uint32_t *__restrict__ deg,
                                                        const uint32_t *__restrict__ Fbits, uint64_t n,
                                                        uint64_t *lp, const uint32_t *__restrict__ visited,
                                                        uint32_t *out_list, uint32_t *out_bits, RoundStats *st,
                                                        uint64_t lvl) {
  __shared__ unsigned long long s_hist[8];
  hist_init(s_hist);
  const unsigned lane = lane_id();
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t W = (n + 31) / 32;
  uint64_t dsum = 0;
  for (uint64_t w = gw; w < W; w += nw) {
    unsigned word = Fbits[w];
    while (word) {
      const uint32_t u = (uint32_t)(w * 32 + __ffs(word) - 1);
      word &= word - 1;
      const uint64_t b = off[u], e = off[u + 1];
      for (uint64_t base = b; base < e; base += 32) {
        const uint64_t j = base + lane;
        bool em = false;
        uint32_t v = kSentinel;
        if (j < e) {
          v = slots[j];
          em = visit(u, v, lvl, lp, visited);
        }
        emit_next(em, v, out_list, out_bits, st, deg, dsum, true, s_hist);
      }
    }
  }
  hist_flush(s_hist, st);
  flush_dsum(dsum, st);
}

// One CTA per hub vertex (degree >= hub_min).
__global__ void __launch_bounds__(256) k_push_hubs(const uint64_t *__restrict__ off,
                                                   const uint32_t *__restrict__ slots,
                                                   const uint32_t *__restrict__ deg,
                                                   const uint32_t *__restrict__ hubs,
                                                   uint64_t *lp, const uint32_t *__restrict__ visited,
                                                   uint32_t *out_list, uint32_t *out_bits,
                                                   RoundStats *st, uint64_t lvl) {
  __shared__ unsigned long long s_hist[8];
  hist_init(s_hist);
  const uint64_t nh = *(volatile unsigned long long *)&st->ndefer;
  uint64_t dsum = 0;
  for (uint64_t h = blockIdx.x; h < nh; h += gridDim.x) {
    const uint32_t u = hubs[h];
    const uint64_t b = off[u], e = off[u + 1];
    for (uint64_t base = b; base < e; base += blockDim.x) {
      uint64_t j = base + threadIdx.x;
      bool em = false;
      uint32_t v = kSentinel;
      if (j < e) {
        v = slots[j];
        em = visit(u, v, lvl, lp, visited);
      }
      emit_next(em, v, out_list, out_bits, st, deg, dsum, true, s_hist);
    }
  }
  hist_flush(s_hist, st);
  flush_dsum(dsum, st);
}

// ---------------------------------------------------------------- blocked
// Edge-balanced: tile t covers frontier-edge ranks [t*TILE, (t+1)*TILE) of
// the exclusive degree prefix `pre`; each rank is mapped to its frontier
// vertex by binary search (the merge-path split of rank space).
__global__ void __launch_bounds__(256) k_push_blocked(const uint64_t *__restrict__ off,
                                                      const uint32_t *__restrict__ slots,
                                                      const uint32_t *__restrict__ deg,
                                                      const uint32_t *__restrict__ F, uint64_t fsize,
                                                      const uint64_t *__restrict__ pre,
                                                      uint64_t *lp,
                                                      const uint32_t *__restrict__ visited,
                                                      uint32_t *out_list, uint32_t *out_bits,
                                                      RoundStats *st, uint64_t lvl, int tile) {
  __shared__ unsigned long long s_hist[8];
  hist_init(s_hist);
  const uint64_t total = pre[fsize];
  const uint64_t ntiles = (total + tile - 1) / tile;
  __shared__ uint64_t s_lo, s_hi;
  uint64_t dsum = 0;
  for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const uint64_t e0 = t * tile;
    const uint64_t e1 = e0 + tile < total ? e0 + tile : total;
    if (threadIdx.x == 0) {
      // last index with pre[i] <= e0, and with pre[i] <= e1-1
      uint64_t lo = 0, hi = fsize;  // search in [0, fsize)
      while (hi - lo > 1) {
        uint64_t mid = (lo + hi) >> 1;
        if (pre[mid] <= e0) lo = mid; else hi = mid;
      }
      s_lo = lo;
      uint64_t lo2 = lo, hi2 = fsize;
      while (hi2 - lo2 > 1) {
        uint64_t mid = (lo2 + hi2) >> 1;
        if (pre[mid] <= e1 - 1) lo2 = mid; else hi2 = mid;
      }
      s_hi = lo2;
    }
    __syncthreads();
    const uint64_t vlo = s_lo, vhi = s_hi;
    for (uint64_t base = e0; base < e1; base += blockDim.x) {
      const uint64_t e = base + threadIdx.x;
      bool em = false;
      uint32_t v = kSentinel;
      if (e < e1) {
        uint64_t lo = vlo, hi = vhi + 1;
        while (hi - lo > 1) {
          uint64_t mid = (lo + hi) >> 1;
          if (pre[mid] <= e) lo = mid; else hi = mid;
        }
        const uint32_t u = F[lo];
        v = slots[off[u] + (e - pre[lo])];
        em = visit(u, v, lvl, lp, visited);
      }
      emit_next(em, v, out_list, out_bits, st, deg, dsum, true, s_hist);
    }
    __syncthreads();
  }
  hist_flush(s_hist, st);
  flush_dsum(dsum, st);
}

// ---------------------------------------------------------------- pull
__device__ __forceinline__ bool in_frontier(const uint32_t *s_bits, int stage_words,
                                            const uint32_t *__restrict__ Fbits, uint32_t u) {
  uint32_t w = u >> 5;
  uint32_t word = (w < (uint32_t)stage_words) ? s_bits[w] : __ldg(Fbits + w);
  return (word >> (u & 31)) & 1u;
}

__global__ void __launch_bounds__(1024, 2) k_pull(const uint64_t *__restrict__ off,
                                               const uint32_t *__restrict__ slots,
                                               const uint32_t *__restrict__ deg,
                                               const uint32_t *__restrict__ Fbits, uint64_t n,
                                               uint64_t *__restrict__ lp, uint32_t *visited,
                                               uint32_t *out_list, uint32_t *out_bits,
                                               RoundStats *st, uint64_t lvl, uint32_t *defer,
                                               int cap, int stage_words) {
  extern __shared__ uint32_t s_bits[];
  __shared__ unsigned long long s_hist[8];
  for (int i = threadIdx.x; i < stage_words; i += blockDim.x) s_bits[i] = Fbits[i];
  if (threadIdx.x < 8) s_hist[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t W = (n + 31) >> 5;
  const unsigned lane = lane_id();
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  uint64_t dsum = 0;
  for (uint64_t w = gw; w < W; w += nw) {
    const uint32_t vword = visited[w];
    if (vword == kFull) continue;
    const uint64_t v = w * 32 + lane;
    bool active = v < n && !((vword >> lane) & 1u);
    bool found = false, deferred = false;
    uint32_t parent = 0;
    if (active) {
      const uint64_t b = off[v], e = off[v + 1];
      const uint64_t lim = (e - b > (uint64_t)cap) ? b + cap : e;
      // eight neighbours at a time: their ids, then their frontier bits, are
      // loaded together; the first hit in slot order is the parent
      for (uint64_t j0 = b; j0 < lim && !found; j0 += 8) {
        uint32_t u[8];
#pragma unroll
        for (int q = 0; q < 8; q++) u[q] = j0 + q < lim ? slots[j0 + q] : kSentinel;
        bool h[8];
#pragma unroll
        for (int q = 0; q < 8; q++) h[q] = u[q] != kSentinel && in_frontier(s_bits, stage_words, Fbits, u[q]);
#pragma unroll
        for (int q = 7; q >= 0; q--)
          if (h[q]) {
            found = true;
            parent = u[q];
          }
      }
      deferred = !found && lim < e;
    }
    if (found) lp[v] = lvl | parent;
    const unsigned fb = __ballot_sync(kFull, found);
    if (lane == 0 && fb) {
      out_bits[w] = fb;
      visited[w] = vword | fb;
    }
    uint64_t slot = warp_append(found, &st->count);
    uint32_t d = 0;
    if (found) {
      out_list[slot] = (uint32_t)v;
      d = deg[v];
      dsum += d;
    }
    hist_warp_add(s_hist, found, d);
    uint64_t ds = warp_append(deferred, &st->ndefer);
    if (deferred) defer[ds] = (uint32_t)v;
  }
  hist_flush(s_hist, st);
  flush_dsum(dsum, st);
}

// Warp per deferred vertex: 32 neighbours per step, ballot, lowest lane wins.
__global__ void __launch_bounds__(256) k_pull_long(const uint64_t *__restrict__ off,
                                                   const uint32_t *__restrict__ slots,
                                                   const uint32_t *__restrict__ deg,
                                                   const uint32_t *__restrict__ Fbits,
                                                   uint64_t *__restrict__ lp, uint32_t *visited,
                                                   uint32_t *out_list, uint32_t *out_bits,
                                                   RoundStats *st, uint64_t lvl,
                                                   const uint32_t *__restrict__ defer, int cap, PolicyTail pt) {
  __shared__ float4 sP[kParamChunks];
  __shared__ unsigned long long s_hist[8];
  policy_prefetch(pt, sP);
  hist_init(s_hist);
  const uint64_t nd = *(volatile unsigned long long *)&st->ndefer;
  const unsigned lane = lane_id();
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t i = gw; i < nd; i += nw) {
    const uint32_t v = defer[i];
    const uint64_t b = off[v] + cap, e = off[v + 1];
    bool found = false;
    uint32_t parent = 0;
    for (uint64_t base = b; base < e && !found; base += 32) {
      uint64_t j = base + lane;
      uint32_t u = j < e ? slots[j] : kSentinel;
      bool hit = u != kSentinel && ((__ldg(Fbits + (u >> 5)) >> (u & 31)) & 1u);
      unsigned m = __ballot_sync(kFull, hit);
      if (m) {
        found = true;
        parent = __shfl_sync(kFull, u, __ffs(m) - 1);
      }
    }
    uint32_t d = 0;
    if (found && lane == 0) {
      lp[v] = lvl | parent;
      atomicOr(out_bits + (v >> 5), 1u << (v & 31));
      atomicOr(visited + (v >> 5), 1u << (v & 31));
      unsigned long long slot = atomicAdd(&st->count, 1ull);
      out_list[slot] = v;
      d = deg[v];
      atomicAdd(&st->outdeg, (unsigned long long)d);
    }
    hist_warp_add(s_hist, found && lane == 0, d);
  }
  hist_flush(s_hist, st);
  policy_tail(pt, st, sP);
}

// ---------------------------------------------------------------- bookkeeping
__global__ void k_mark_visited(const uint32_t *__restrict__ list, RoundStats *st, uint32_t *visited,
                               PolicyTail pt) {
  __shared__ float4 sP[kParamChunks];
  policy_prefetch(pt, sP);
  const uint64_t cnt = st->count;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t v = list[i];
    atomicOr(visited + (v >> 5), 1u << (v & 31));
  }
  policy_tail(pt, st, sP);
}

__global__ void k_clear_words_from_list(const uint32_t *__restrict__ list, uint64_t cnt,
                                        uint32_t *bits) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt;
       i += (uint64_t)gridDim.x * blockDim.x)
    bits[list[i] >> 5] = 0;  // every set bit of `bits` belongs to some list entry
}

__global__ void k_set_bits_from_list(const uint32_t *__restrict__ list, uint64_t cnt, uint32_t *bits) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t v = list[i];
    atomicOr(bits + (v >> 5), 1u << (v & 31));
  }
}

__global__ void k_trav_init(uint64_t *lp, uint32_t *visited, uint64_t n, uint32_t src) {
  const uint64_t W = (n + 31) >> 5;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    lp[i] = (i == src) ? (uint64_t)src : kNone64;
    if (i < W) visited[i] = (i == (src >> 5)) ? (1u << (src & 31)) : 0u;
  }
}

__global__ void k_trav_extract(const uint64_t *__restrict__ lp, uint64_t n, uint32_t *parent,
                               uint32_t *level) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t x = lp[i];
    if (parent) parent[i] = x == kNone64 ? kSentinel : (uint32_t)x;
    if (level) level[i] = x == kNone64 ? kSentinel : (uint32_t)(x >> 32);
  }
}

// ---------------------------------------------------------------- host side

byo_tuning effective_tuning(const byo_graph *g) {
  byo_tuning t = g->tune;
  const double avg = g->n ? (double)g->m / (double)g->n : 0.0;
  if (!t.push_group) t.push_group = avg >= 24 ? 32 : avg >= 12 ? 16 : avg >= 6 ? 8 : 4;
  if (!t.hub_min) t.hub_min = 4096;
  if (!t.pull_cap) t.pull_cap = 32;
  if (!t.blocked_tile) t.blocked_tile = 2048;
  if (!t.ms_heavy_deg) t.ms_heavy_deg = 32;
  if (!t.ms_hub_deg) t.ms_hub_deg = 2048;
  if (!t.ms_push_div) t.ms_push_div = 20;
  if (!t.tc_stage) t.tc_stage = 40960;
  t.reserved = 0;
  if (!t.pull_stage_words) {
    const uint64_t W = (g->n + 31) / 32;
    t.pull_stage_words = (uint32_t)(W < 16384 ? (W < 256 ? 256 : W) : 16384);
  }
  return t;
}

int check_tuning(byo_ctx *ctx, const byo_tuning *t) {
  const char *bad = nullptr;
  if (t->push_group && t->push_group != 4 && t->push_group != 8 && t->push_group != 16 && t->push_group != 32)
    bad = "push_group must be 4, 8, 16 or 32";
  else if (t->hub_min && t->hub_min < 32)
    bad = "hub_min must be >= 32";
  else if (t->pull_cap > 4096)
    bad = "pull_cap must be <= 4096";
  else if (t->blocked_tile && (t->blocked_tile < 64 || t->blocked_tile > 65536))
    bad = "blocked_tile must be in [64, 65536]";
  else if (t->ms_heavy_deg > 65536)
    bad = "ms_heavy_deg must be <= 65536";
  else if (t->ms_hub_deg && (t->ms_hub_deg < 32 || t->ms_hub_deg > (1u << 20)))
    bad = "ms_hub_deg must be in [32, 2^20]";
  else if (t->pull_stage_words && (t->pull_stage_words < 256 || t->pull_stage_words > 49152))
    bad = "pull_stage_words must be in [256, 49152]";
  else if (t->tc_stage && (t->tc_stage < 512 || t->tc_stage > 49152))
    bad = "tc_stage must be in [512, 49152]";
  else if (t->reserved)
    bad = "reserved field must be zero";
  return bad ? set_error(ctx, BYO_EINVAL, bad) : BYO_OK;
}

EngineTuning default_tuning(const byo_graph *g) {
  EngineTuning t;
  const uint64_t W = (g->n + 31) / 32;
  const byo_tuning e = effective_tuning(g);
  t.pull_stage_words = (int)(W < e.pull_stage_words ? W : e.pull_stage_words);
  t.push_group = (int)e.push_group;
  t.hub_min = e.hub_min;
  t.pull_cap = (int)e.pull_cap;
  t.blocked_tile = (int)e.blocked_tile;
  return t;
}

int m20_mode(const byo_graph *g, const Frontier &f, int64_t threshold, int sparse_mode) {
  const uint64_t n = g->n, M = g->m;
  const uint64_t dense_threshold = threshold < 0 ? M / 20 : (uint64_t)threshold;
  if (f.dense && f.size > n / 10) return MODE_PULL;
  if (f.size + f.outdeg > dense_threshold) return MODE_PULL;
  return sparse_mode;
}

int trav_init(byo_graph *g, TravState &st, uint32_t src) {
  byo_ctx *ctx = g->ctx;
  launch(ctx, k_trav_init, dim3(grid_for(ctx, g->n, 256)), dim3(256), 0, st.lp, st.visited, g->n, src);
  st.round = 1;
  st.reached = 1;
  return check_launch(ctx, "trav_init");
}

int trav_extract(byo_graph *g, const TravState &st, uint32_t *d_parent, uint32_t *d_level) {
  byo_ctx *ctx = g->ctx;
  launch(ctx, k_trav_extract, dim3(grid_for(ctx, g->n, 256)), dim3(256), 0, (const uint64_t *)st.lp,
         g->n, d_parent, d_level);
  return check_launch(ctx, "trav_extract");
}

int clear_frontier_bits(byo_graph *g, Frontier &f) {
  byo_ctx *ctx = g->ctx;
  const uint64_t W = (g->n + 31) / 32;
  if (f.has_list && f.size < W / 8) {
    if (f.size)
      launch(ctx, k_clear_words_from_list, dim3(grid_for(ctx, f.size, 256)), dim3(256), 0,
             (const uint32_t *)f.list, f.size, f.bits);
  } else {
    BYO_TRY(memset_async(ctx, f.bits, 0, W * sizeof(uint32_t)));
  }
  return check_launch(ctx, "clear_frontier_bits");
}

int ensure_bits(byo_graph *g, Frontier &f) {
  if (f.has_bits) return BYO_OK;
  byo_ctx *ctx = g->ctx;
  const uint64_t W = (g->n + 31) / 32;
  BYO_TRY(memset_async(ctx, f.bits, 0, W * sizeof(uint32_t)));
  if (f.size)
    launch(ctx, k_set_bits_from_list, dim3(grid_for(ctx, f.size, 256)), dim3(256), 0,
           (const uint32_t *)f.list, f.size, f.bits);
  f.has_bits = true;
  return check_launch(ctx, "ensure_bits");
}

static int pull_smem_ok(int bytes) {
  static int configured = 0;
  if (bytes > 48 * 1024 && configured < bytes) {
    if (cudaFuncSetAttribute(k_pull, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess)
      return 0;
    configured = bytes;
  }
  return 1;
}

int edge_map_round(byo_graph *g, TravState &st, Frontier &in, Frontier &out, int mode,
                   const EngineTuning &tune, bool run_policy) {
  byo_ctx *ctx = g->ctx;
  RoundStats *d_st = nullptr;
  BYO_TRY(ws(g, WS_STATS, sizeof(RoundStats) / sizeof(uint64_t) + 2, (uint64_t **)&d_st));
  BYO_CU(ctx, cudaMemsetAsync(d_st, 0, sizeof(RoundStats) + 8, ctx->stream));
  // the policy for the next round runs as the epilogue of this round's last kernel
  PolicyTail pt;
  if (run_policy) BYO_TRY(policy_tail_args(g, (unsigned int *)(d_st + 1), st.reached, mode == MODE_PULL, &pt));
  uint32_t *defer = nullptr;
  BYO_TRY(ws(g, WS_DEFER, g->n + 1, &defer));
  const uint64_t lvl = (uint64_t)st.round << 32;
  if (mode == MODE_PULL) {
    BYO_TRY(ensure_bits(g, in));
    int stage = tune.pull_stage_words;
    int smem = stage * 4;
    if (!pull_smem_ok(smem)) {
      if (stage > 12 * 1024) stage = 12 * 1024;
      smem = stage * 4;
    }
    const uint64_t W = (g->n + 31) / 32;
    int block = 1024;
    int grid = (int)((W + 31) / 32);
    int maxg = ctx->num_sms * (smem > 100 * 1024 ? 1 : 2);
    if (grid > maxg) grid = maxg;
    if (grid < 1) grid = 1;
    launch_t(ctx, "bfs_pull", k_pull, dim3(grid), dim3(block), (size_t)smem, (const uint64_t *)g->d_off,
           (const uint32_t *)g->d_slots, (const uint32_t *)g->d_deg, (const uint32_t *)in.bits, g->n,
           st.lp, st.visited, out.list, out.bits, d_st, lvl, defer, tune.pull_cap, stage);
    pt.prefetch = 1;
    launch(ctx, k_pull_long, dim3(ctx->num_sms * 4), dim3(256), 0, (const uint64_t *)g->d_off,
           (const uint32_t *)g->d_slots, (const uint32_t *)g->d_deg, (const uint32_t *)in.bits, st.lp,
           st.visited, out.list, out.bits, d_st, lvl, (const uint32_t *)defer, tune.pull_cap, pt);
  } else {
    if (mode == MODE_DENSE_FWD) {
      BYO_TRY(ensure_bits(g, in));
      const uint64_t W = (g->n + 31) / 32;
      launch_t(ctx, "bfs_push", k_push_dense_fwd, dim3(grid_for(ctx, W * 32, 256, 16)), dim3(256), 0,
               (const uint64_t *)g->d_off, (const uint32_t *)g->d_slots, (const uint32_t *)g->d_deg,
               (const uint32_t *)in.bits, g->n, st.lp, (const uint32_t *)st.visited, out.list, out.bits, d_st, lvl);
    } else if (!in.has_list) {
      return set_error(ctx, BYO_EINVAL, "sparse round needs a frontier list");
    } else if (mode == MODE_PUSH) {
      const int grid = grid_for(ctx, (in.size * (uint64_t)tune.push_group + 255) / 256 * 256, 256, 16);
      switch (tune.push_group) {
#define PUSH_CASE(GS)                                                                            \
  case GS:                                                                                       \
    launch_t(ctx, "bfs_push", k_push<GS>, dim3(grid), dim3(256), 0, (const uint64_t *)g->d_off,                \
           (const uint32_t *)g->d_slots, (const uint32_t *)g->d_deg, (const uint32_t *)in.list,  \
           in.size, st.lp, (const uint32_t *)st.visited, out.list, out.bits, d_st, lvl, defer,   \
           tune.hub_min);                                                                        \
    break;
        PUSH_CASE(4)
        PUSH_CASE(8)
        PUSH_CASE(16)
        PUSH_CASE(32)
#undef PUSH_CASE
        default:
          return set_error(ctx, BYO_EINVAL, "push group must be 4, 8, 16 or 32");
      }
      launch(ctx, k_push_hubs, dim3(ctx->num_sms * 2), dim3(256), 0, (const uint64_t *)g->d_off,
             (const uint32_t *)g->d_slots, (const uint32_t *)g->d_deg, (const uint32_t *)defer, st.lp,
             (const uint32_t *)st.visited, out.list, out.bits, d_st, lvl);
    } else {
      uint64_t *pre = nullptr;
      BYO_TRY(ws(g, WS_SCAN, in.size + 1, &pre));
      // prefix over slot-range lengths (= degrees for a CSR; gaps included
      // for the PMA so ranks map to slots)
      BYO_TRY(scan_gather_range(ctx, g->d_off, in.list, in.size, pre));
      const uint64_t est_tiles = (in.outdeg + tune.blocked_tile - 1) / tune.blocked_tile;
      const int grid = grid_for(ctx, est_tiles ? est_tiles : 1, 1, 16);
      launch_t(ctx, "bfs_blocked", k_push_blocked, dim3(grid), dim3(256), 0, (const uint64_t *)g->d_off,
             (const uint32_t *)g->d_slots, (const uint32_t *)g->d_deg, (const uint32_t *)in.list,
             in.size, (const uint64_t *)pre, st.lp, (const uint32_t *)st.visited, out.list, out.bits,
             d_st, lvl, tune.blocked_tile);
    }
    const int mgrid = grid_for(ctx, in.outdeg + 1, 256);
    pt.prefetch = mgrid >= ctx->num_sms;
    launch(ctx, k_mark_visited, dim3(mgrid), dim3(256), 0, (const uint32_t *)out.list, d_st, st.visited, pt);
  }
  BYO_TRY(check_launch(ctx, "edge_map_round"));
  RoundStats *h = nullptr;
  BYO_TRY(pinned(ctx, 4096, (void **)&h));
  BYO_CU(ctx, cudaMemcpyAsync(h, d_st, sizeof(RoundStats), cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  out.size = h->count;
  out.outdeg = h->outdeg;
  for (int i = 0; i < 8; i++) out.hist[i] = h->hist[i];
  if (run_policy) {
    out.next_mode = (int)h->mode;
    for (int i = 0; i < 16; i++) out.feat[i] = h->feat[i];
  }
  out.dense = (mode == MODE_PULL || mode == MODE_DENSE_FWD);
  out.has_list = true;
  out.has_bits = true;
  st.round++;
  st.reached += out.size;
  return BYO_OK;
}

// ---------------------------------------------------------------- BFS driver

int bfs_run(byo_graph *g, uint32_t src, uint32_t *d_parent, uint32_t *d_level, int policy,
            uint32_t *rounds) {
  byo_ctx *ctx = g->ctx;
  if (src >= g->n) return set_error(ctx, BYO_EINVAL, "bfs: src >= n");
  const uint64_t n = g->n, W = (n + 31) / 32;
  TravState st;
  Frontier fa, fb;
  BYO_TRY(ws(g, WS_LP, n, &st.lp));
  BYO_TRY(ws(g, WS_VISITED, W, &st.visited));
  BYO_TRY(ws(g, WS_FRONT_LIST_A, n, &fa.list));
  BYO_TRY(ws(g, WS_FRONT_LIST_B, n, &fb.list));
  BYO_TRY(ws(g, WS_FRONT_BITS_A, W, &fa.bits));
  BYO_TRY(ws(g, WS_FRONT_BITS_B, W, &fb.bits));
  BYO_TRY(trav_init(g, st, src));
  BYO_CU(ctx, cudaMemcpyAsync(fa.list, &src, sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream));
  BYO_TRY(memset_async(ctx, fa.bits, 0, W * 4));
  BYO_TRY(memset_async(ctx, fb.bits, 0, W * 4));
  uint32_t word = 1u << (src & 31);
  BYO_CU(ctx, cudaMemcpyAsync(fa.bits + (src >> 5), &word, 4, cudaMemcpyHostToDevice, ctx->stream));
  uint32_t dsrc = 0;
  BYO_CU(ctx, cudaMemcpyAsync(&dsrc, g->d_deg + src, 4, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  fa.size = 1;
  fa.outdeg = dsrc;
  fa.hist[log4_bin(dsrc)] = 1;
  fa.has_list = fa.has_bits = true;
  fb.size = 0;
  fb.has_list = true;  // empty list: its bitmap is all zero
  const EngineTuning tune = default_tuning(g);
  ctx->rounds.clear();
  // features (and the learned choice) are computed on the device after every
  // round when the learned policy runs or rounds are being logged
  const bool run_policy = policy == BYO_POLICY_LEARNED || ctx->time_rounds;
  if (run_policy) {
    RoundStats *d_st = nullptr, *h = nullptr;
    BYO_TRY(ws(g, WS_STATS, sizeof(RoundStats) / sizeof(uint64_t) + 2, (uint64_t **)&d_st));
    BYO_TRY(pinned(ctx, 4096, (void **)&h));
    std::memset(h, 0, sizeof(RoundStats));
    h->count = 1;
    h->outdeg = dsrc;
    int bin = dsrc ? (31 - __builtin_clz(dsrc)) / 2 : 0;
    h->hist[bin > 7 ? 7 : bin] = 1;
    BYO_CU(ctx, cudaMemcpyAsync(d_st, h, sizeof(RoundStats), cudaMemcpyHostToDevice, ctx->stream));
    BYO_TRY(round_policy(g, d_st, 0, false));
    BYO_CU(ctx, cudaMemcpyAsync(h, d_st, sizeof(RoundStats), cudaMemcpyDeviceToHost, ctx->stream));
    BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
    fa.next_mode = (int)h->mode;
    for (int i = 0; i < 16; i++) fa.feat[i] = h->feat[i];
  }
  Frontier *cur = &fa, *nxt = &fb;
  uint32_t nr = 0;
  // small push rounds run back to back in one persistent kernel (not while
  // rounds are timed one by one for the policy's training samples)
  const bool small_ok = !ctx->time_rounds &&
                        (policy == BYO_POLICY_M20 || policy == BYO_POLICY_LEARNED || policy == BYO_POLICY_PUSH);
  const uint64_t small_limit = std::max<uint64_t>(4096, g->m / 20 / 64);
  // a frontier holding a vertex of degree >= 4^5 goes to the round kernels,
  // which give such vertices whole CTAs (and which the learned policy inspects)
  const bool gate_hub = true;
  while (cur->size > 0) {
    int mode;
    switch (policy) {
      case BYO_POLICY_PUSH: mode = MODE_PUSH; break;
      case BYO_POLICY_PULL: mode = MODE_PULL; break;
      case BYO_POLICY_BLOCKED: mode = MODE_BLOCKED; break;
      case BYO_POLICY_M20_BLOCKED: mode = m20_mode(g, *cur, -1, MODE_BLOCKED); break;
      case BYO_POLICY_LEARNED: mode = cur->next_mode; break;  // network, or m/20 if untrained
      default: mode = m20_mode(g, *cur, -1, MODE_PUSH); break;
    }
    if (mode != MODE_PULL && cur->outdeg == 0) break;  // edge_map_data.h:290
    // next's bitmap still holds the frontier before `cur`: clear it
    BYO_TRY(clear_frontier_bits(g, *nxt));
    bool hub = false;
    for (int q = 5; q < 8; q++) hub |= cur->hist[q] != 0;
    if (small_ok && mode == MODE_PUSH && cur->has_list && cur->size + cur->outdeg <= small_limit &&
        !(gate_hub && hub)) {
      RoundStats *d_st = nullptr;
      BYO_TRY(ws(g, WS_STATS, sizeof(RoundStats) / sizeof(uint64_t) + 2, (uint64_t **)&d_st));
      uint32_t R = 0;
      BYO_TRY(bfs_small_rounds(g, st, cur, nxt, small_limit, gate_hub, run_policy ? d_st : nullptr, &R));
      nr += R;
      if (run_policy && cur->size > 0) {
        // the policy for the frontier the kernel stopped at
        RoundStats *h = nullptr;
        BYO_TRY(round_policy(g, d_st, st.reached - cur->size, false));
        BYO_TRY(pinned(ctx, 4096, (void **)&h));
        BYO_CU(ctx, cudaMemcpyAsync(h, d_st, sizeof(RoundStats), cudaMemcpyDeviceToHost, ctx->stream));
        BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
        cur->next_mode = (int)h->mode;
        for (int i = 0; i < 16; i++) cur->feat[i] = h->feat[i];
      }
      continue;
    }
    byo_round_log lg{};
    lg.round = st.round;
    lg.mode = (uint32_t)mode;
    lg.frontier = cur->size;
    lg.frontier_deg = cur->outdeg;
    lg.unvisited = n - st.reached;
    for (int i = 0; i < 16; i++) lg.features[i] = cur->feat[i];
    if (ctx->time_rounds) BYO_CU(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
    nxt->size = 0;
    BYO_TRY(edge_map_round(g, st, *cur, *nxt, mode, tune, run_policy));
    if (ctx->time_rounds) {
      BYO_CU(ctx, cudaEventRecord(ctx->ev[1], ctx->stream));
      BYO_CU(ctx, cudaEventSynchronize(ctx->ev[1]));
      cudaEventElapsedTime(&lg.ms, ctx->ev[0], ctx->ev[1]);
    }
    ctx->rounds.push_back(lg);
    nr++;
    Frontier *t = cur;
    cur = nxt;
    nxt = t;
  }
  if (rounds) *rounds = nr;
  return trav_extract(g, st, d_parent, d_level);
}

}  // namespace byo

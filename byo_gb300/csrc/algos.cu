// algos.cu -- connectivity, PageRank and triangle counting over the shared
// graph view (d_off / d_slots with kSentinel gaps / d_deg).
//
// Connectivity (SimpleUnionAsync semantics, Connectivity.h:32-136): union-find
// that always hooks the larger root under the smaller, so every root is the
// minimum id of its component.  Edges are processed Afforest-style
// (Sutton, Ben-Nun & Barak, IPDPS 2018): link the first kSample neighbours of
// every vertex, compress, pick the most frequent root among sampled vertices,
// then link the remaining edges of vertices outside that component only.  The
// final labels do not depend on the order of links.
//
// PageRank (PageRank.h:125-193): Jacobi pull over warp-sized work units,
// FP32 state with compensated (TwoSum) per-vertex sums, FP64 L1 residual.
// Bytes per iteration: 4 B per slot (ids) + 4 B per slot (p_div gather) +
// 16 B offsets/degrees + 12 B state per vertex.
//
// Triangle counting (Triangle.h:167-204): rank by (degree, id) with the
// device radix sort, keep u->v with rank[u] < rank[v], then count
// |N+(u) cap N+(v)| per DAG edge with lane groups binary-searching the
// shorter list in the longer (gbbs/intersect.h:72-151 uses a merge; the count
// is the same).
#include <algorithm>
#include <cmath>
#include <vector>

#include "device.cuh"
#include "engine.h"
#include "internal.h"
#include "scan.cuh"

namespace byo {

// ================================================================ connectivity

constexpr int kSample = 2;

__device__ __forceinline__ uint32_t ld_parent(const uint32_t *p, uint32_t v) { return __ldcg(p + v); }

// Root of v, with path halving when kHalve; parents only ever point to
// smaller ids.
template <bool kHalve = true>
__device__ __forceinline__ uint32_t cc_find(uint32_t *p, uint32_t v) {
  uint32_t cur = ld_parent(p, v);
  if (cur == v) return v;
  uint32_t prev = v, next;
  while (cur > (next = ld_parent(p, cur))) {
    if (kHalve) p[prev] = next;
    prev = cur;
    cur = next;
  }
  return cur;
}

// Hook the larger root under the smaller until both share a root.
__device__ __forceinline__ void cc_link(uint32_t *p, uint32_t u, uint32_t v) {
  uint32_t ru = cc_find(p, u), rv = cc_find(p, v);
  while (ru != rv) {
    uint32_t hi = ru > rv ? ru : rv, lo = ru > rv ? rv : ru;
    uint32_t old = atomicCAS(p + hi, hi, lo);
    if (old == hi) return;
    // hi got a parent meanwhile: continue from the new roots
    ru = cc_find(p, old);
    rv = cc_find(p, lo);
  }
}

__global__ void k_cc_init(uint32_t *p, uint64_t n) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    p[v] = (uint32_t)v;
}

// Link the first kSample neighbours of every vertex (one thread per vertex).
// Sampling round r (Afforest): every vertex links to its r-th neighbour;
// a compress between rounds keeps the trees flat for the next round's finds.
__global__ void k_cc_sample(const uint64_t *__restrict__ off, const uint32_t *__restrict__ slots,
                            uint32_t *p, uint64_t n, int round) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = off[v], e = off[v + 1];
    if (b + round >= e) continue;  // fewer than round + 1 slots
    // slots b .. b + round: the sampled neighbour is the last when none is a
    // gap (always, on a compact CSR)
    uint32_t x = kSentinel;
    bool gap = false;
    for (int r = 0; r <= round; r++) {
      x = slots[b + r];
      gap |= x == kSentinel;
    }
    if (gap) {  // a gapped view: the round-th neighbour past the gaps
      x = kSentinel;
      int taken = 0;
      for (uint64_t j = b; j < e; j++) {
        const uint32_t y = slots[j];
        if (y == kSentinel) continue;
        if (taken++ == round) {
          x = y;
          break;
        }
      }
    }
    if (x != kSentinel) cc_link(p, (uint32_t)v, x);
  }
}

// Every vertex to its root.  The finds do not halve: a halving store into
// p[w] by a thread passing through w could land after w's own thread wrote
// its root there, and leave a stale ancestor behind the last pass.
__global__ void k_cc_compress(uint32_t *p, uint64_t n) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    p[v] = cc_find<false>(p, (uint32_t)v);
}

// The vertices whose remaining edges must be linked: more than kSample
// neighbours (the first kSample are linked by the sampling rounds) and a root
// other than the giant component's, a thread per vertex, appended to `list`.
// A vertex inside the giant component is skipped entirely: each of its
// neighbours outside it will link the edge from its own side, and roots only
// merge, so a vertex found inside stays inside.
__global__ void __launch_bounds__(256) k_cc_outside(const uint32_t *__restrict__ deg, uint32_t *p, uint64_t n,
                                                    const uint32_t *__restrict__ giant_root, uint32_t *list,
                                                    unsigned long long *count) {
  const uint32_t giant = *giant_root;
  for (uint64_t base = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) & ~31ull; base < n;
       base += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t v = base + lane_id();
    const bool keep = v < n && deg[v] > (uint32_t)kSample && cc_find(p, (uint32_t)v) != giant;
    const uint64_t at = warp_append(keep, count);
    if (keep) list[at] = (uint32_t)v;
  }
}

// Remaining edges of the listed vertices, GS lanes per vertex.
template <int GS>
__global__ void __launch_bounds__(256) k_cc_finish(const uint64_t *__restrict__ off,
                                                   const uint32_t *__restrict__ slots, uint32_t *p,
                                                   const uint32_t *__restrict__ list,
                                                   const unsigned long long *__restrict__ count) {
  const uint64_t nl = *count;
  const unsigned gl = threadIdx.x % GS;
  const uint64_t gid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / GS;
  const uint64_t ng = ((uint64_t)gridDim.x * blockDim.x) / GS;
  for (uint64_t t = gid; t < nl; t += ng) {
    const uint32_t v = list[t];
    const uint64_t b = off[v], e = off[v + 1];
    // skip the first kSample non-gap neighbours: already linked
    uint64_t start = b;
    for (int taken = 0; start < e && taken < kSample; start++)
      if (slots[start] != kSentinel) taken++;
    for (uint64_t j = start + gl; j < e; j += GS) {
      uint32_t u = slots[j];
      if (u == kSentinel) continue;
      cc_link(p, v, u);
    }
  }
}

// The most frequent root among kCcProbe vertices drawn by a fixed hash (the
// giant component, skipped by k_cc_finish): one CTA sorts the roots in
// shared memory and keeps the longest run (ties: the smallest root).
constexpr uint32_t kCcProbe = 1024;
__global__ void __launch_bounds__(kCcProbe) k_cc_giant(const uint32_t *__restrict__ p, uint64_t n, uint64_t seed,
                                                       uint32_t *giant) {
  __shared__ uint32_t s[kCcProbe], st[kCcProbe];
  __shared__ unsigned long long best;
  const uint32_t t = threadIdx.x;
  uint64_t z = seed + (uint64_t)(t + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  s[t] = __ldcg(p + (uint32_t)(((z & 0xFFFFFFFFull) * n) >> 32));
  if (t == 0) best = 0;
  __syncthreads();
  for (uint32_t k = 2; k <= kCcProbe; k <<= 1)
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      const uint32_t x = t ^ j;
      if (x > t) {
        const uint32_t a = s[t], b = s[x];
        if ((a > b) == ((t & k) == 0)) {
          s[t] = b;
          s[x] = a;
        }
      }
      __syncthreads();
    }
  st[t] = (t == 0 || s[t] != s[t - 1]) ? t : 0;  // start of t's run after a max-scan
  __syncthreads();
  for (uint32_t d = 1; d < kCcProbe; d <<= 1) {
    const uint32_t v = t >= d ? st[t - d] : 0;
    __syncthreads();
    if (v > st[t]) st[t] = v;
    __syncthreads();
  }
  if (t == kCcProbe - 1 || s[t] != s[t + 1])
    atomicMax(&best, ((unsigned long long)(t - st[t] + 1) << 32) | (0xFFFFFFFFu - s[t]));
  __syncthreads();
  if (t == 0) *giant = 0xFFFFFFFFu - (uint32_t)best;
}

int cc_run(byo_graph *g, uint32_t *d_label) {
  byo_ctx *ctx = g->ctx;
  const uint64_t n = g->n;
  if (n == 0) return BYO_OK;
  uint32_t *p = d_label;
  launch(ctx, k_cc_init, dim3(grid_for(ctx, n, 256)), dim3(256), 0, p, n);
  for (int r = 0; r < kSample; r++) {
    launch(ctx, k_cc_sample, dim3(grid_for(ctx, n, 256)), dim3(256), 0, (const uint64_t *)g->d_off,
           (const uint32_t *)g->d_slots, p, n, r);
    launch(ctx, k_cc_compress, dim3(grid_for(ctx, n, 256)), dim3(256), 0, p, n);
  }
  uint32_t *giant = nullptr, *list = nullptr;
  BYO_TRY(ws(g, WS_MISC, 4, &giant));  // [0] giant root, [2..3] count of listed vertices
  BYO_TRY(ws(g, WS_FRONT_LIST_A, n, &list));
  unsigned long long *count = reinterpret_cast<unsigned long long *>(giant + 2);
  BYO_CU(ctx, cudaMemsetAsync(count, 0, 8, ctx->stream));
  launch(ctx, k_cc_giant, dim3(1), dim3(kCcProbe), 0, (const uint32_t *)p, n, (uint64_t)0x5EEDull, giant);
  launch(ctx, k_cc_outside, dim3(grid_for(ctx, n, 256)), dim3(256), 0, (const uint32_t *)g->d_deg, p, n,
         (const uint32_t *)giant, list, count);
  const double avg = (double)g->m / (double)n;
  const int GS = avg >= 24 ? 16 : avg >= 8 ? 8 : 4;
  const int grid = grid_for(ctx, n * GS, 256, 16);
  if (GS == 16)
    launch_t(ctx, "cc_finish", k_cc_finish<16>, dim3(grid), dim3(256), 0, (const uint64_t *)g->d_off,
             (const uint32_t *)g->d_slots, p, (const uint32_t *)list, (const unsigned long long *)count);
  else if (GS == 8)
    launch_t(ctx, "cc_finish", k_cc_finish<8>, dim3(grid), dim3(256), 0, (const uint64_t *)g->d_off,
             (const uint32_t *)g->d_slots, p, (const uint32_t *)list, (const unsigned long long *)count);
  else
    launch_t(ctx, "cc_finish", k_cc_finish<4>, dim3(grid), dim3(256), 0, (const uint64_t *)g->d_off,
             (const uint32_t *)g->d_slots, p, (const uint32_t *)list, (const unsigned long long *)count);
  launch(ctx, k_cc_compress, dim3(grid_for(ctx, n, 256)), dim3(256), 0, p, n);
  return check_launch(ctx, "cc");
}

// ---------------------------------------------------------------- BFS-CC

__global__ void k_bfscc_isolated(const uint32_t *__restrict__ deg, uint64_t n, uint32_t *label) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    label[v] = deg[v] == 0 ? (uint32_t)v : kSentinel;
}

__global__ void k_bfscc_first_unlabeled(const uint32_t *__restrict__ label, uint64_t n,
                                        unsigned int *out) {
  uint32_t best = kSentinel;
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    if (label[v] == kSentinel) {
      best = (uint32_t)v;
      break;  // grid-stride order: first hit per thread is its smallest
    }
  if (best != kSentinel) atomicMin(out, best);
}

// label every vertex reached by the traversal (lp set) that has no label yet
__global__ void k_bfscc_assign(const uint64_t *__restrict__ lp, uint64_t n, uint32_t src,
                               uint32_t *label) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    if (label[v] == kSentinel && lp[v] != kNone64) label[v] = src;
}

__global__ void k_trav_seed(uint64_t *lp, uint32_t *visited, uint32_t src) {
  lp[src] = src;
  atomicOr(visited + (src >> 5), 1u << (src & 31));
}

int bfs_cc_run(byo_graph *g, uint32_t *d_label) {
  // BFSCC/Connectivity.h:57-88: components in order of their smallest vertex,
  // one edgeMap traversal each; isolated vertices label themselves.  After
  // kMaxBfs traversals the remaining (small) components are finished by the
  // union-find pass, whose labels (component minimum) are the same.
  byo_ctx *ctx = g->ctx;
  const uint64_t n = g->n, W = (n + 31) / 32;
  if (n == 0) return BYO_OK;
  constexpr int kMaxBfs = 64;
  TravState st;
  Frontier fa, fb;
  BYO_TRY(ws(g, WS_LP, n, &st.lp));
  BYO_TRY(ws(g, WS_VISITED, W, &st.visited));
  BYO_TRY(ws(g, WS_FRONT_LIST_A, n, &fa.list));
  BYO_TRY(ws(g, WS_FRONT_LIST_B, n, &fb.list));
  BYO_TRY(ws(g, WS_FRONT_BITS_A, W, &fa.bits));
  BYO_TRY(ws(g, WS_FRONT_BITS_B, W, &fb.bits));
  unsigned int *d_first = nullptr;
  BYO_TRY(ws(g, WS_MISC, 4, (uint32_t **)&d_first));
  launch(ctx, k_bfscc_isolated, dim3(grid_for(ctx, n, 256)), dim3(256), 0, (const uint32_t *)g->d_deg, n,
         d_label);
  BYO_TRY(trav_init(g, st, 0));
  // start from an empty traversal state: no vertex visited
  BYO_CU(ctx, cudaMemsetAsync(st.lp, 0xFF, n * 8, ctx->stream));
  BYO_CU(ctx, cudaMemsetAsync(st.visited, 0, W * 4, ctx->stream));
  BYO_TRY(memset_async(ctx, fa.bits, 0, W * 4));
  BYO_TRY(memset_async(ctx, fb.bits, 0, W * 4));
  const EngineTuning tune = default_tuning(g);
  uint32_t *h = nullptr;
  BYO_TRY(pinned(ctx, 4096, (void **)&h));
  for (int it = 0; it < kMaxBfs; it++) {
    BYO_CU(ctx, cudaMemsetAsync(d_first, 0xFF, 4, ctx->stream));
    launch(ctx, k_bfscc_first_unlabeled, dim3(grid_for(ctx, n, 256)), dim3(256), 0,
           (const uint32_t *)d_label, n, d_first);
    BYO_CU(ctx, cudaMemcpyAsync(h, d_first, 4, cudaMemcpyDeviceToHost, ctx->stream));
    BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
    const uint32_t s = h[0];
    if (s == kSentinel) return check_launch(ctx, "bfs_cc");
    launch(ctx, k_trav_seed, dim3(1), dim3(1), 0, st.lp, st.visited, s);
    BYO_CU(ctx, cudaMemcpyAsync(fa.list, &s, 4, cudaMemcpyHostToDevice, ctx->stream));
    BYO_TRY(memset_async(ctx, fa.bits, 0, W * 4));
    BYO_TRY(memset_async(ctx, fb.bits, 0, W * 4));
    uint32_t ds = 0;
    BYO_CU(ctx, cudaMemcpyAsync(&ds, g->d_deg + s, 4, cudaMemcpyDeviceToHost, ctx->stream));
    BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
    fa.size = 1;
    fa.outdeg = ds;
    fa.dense = false;
    fa.has_list = true;
    fa.has_bits = false;
    fb.size = 0;
    fb.has_list = true;
    st.round = 1;
    Frontier *cur = &fa, *nxt = &fb;
    while (cur->size > 0 && cur->outdeg > 0) {
      int mode = m20_mode(g, *cur, -1, MODE_PUSH);
      BYO_TRY(clear_frontier_bits(g, *nxt));
      BYO_TRY(edge_map_round(g, st, *cur, *nxt, mode, tune));
      std::swap(cur, nxt);
    }
    // clear both bitmaps for the next traversal
    launch(ctx, k_bfscc_assign, dim3(grid_for(ctx, n, 256)), dim3(256), 0, (const uint64_t *)st.lp, n,
           s, d_label);
  }
  // finish with union-find over the whole graph; keep traversal labels (equal)
  uint32_t *lab2 = nullptr;
  BYO_TRY(ws(g, WS_LABEL, n, &lab2));
  BYO_TRY(cc_run(g, lab2));
  BYO_CU(ctx, cudaMemcpyAsync(d_label, lab2, n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  return check_launch(ctx, "bfs_cc");
}

// ================================================================ PageRank

template <typename T>
struct Acc {
  T s, c;
};

template <bool kComp, typename T>
__device__ __forceinline__ void acc_add(T &s, T &c, T x) {
  if constexpr (kComp) {
    T t = s + x;
    T bb = t - s;
    c += (s - (t - bb)) + (x - bb);
    s = t;
  } else {
    s += x;
  }
}

template <bool kComp, typename T, int GS>
__device__ __forceinline__ T group_total(T s, T c) {
#pragma unroll
  for (int o = GS / 2; o > 0; o >>= 1) {
    T s2 = __shfl_xor_sync(kFull, s, o, GS);
    T c2 = __shfl_xor_sync(kFull, c, o, GS);
    if constexpr (kComp) {
      T t = s + s2;
      T bb = t - s;
      T e = (s - (t - bb)) + (s2 - bb);
      s = t;
      c = c + c2 + e;
    } else {
      s += s2;
    }
  }
  return kComp ? s + c : s;
}

// ---------------------------------------------------------------- PageRank plan
// Work units of at most kPrTile + kPrLightMax slots, all processed by one
// kernel so every CTA streams the same amount:
//   light tile   consecutive vertices with runs <= kPrLightMax; one run of
//                slots; per-vertex sums written directly
//   heavy chunk  kPrTile consecutive slots of one heavier vertex; its
//                compensated partial goes to part[chunk] and k_pr_combine sums
//                a vertex's chunks in order
// A warp gathers a unit's p_div values with plain loads, 16 independent
// loads per lane in flight, into its own stage in shared memory, then reduces
// from the stage (k_pr_units; light tiles by pr_light_tile).
constexpr int kPrTile = 512;            // slots per warp tile / heavy chunk
constexpr uint32_t kPrLightMax = 128;   // longest run of a light vertex
constexpr int kPrBlock = 256;
constexpr int kPrStage = kPrTile + kPrLightMax;  // staged values per warp

struct InLightLen {
  const uint64_t *off;
  __device__ uint64_t operator()(uint64_t v) const {
    uint64_t len = off[v + 1] - off[v];
    return len <= kPrLightMax ? len : 0;
  }
};

// tile starts: v == 0, v heavy, v-1 heavy, the light prefix crossed a
// multiple of kPrTile between v-1 and v, or v is a multiple of kPrTile (so a
// tile never holds more than kPrTile vertices, however many have no edges)
struct InTileStart {
  const uint64_t *off;
  const uint64_t *pre;
  __device__ uint64_t operator()(uint64_t v) const {
    if (v == 0 || v % kPrTile == 0) return 1;
    bool heavy = off[v + 1] - off[v] > kPrLightMax;
    bool prev_heavy = off[v] - off[v - 1] > kPrLightMax;
    return (heavy || prev_heavy || (pre[v] / kPrTile) != (pre[v - 1] / kPrTile)) ? 1 : 0;
  }
};
struct OutTileStart {
  uint32_t *starts;
  __device__ void operator()(uint64_t v, uint64_t pre, uint64_t f) const {
    if (f) starts[pre] = (uint32_t)v;
  }
};
// heavy vertices and their chunk counts
struct InHeavy {
  const uint64_t *off;
  __device__ uint64_t operator()(uint64_t v) const { return off[v + 1] - off[v] > kPrLightMax ? 1 : 0; }
};
struct OutHeavy {
  uint32_t *heavy;
  __device__ void operator()(uint64_t v, uint64_t pre, uint64_t f) const {
    if (f) heavy[pre] = (uint32_t)v;
  }
};
struct InChunks {
  const uint64_t *off;
  const uint32_t *heavy;
  __device__ uint64_t operator()(uint64_t h) const {
    uint32_t v = heavy[h];
    return (off[v + 1] - off[v] + kPrTile - 1) / kPrTile;
  }
};

// Unit descriptor (built once per PageRank call): slot range and either a
// light tile's vertices [v0, v1) or a heavy chunk (v1 == kNoVertex).
struct PrDesc {
  uint64_t s0, s1;
  uint32_t v0, v1;
  uint32_t chunk, pad;
};
constexpr uint32_t kNoVertex = 0xFFFFFFFFu;

// light tiles that are not a lone heavy vertex
struct InLightTile {
  const uint64_t *off;
  const uint32_t *tstart;
  __device__ uint64_t operator()(uint64_t t) const {
    uint32_t v0 = tstart[t], v1 = tstart[t + 1];
    return (v1 - v0 == 1 && off[v1] - off[v0] > kPrLightMax) ? 0 : 1;
  }
};
struct OutLightTile {
  const uint64_t *off;
  const uint32_t *tstart;
  PrDesc *desc;
  __device__ void operator()(uint64_t t, uint64_t pre, uint64_t f) const {
    if (!f) return;
    PrDesc d;
    d.v0 = tstart[t];
    d.v1 = tstart[t + 1];
    d.s0 = off[d.v0];
    d.s1 = off[d.v1];
    d.chunk = 0;
    d.pad = 0;
    desc[pre] = d;
  }
};

// heavy chunks after the light tiles (their count read on the device)
__global__ void k_pr_desc_chunks(const uint64_t *__restrict__ off, const uint32_t *__restrict__ heavy,
                                 const uint64_t *__restrict__ cbase, uint64_t nheavy,
                                 const uint64_t *__restrict__ nlight, PrDesc *desc) {
  const uint64_t base = *nlight;
  for (uint64_t h = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; h < nheavy;
       h += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t v = heavy[h];
    const uint64_t b = off[v], e = off[v + 1];
    for (uint64_t k = 0; k < cbase[h + 1] - cbase[h]; k++) {
      PrDesc d;
      d.s0 = b + k * kPrTile;
      d.s1 = d.s0 + kPrTile < e ? d.s0 + kPrTile : e;
      d.v0 = v;
      d.v1 = kNoVertex;
      d.chunk = (uint32_t)(cbase[h] + k);
      d.pad = cbase[h + 1] - cbase[h] == 1;  // the vertex's only chunk: its unit finishes it
      desc[base + cbase[h] + k] = d;
    }
  }
}

template <bool kComp, typename T>
__device__ __forceinline__ void pr_finish(uint64_t v, T tot, const uint32_t *__restrict__ deg,
                                          const T *__restrict__ p_curr, T *__restrict__ p_next,
                                          T *__restrict__ pdiv_out, T damping, T added, double &l1loc) {
  T p = damping * tot + added;
  p_next[v] = p;
  pdiv_out[v] = p / (T)deg[v];
  l1loc += fabs((double)p_curr[v] - (double)p);
}

// (s, c) += (s2, c2), compensated when kComp (TwoSum of the sums, errors added)
template <bool kComp, typename T>
__device__ __forceinline__ void acc_merge(T &s, T &c, T s2, T c2) {
  if constexpr (kComp) {
    T t = s + s2;
    T bb = t - s;
    T e = (s - (t - bb)) + (s2 - bb);
    s = t;
    c = c + c2 + e;
  } else {
    s += s2;
  }
}

// Per-warp scratch of a light tile beside its stage: a head flag for the first
// slot of every non-empty run.
constexpr uint32_t kPrFlagWords = (kPrStage + 31) / 32;
template <typename T>
constexpr size_t pr_warp_smem() {
  return (size_t)kPrStage * sizeof(T) + kPrFlagWords * 4;
}

// Position of the last head flag below pos (there is one: slot 0 is a head).
__device__ __forceinline__ uint32_t last_head_below(const uint32_t *flags, uint32_t pos) {
  for (int w = (int)((pos - 1) >> 5); w >= 0; w--) {
    uint32_t word = flags[w];
    const uint32_t lim = pos - 32u * (uint32_t)w;  // bits below pos in this word
    if (lim < 32) word &= (1u << lim) - 1u;
    if (word) return 32u * (uint32_t)w + 31u - __clz(word);
  }
  return 0;
}

// Sums of a light tile's runs from the staged values buf[0, len).  Each lane
// takes an odd-length chunk of consecutive slots (odd, so the lanes' reads
// fall in different banks) and sums it in order; the partial of a run that
// crosses chunk boundaries is carried by an inclusive segmented warp scan (a
// lane holding a head starts a new segment) and the run open at a lane's
// start is completed by the lane that holds its end.  Each run's total is
// written over the staged value of its first slot, and a last pass finishes
// the tile's vertices a lane each (consecutive vertices, coalesced).  One
// fixed order per graph, so results are deterministic.
template <bool kComp, typename T>
__device__ __forceinline__ void pr_light_tile(const PrDesc &d, uint32_t len, T *buf, uint32_t *flags,
                                              const uint64_t *__restrict__ off, const uint32_t *__restrict__ deg,
                                              const T *__restrict__ p_curr, T *__restrict__ p_next,
                                              T *__restrict__ pdiv_out, T damping, T added, double &l1loc) {
  const unsigned lane = lane_id();
  for (uint32_t w = lane; w < kPrFlagWords; w += 32) flags[w] = 0;
  __syncwarp();
  for (uint32_t x = d.v0 + lane; x < d.v1; x += 32) {
    const uint64_t a = off[x], b = off[x + 1];
    if (b > a) {
      const uint32_t r0 = (uint32_t)(a - d.s0);
      atomicOr(flags + (r0 >> 5), 1u << (r0 & 31));
    }
  }
  __syncwarp();
  const uint32_t C = ((len + 31) >> 5) | 1u;
  const uint32_t lo = min(lane * C, len), hi = min(lo + C, len);
  T s = T(0), c = T(0), hs = T(0), hc = T(0);
  bool head = false;
  uint32_t hpos = 0, fw = 0;
  for (uint32_t r = lo; r < hi; r++) {
    if (r == lo || (r & 31) == 0) fw = flags[r >> 5];
    if ((fw >> (r & 31)) & 1u) {
      if (!head) {
        hs = s;
        hc = c;
        head = true;
      } else {
        buf[hpos] = kComp ? s + c : s;  // a run inside this chunk
      }
      s = T(0);
      c = T(0);
      hpos = r;
    }
    acc_add<kComp>(s, c, buf[r]);
  }
  T ss = s, sc = c;
  int f = head ? 1 : 0;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T ps = __shfl_up_sync(kFull, ss, o), pc = __shfl_up_sync(kFull, sc, o);
    const int pf = __shfl_up_sync(kFull, f, o);
    if ((int)lane >= o) {
      if (!f) {
        T ts = ps, tc = pc;
        acc_merge<kComp>(ts, tc, ss, sc);
        ss = ts;
        sc = tc;
      }
      f |= pf;
    }
  }
  T cs = __shfl_up_sync(kFull, ss, 1), cc = __shfl_up_sync(kFull, sc, 1);
  __syncwarp();  // every lane's reads of the stage are done
  if (head && lo > 0) {  // the run open at lo ends in this chunk
    acc_merge<kComp>(cs, cc, hs, hc);
    buf[last_head_below(flags, lo)] = kComp ? cs + cc : cs;
  }
  if (lane == 31 && len)  // the run open at the tile's end
    buf[last_head_below(flags, len)] = kComp ? ss + sc : ss;
  __syncwarp();
  for (uint32_t x = d.v0 + lane; x < d.v1; x += 32) {
    const uint64_t a = off[x], b = off[x + 1];
    pr_finish<kComp, T>(x, b > a ? buf[a - d.s0] : T(0), deg, p_curr, p_next, pdiv_out, damping, added, l1loc);
  }
  __syncwarp();
}

// One warp per unit, no block-wide barriers: the warp gathers p_div of the
// unit's slots (16 independent loads per lane in flight) into its own stage in
// shared memory, then reduces.  Light tile: runs of <= 32 one lane each, longer
// runs (found by ballot) one warp each.  Heavy chunk: warp partial to part[];
// with kDirectHeavy (FP64) each lane sums its gathered slots lane, lane+32, ...
// in registers without the stage, in the same order: measured at RMAT 2^22,
// 20 FP64 iterations 34.0 -> 28.8 ms, while FP32 runs 1% faster staged.
template <bool kComp, typename T, bool kDirectHeavy>
__global__ void __launch_bounds__(kPrBlock, 5) k_pr_units(const uint64_t *__restrict__ off,
                                                       const uint32_t *__restrict__ slots,
                                                       const uint32_t *__restrict__ deg,
                                                       const PrDesc *__restrict__ desc,
                                                       const uint64_t *__restrict__ counts,
                                                       const T *__restrict__ pdiv_in, const T *__restrict__ p_curr,
                                                       T *__restrict__ p_next, T *__restrict__ pdiv_out,
                                                       T *__restrict__ part, T damping, T added, double *l1) {
  extern __shared__ __align__(16) unsigned char pr_smem[];
  __shared__ double sm[kPrBlock / 32 + 1];
  const uint64_t nunits = counts[0] + counts[1];  // light tiles + heavy chunks
  const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
  T *buf = reinterpret_cast<T *>(pr_smem) + (size_t)warp * kPrStage;
  uint32_t *flags = reinterpret_cast<uint32_t *>(reinterpret_cast<T *>(pr_smem) + (size_t)(kPrBlock / 32) * kPrStage) +
                    (size_t)warp * kPrFlagWords;
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  double l1loc = 0.0;
  for (uint64_t t = gw; t < nunits; t += nw) {
    const PrDesc d = desc[t];
    const uint32_t len = (uint32_t)(d.s1 - d.s0);
    const uint32_t *id = slots + d.s0;
    if (d.v1 == kNoVertex && kDirectHeavy) {
      T s = T(0), c = T(0);
      for (uint32_t i = lane; i < len; i += 32 * 16) {
        uint32_t u[16];
#pragma unroll
        for (int q = 0; q < 16; q++) u[q] = i + 32 * q < len ? __ldcs(id + i + 32 * q) : kSentinel;
        T g[16];
#pragma unroll
        for (int q = 0; q < 16; q++) g[q] = u[q] != kSentinel ? __ldg(pdiv_in + u[q]) : T(0);
#pragma unroll
        for (int q = 0; q < 16; q++)
          if (i + 32 * q < len) acc_add<kComp>(s, c, g[q]);
      }
      T tot = group_total<kComp, T, 32>(s, c);
      if (lane == 0) {
        if (d.pad) {
          pr_finish<kComp, T>(d.v0, tot, deg, p_curr, p_next, pdiv_out, damping, added, l1loc);
        } else {
          part[2 * (uint64_t)d.chunk] = tot;
          part[2 * (uint64_t)d.chunk + 1] = T(0);
        }
      }
      continue;
    }
    for (uint32_t i = lane; i < len; i += 32 * 16) {
      uint32_t u[16];
#pragma unroll
      for (int q = 0; q < 16; q++) u[q] = i + 32 * q < len ? __ldcs(id + i + 32 * q) : kSentinel;
#pragma unroll
      for (int q = 0; q < 16; q++)
        if (i + 32 * q < len) buf[i + 32 * q] = u[q] != kSentinel ? __ldg(pdiv_in + u[q]) : T(0);
    }
    __syncwarp();
    if (d.v1 != kNoVertex) {
      pr_light_tile<kComp, T>(d, len, buf, flags, off, deg, p_curr, p_next, pdiv_out, damping, added, l1loc);
    } else {
      T s = T(0), c = T(0);
      for (uint32_t r = lane; r < len; r += 32) acc_add<kComp>(s, c, buf[r]);
      T tot = group_total<kComp, T, 32>(s, c);
      if (lane == 0) {
        if (d.pad) {
          pr_finish<kComp, T>(d.v0, tot, deg, p_curr, p_next, pdiv_out, damping, added, l1loc);
        } else {
          part[2 * (uint64_t)d.chunk] = tot;
          part[2 * (uint64_t)d.chunk + 1] = T(0);
        }
      }
    }
    __syncwarp();
  }
  l1loc = block_sum(l1loc, sm);
  if (threadIdx.x == 0 && l1loc != 0.0) atomicAdd(l1, l1loc);
}

// A group of kCombineLanes lanes per heavy vertex (32 / kCombineLanes
// vertices per warp; most heavy vertices have a few chunks): its chunk
// partials, lane l of the group taking chunks l, l + G, ... in order, summed
// by a fixed tree over the group; then the vertex is finished by the group's
// first lane.  Measured at RMAT 2^22 (ms per iteration of units + combine):
// groups of 32 / 8 / 4 lanes 0.563 / 0.543 / 0.549.
constexpr int kCombineLanes = 8;
template <bool kComp, typename T>
__global__ void __launch_bounds__(256) k_pr_combine(const uint32_t *__restrict__ heavy,
                                                    const uint64_t *__restrict__ cbase, uint64_t nheavy,
                                                    const T *__restrict__ part, const uint32_t *__restrict__ deg,
                                                    const T *__restrict__ p_curr, T *__restrict__ p_next,
                                                    T *__restrict__ pdiv_out, T damping, T added, double *l1) {
  __shared__ double sm[9];
  constexpr int kPer = 32 / kCombineLanes;
  const unsigned lane = lane_id(), gl = lane % kCombineLanes;
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  double l1loc = 0.0;
  for (uint64_t base = gw * kPer; base < nheavy; base += nw * kPer) {
    const uint64_t h = base + lane / kCombineLanes;
    T s = T(0), c = T(0);
    bool mine = false;  // a vertex of several chunks (one chunk: finished by its unit)
    if (h < nheavy) {
      const uint64_t c0 = cbase[h], c1 = cbase[h + 1];
      mine = c1 - c0 > 1;
      if (mine)
        for (uint64_t k = c0 + gl; k < c1; k += kCombineLanes) {
          acc_add<kComp>(s, c, part[2 * k]);
          if (kComp) c += part[2 * k + 1];
        }
    }
    const T tot = group_total<kComp, T, kCombineLanes>(s, c);
    if (mine && gl == 0)
      pr_finish<kComp, T>(heavy[h], tot, deg, p_curr, p_next, pdiv_out, damping, added, l1loc);
  }
  l1loc = block_sum(l1loc, sm);
  if (threadIdx.x == 0 && l1loc != 0.0) atomicAdd(l1, l1loc);
}

template <typename T>
__global__ void k_pr_init(const uint32_t *__restrict__ deg, uint64_t n, T *p_curr, T *pdiv, T one_over_n) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    p_curr[v] = one_over_n;
    pdiv[v] = one_over_n / (T)deg[v];
  }
}

// State of the graph-driven iteration loop (device side).
struct PrLoop {
  double l1;
  uint32_t iters;
  int32_t last;  // -1: no iteration ran; 0: the last iterate is in pb; 1: in pa
};

// After an iteration: records its L1 norm, clears the accumulators, and
// tells the loop whether another iteration runs (PageRank.h:176-190: stop
// when L1 < eps or after max_iters).  half 0 ends the first iteration of a
// loop body (pa -> pb) and sets both conditions; half 1 ends the second
// (pb -> pa) and sets the loop's.
__global__ void k_pr_check(double *d_l1, double eps, uint32_t max_iters, PrLoop *st, int half,
                           cudaGraphConditionalHandle h_if, cudaGraphConditionalHandle h_while) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const uint32_t it = ++st->iters;
  const double L = d_l1[0];
  st->l1 = L;
  st->last = half;
  d_l1[0] = 0.0;
  d_l1[1] = 0.0;
  const unsigned cont = (!(L < eps) && it < max_iters) ? 1u : 0u;
  if (half == 0) cudaGraphSetConditional(h_if, cont);
  cudaGraphSetConditional(h_while, cont);
}

// k_pr_check for stream launches: records the iteration's L1 and clears the
// accumulators; the host reads the state and decides.
__global__ void k_pr_check_plain(double *d_l1, PrLoop *st, int half) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  ++st->iters;
  st->l1 = d_l1[0];
  st->last = half;
  d_l1[0] = 0.0;
  d_l1[1] = 0.0;
}

template <typename T>
__global__ void k_to_f64(const T *__restrict__ in, uint64_t n, double *out) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    out[v] = (double)in[v];
}

template <bool kComp, typename T>
static int pagerank_impl(byo_graph *g, double eps, uint32_t max_iters, double *d_p, uint32_t *iters_out,
                         double *l1_out) {
  byo_ctx *ctx = g->ctx;
  const uint64_t n = g->n;
  T *pa, *pb, *da, *db;
  BYO_TRY(ws(g, WS_PR_A, n + 2, &pa));
  BYO_TRY(ws(g, WS_PR_B, n, &pb));
  BYO_TRY(ws(g, WS_PR_C, n, &da));
  BYO_TRY(ws(g, WS_PR_D, n + 2 + (sizeof(PrLoop) + sizeof(T) - 1) / sizeof(T) + 2, &db));  // p_div, loop state
  // plan
  uint64_t *pre = nullptr;
  uint32_t *lists = nullptr;
  BYO_TRY(ws(g, WS_SCAN, 2 * n + 4, &pre));
  uint64_t *cbase = pre + n + 2;
  BYO_TRY(ws(g, WS_BUCKETS, 2 * n + 8, &lists));
  uint32_t *tstart = lists, *heavy = lists + (n + 4);
  double *d_l1 = nullptr;
  BYO_TRY(ws(g, WS_MISC, 8, (uint32_t **)&d_l1));
  uint64_t *counts = reinterpret_cast<uint64_t *>(d_l1 + 2);  // [0] light tiles, [1] heavy chunks
  uint64_t *h = nullptr;
  BYO_TRY(pinned(ctx, 4096, (void **)&h));
  const uint64_t *tot = nullptr;
  BYO_TRY(scan_apply(ctx, n, InLightLen{g->d_off}, OutPrefix{pre}, &tot));
  BYO_TRY(scan_apply(ctx, n, InTileStart{g->d_off, pre}, OutTileStart{tstart}, &tot));
  BYO_CU(ctx, cudaMemcpyAsync(h, tot, 8, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_TRY(scan_apply(ctx, n, InHeavy{g->d_off}, OutHeavy{heavy}, &tot));
  BYO_CU(ctx, cudaMemcpyAsync(h + 1, tot, 8, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  const uint64_t ntiles = h[0], nheavy = h[1];
  // From here the plan stays on the device: the counts of light tiles and
  // heavy chunks go to `counts`, which k_pr_desc_chunks and k_pr_units read,
  // and the buffers and grid are sized by upper bounds (a heavy vertex of d
  // slots makes ceil(d / kPrTile) chunks), so the host builds the graph
  // below while the GPU finishes the plan.
  BYO_TRY(scan_apply(ctx, nheavy, InChunks{g->d_off, heavy}, OutPrefix{cbase}, &tot));
  BYO_CU(ctx, cudaMemcpyAsync(cbase + nheavy, tot, 8, cudaMemcpyDeviceToDevice, ctx->stream));
  BYO_CU(ctx, cudaMemcpyAsync(counts + 1, tot, 8, cudaMemcpyDeviceToDevice, ctx->stream));
  h[3] = n;  // h[3] is not written again before the next synchronisation
  BYO_CU(ctx, cudaMemcpyAsync(tstart + ntiles, h + 3, 4, cudaMemcpyHostToDevice, ctx->stream));
  launch(ctx, k_pr_init<T>, dim3(grid_for(ctx, n, 256)), dim3(256), 0, (const uint32_t *)g->d_deg, n, pa, da,
         (T)(1.0 / (double)n));
  const uint64_t max_chunks = g->nslots / kPrTile + nheavy + 1;
  // descriptors: compacted light tiles, then heavy chunks
  PrDesc *desc = nullptr;
  BYO_TRY(ws(g, WS_TC_NBR, (ntiles + max_chunks + 1) * sizeof(PrDesc) / 4, (uint32_t **)&desc));
  BYO_TRY(scan_apply(ctx, ntiles, InLightTile{g->d_off, tstart}, OutLightTile{g->d_off, tstart, desc}, &tot));
  BYO_CU(ctx, cudaMemcpyAsync(counts, tot, 8, cudaMemcpyDeviceToDevice, ctx->stream));
  if (nheavy)
    launch(ctx, k_pr_desc_chunks, dim3(grid_for(ctx, nheavy, 256)), dim3(256), 0, (const uint64_t *)g->d_off,
           (const uint32_t *)heavy, (const uint64_t *)cbase, nheavy, (const uint64_t *)counts, desc);
  T *part = nullptr;
  BYO_TRY(ws(g, WS_TC_CNT, 2 * max_chunks + 2, &part));
  const T damping = (T)0.85;
  const T added = (T)((1 - 0.85) * (1 / (double)n));
  const int grid_c = grid_for(ctx, nheavy * kCombineLanes, 256, 8);
  const size_t units_smem = (size_t)(kPrBlock / 32) * pr_warp_smem<T>();
  BYO_CU(ctx, cudaFuncSetAttribute(k_pr_units<kComp, T, sizeof(T) == 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)units_smem));
  int units_per_sm = 0;
  BYO_CU(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&units_per_sm, k_pr_units<kComp, T, sizeof(T) == 8>,
                                                            kPrBlock, units_smem));
  const int grid_u = grid_for(ctx, (ntiles + max_chunks) * 32, kPrBlock, units_per_sm > 0 ? units_per_sm : 1);
  // The iterations run as one CUDA graph: a WHILE node whose body holds two
  // iterations (pa -> pb, then under an IF node pb -> pa), each ending in
  // k_pr_check, which sets the conditions from the L1 norm on the device.
  // No host round trip happens between iterations.
  PrLoop *loop = reinterpret_cast<PrLoop *>((reinterpret_cast<uintptr_t>(db + n + 2) + 7) & ~(uintptr_t)7);
  BYO_CU(ctx, cudaMemsetAsync(d_l1, 0, 16, ctx->stream));
  {
    PrLoop z{0.0, 0u, -1};
    BYO_CU(ctx, cudaMemcpyAsync(loop, &z, sizeof(PrLoop), cudaMemcpyHostToDevice, ctx->stream));
  }
  uint32_t it = 0;
  double L1 = 0.0;
  const T *last = pa;
  if (max_iters > 0 && !ctx->pr_graphs) {
    // one stream launch per kernel and a host check of the residual after
    // each iteration (the same kernels in the same order: the same results)
    PrLoop *hs = nullptr;
    BYO_TRY(pinned(ctx, 4096, (void **)&hs));
    const T *pdiv_in[2] = {da, db}, *pcur[2] = {pa, pb};
    T *pnext[2] = {pb, pa}, *pdiv_out[2] = {db, da};
    for (int hh = 0;; hh ^= 1) {
      launch_t(ctx, "pr_pull", k_pr_units<kComp, T, sizeof(T) == 8>, dim3(grid_u), dim3(kPrBlock), units_smem,
               (const uint64_t *)g->d_off, (const uint32_t *)g->d_slots, (const uint32_t *)g->d_deg,
               (const PrDesc *)desc, (const uint64_t *)counts, pdiv_in[hh], pcur[hh], pnext[hh], pdiv_out[hh], part,
               damping, added, d_l1);
      if (nheavy)
        launch_t(ctx, "pr_pull", k_pr_combine<kComp, T>, dim3(grid_c), dim3(256), 0, (const uint32_t *)heavy,
                 (const uint64_t *)cbase, nheavy, (const T *)part, (const uint32_t *)g->d_deg, pcur[hh], pnext[hh],
                 pdiv_out[hh], damping, added, d_l1);
      launch(ctx, k_pr_check_plain, dim3(1), dim3(32), 0, d_l1, loop, hh);
      BYO_CU(ctx, cudaMemcpyAsync(hs, loop, sizeof(PrLoop), cudaMemcpyDeviceToHost, ctx->stream));
      BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
      if (hs->l1 < eps || hs->iters >= max_iters) break;
    }
    it = hs->iters;
    L1 = hs->l1;
    last = hs->last == 0 ? pb : pa;
  } else if (max_iters > 0) {
    cudaGraph_t graph = nullptr, body = nullptr, second = nullptr;
    cudaGraphExec_t exec = nullptr;
    int rc = BYO_OK;
    auto fail = [&](const char *what, cudaError_t e) {
      if (rc == BYO_OK) rc = set_error(ctx, BYO_EDEVICE, what, e);
    };
    cudaError_t e = cudaGraphCreate(&graph, 0);
    if (e != cudaSuccess) fail("pagerank graph", e);
    cudaGraphConditionalHandle h_while = 0, h_if = 0;
    cudaGraphNode_t wnode = nullptr, inode = nullptr;
    if (rc == BYO_OK && (e = cudaGraphConditionalHandleCreate(&h_while, graph, 1, cudaGraphCondAssignDefault)) !=
                            cudaSuccess)
      fail("pagerank loop condition", e);
    if (rc == BYO_OK) {
      cudaGraphNodeParams wp = {};
      wp.type = cudaGraphNodeTypeConditional;
      wp.conditional.handle = h_while;
      wp.conditional.type = cudaGraphCondTypeWhile;
      wp.conditional.size = 1;
      if ((e = cudaGraphAddNode(&wnode, graph, nullptr, nullptr, 0, &wp)) != cudaSuccess) fail("pagerank loop", e);
      else body = wp.conditional.phGraph_out[0];
    }
    if (rc == BYO_OK &&
        (e = cudaGraphConditionalHandleCreate(&h_if, graph, 0, cudaGraphCondAssignDefault)) != cudaSuccess)
      fail("pagerank half condition", e);
    // one iteration: units, combine, check; returns its last node
    const uint64_t *off_ = g->d_off;
    const uint32_t *slots_ = g->d_slots, *deg_ = g->d_deg, *heavy_ = heavy;
    const uint64_t *cbase_ = cbase;
    const PrDesc *desc_ = desc;
    const uint64_t *counts_ = counts;
    T *pa_ = pa, *pb_ = pb, *da_ = da, *db_ = db;
    double *l1_ = d_l1;
    PrLoop *loop_ = loop;
    const double eps_ = eps;
    const uint32_t maxit_ = max_iters;
    T damping_ = damping, added_ = added;
    uint64_t nheavy_ = nheavy;
    int half0 = 0, half1 = 1;
    const T *pdiv_in[2] = {da_, db_}, *pcur[2] = {pa_, pb_};
    T *pnext[2] = {pb_, pa_}, *pdiv_out[2] = {db_, da_};
    auto add_iter = [&](cudaGraph_t gr, int h, cudaGraphNode_t dep, cudaGraphNode_t *lastn) {
      if (rc != BYO_OK) return;
      cudaKernelNodeParams kp = {};
      cudaGraphNode_t nu = nullptr, nc = nullptr, nk = nullptr;
      void *ua[] = {(void *)&off_, (void *)&slots_, (void *)&deg_, (void *)&desc_, (void *)&counts_,
                    (void *)&pdiv_in[h], (void *)&pcur[h], (void *)&pnext[h], (void *)&pdiv_out[h], (void *)&part,
                    (void *)&damping_, (void *)&added_, (void *)&l1_};
      kp.func = (void *)k_pr_units<kComp, T, sizeof(T) == 8>;
      kp.gridDim = dim3(grid_u);
      kp.blockDim = dim3(kPrBlock);
      kp.sharedMemBytes = (unsigned)units_smem;
      kp.kernelParams = ua;
      cudaError_t x = cudaGraphAddKernelNode(&nu, gr, dep ? &dep : nullptr, dep ? 1 : 0, &kp);
      kp.sharedMemBytes = 0;
      if (x != cudaSuccess) return fail("pagerank units node", x);
      cudaGraphNode_t prev = nu;
      if (nheavy_) {
        void *ca[] = {(void *)&heavy_, (void *)&cbase_, (void *)&nheavy_, (void *)&part, (void *)&deg_,
                      (void *)&pcur[h], (void *)&pnext[h], (void *)&pdiv_out[h], (void *)&damping_, (void *)&added_,
                      (void *)&l1_};
        kp.func = (void *)k_pr_combine<kComp, T>;
        kp.gridDim = dim3(grid_c);
        kp.blockDim = dim3(256);
        kp.kernelParams = ca;
        x = cudaGraphAddKernelNode(&nc, gr, &prev, 1, &kp);
        if (x != cudaSuccess) return fail("pagerank combine node", x);
        prev = nc;
      }
      void *ka[] = {(void *)&l1_, (void *)&eps_, (void *)&maxit_, (void *)&loop_, (void *)(h ? &half1 : &half0),
                    (void *)&h_if, (void *)&h_while};
      kp.func = (void *)k_pr_check;
      kp.gridDim = dim3(1);
      kp.blockDim = dim3(32);
      kp.kernelParams = ka;
      x = cudaGraphAddKernelNode(&nk, gr, &prev, 1, &kp);
      if (x != cudaSuccess) return fail("pagerank check node", x);
      *lastn = nk;
    };
    cudaGraphNode_t k0 = nullptr, k1 = nullptr;
    add_iter(body, 0, nullptr, &k0);
    if (rc == BYO_OK) {
      cudaGraphNodeParams ip = {};
      ip.type = cudaGraphNodeTypeConditional;
      ip.conditional.handle = h_if;
      ip.conditional.type = cudaGraphCondTypeIf;
      ip.conditional.size = 1;
      if ((e = cudaGraphAddNode(&inode, body, &k0, nullptr, 1, &ip)) != cudaSuccess) fail("pagerank half", e);
      else second = ip.conditional.phGraph_out[0];
    }
    add_iter(second, 1, nullptr, &k1);
    if (rc == BYO_OK && (e = cudaGraphInstantiate(&exec, graph, 0)) != cudaSuccess) fail("pagerank instantiate", e);
    if (rc == BYO_OK) {
      const bool timed = !ctx->ktag.empty() && ktimer_begin(ctx, "pr_pull");
      if ((e = cudaGraphLaunch(exec, ctx->stream)) != cudaSuccess) fail("pagerank launch", e);
      if (timed) ktimer_end(ctx);
      ctx->launches += 1;
    }
    PrLoop hs{0.0, 0u, -1};
    if (rc == BYO_OK && (e = cudaMemcpyAsync(&hs, loop, sizeof(PrLoop), cudaMemcpyDeviceToHost, ctx->stream)) !=
                            cudaSuccess)
      fail("pagerank state", e);
    if (rc == BYO_OK && (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) fail("pagerank sync", e);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    BYO_TRY(rc);
    ctx->launches += (uint64_t)(nheavy ? 3 : 2) * hs.iters - 1;  // kernels the graph ran
    it = hs.iters;
    L1 = hs.l1;
    last = hs.last == 0 ? pb : pa;
  }
  // the last computed iterate (the reference's final swap would hand back the
  // zeroed previous one when max_iters ends the loop, PageRank.h:181-192)
  launch(ctx, k_to_f64<T>, dim3(grid_for(ctx, n, 256)), dim3(256), 0, last, n, d_p);
  if (iters_out) *iters_out = it;
  if (l1_out) *l1_out = L1;
  return check_launch(ctx, "pagerank");
}

int pagerank_run(byo_graph *g, double eps, uint32_t max_iters, int precision, double *d_p,
                 uint32_t *iters, double *l1) {
  if (g->n == 0) return BYO_OK;
  switch (precision) {
    case BYO_PR_FP32_KAHAN: return pagerank_impl<true, float>(g, eps, max_iters, d_p, iters, l1);
    case BYO_PR_FP64: return pagerank_impl<false, double>(g, eps, max_iters, d_p, iters, l1);
    case BYO_PR_FP32: return pagerank_impl<false, float>(g, eps, max_iters, d_p, iters, l1);
    default: return set_error(g->ctx, BYO_EINVAL, "pagerank: unknown precision");
  }
}

// ================================================================ triangle counting

__global__ void k_tc_rank_keys(const uint32_t *__restrict__ deg, uint64_t n, uint64_t *keys) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    keys[v] = ((uint64_t)deg[v] << 32) | v;
}

__global__ void k_tc_rank_scatter(const uint64_t *__restrict__ sorted, uint64_t n, uint32_t *rank) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    rank[(uint32_t)sorted[i]] = (uint32_t)i;
}

// out-degree in the DAG: neighbours of higher rank
__global__ void k_tc_count(const uint64_t *__restrict__ off, const uint32_t *__restrict__ slots,
                           const uint32_t *__restrict__ rank, uint64_t n, uint32_t *dcnt) {
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t v = gw; v < n; v += nw) {
    const uint32_t rv = rank[v];
    const uint64_t b = off[v], e = off[v + 1];
    uint32_t c = 0;
    for (uint64_t j = b + lane_id(); j < e; j += 32) {
      uint32_t u = slots[j];
      c += (u != kSentinel && rank[u] > rv);
    }
    c = warp_sum(c);
    if (lane_id() == 0) dcnt[v] = c;
  }
}

__global__ void k_tc_fill(const uint64_t *__restrict__ off, const uint32_t *__restrict__ slots,
                          const uint32_t *__restrict__ rank, uint64_t n,
                          const uint64_t *__restrict__ doff, uint32_t *dn) {
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t v = gw; v < n; v += nw) {
    const uint32_t rv = rank[v];
    const uint64_t b = off[v], e = off[v + 1];
    uint64_t w = doff[v];
    for (uint64_t base = b; base < e; base += 32) {
      uint64_t j = base + lane_id();
      uint32_t u = j < e ? slots[j] : kSentinel;
      bool keep = u != kSentinel && rank[u] > rv;
      unsigned m = __ballot_sync(kFull, keep);
      if (keep) dn[w + __popc(m & lanemask_lt())] = u;
      w += __popc(m);
    }
  }
}

// Wedge counting over the DAG.  For a vertex u, A = N+(u) is staged in
// shared memory; every w of N+(v) for v in A is looked up in A by binary
// search, and each hit is one triangle (u, v, w) with rank(u) < rank(v) <
// rank(w), so every triangle counts once (Triangle.h:99-150 counts the same
// |N+(u) cap N+(v)| per DAG edge).  A warp enumerates the wedges of 32 v's at
// a time flattened by a warp scan over their out-degrees, so lanes stay busy
// whatever the degrees.
constexpr uint32_t kTcWarpCap = 512;  // N+(u) a warp stages (2 KB per warp)

__device__ __forceinline__ bool tc_member(const uint32_t *A, uint32_t na, uint32_t x) {
  uint32_t lo = 0, hi = na;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (A[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo < na && A[lo] == x;
}

// N+(u) as a sorted array (binary search) or as an open-addressing hash set
// in shared memory (linear probing, load <= 1/2: about two probes a lookup
// against log2 |N+(u)| steps).
struct TcSorted {
  const uint32_t *A;
  uint32_t na;
  __device__ __forceinline__ bool has(uint32_t x) const { return tc_member(A, na, x); }
};
struct TcHash {
  const uint32_t *t;
  uint32_t mask, shift;
  __device__ __forceinline__ bool has(uint32_t x) const {
    uint32_t h = (x * 0x9E3779B1u) >> shift;
    for (;;) {
      const uint32_t y = t[h];
      if (y == x) return true;
      if (y == kSentinel) return false;
      h = (h + 1) & mask;
    }
  }
};
constexpr uint32_t kTcHash = 2 * kTcWarpCap;  // table entries per warp

// Wedges of the v's at positions c, c + stride, ... (chunks of 32) of V =
// N+(u), each w of N+(v) looked up in S.  Warp-collective; pre/bas are this
// warp's 32-entry scratch.
template <class Set>
__device__ __forceinline__ uint64_t tc_wedges(const uint64_t *__restrict__ doff, const uint32_t *__restrict__ dn,
                                              const uint32_t *A, uint32_t na, uint32_t c0, uint32_t stride,
                                              uint32_t *pre, uint64_t *bas, const Set &S) {
  const unsigned lane = lane_id();
  uint64_t cnt = 0;
  for (uint32_t c = c0; c < na; c += stride) {
    const uint32_t i = c + lane;
    uint32_t d = 0;
    uint64_t b = 0;
    if (i < na) {
      const uint32_t v = A[i];
      b = doff[v];
      d = (uint32_t)(doff[v + 1] - b);
    }
    const uint32_t incl = warp_inclusive_scan(d);
    pre[lane] = incl;
    bas[lane] = b;
    __syncwarp();
    const uint32_t total = __shfl_sync(kFull, incl, 31);
    uint32_t lo = 0;  // first lane whose inclusive prefix exceeds t: a binary search for
    if (lane < total) {  // the lane's first t, then a forward walk as t rises by 32
      uint32_t hi = 31;
      while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (pre[mid] <= lane) lo = mid + 1; else hi = mid;
      }
    }
    for (uint32_t t = lane; t < total; t += 32) {
      while (pre[lo] <= t) lo++;
      const uint32_t start = lo ? pre[lo - 1] : 0;
      const uint32_t w = dn[bas[lo] + (t - start)];
      cnt += S.has(w);
    }
    __syncwarp();
  }
  return cnt;
}

// A warp per vertex with 2 <= |N+(u)| <= kTcWarpCap: N+(u) goes into a hash
// set of the next power of two >= 4 |N+(u)| entries (at least 64, at most
// kTcHash) in the warp's shared memory; the v's are read from the list itself.
__global__ void __launch_bounds__(256) k_tc_warp(const uint64_t *__restrict__ doff, const uint32_t *__restrict__ dn,
                                                 uint64_t n, unsigned long long *total) {
  __shared__ uint32_t Ht[8][kTcHash];
  __shared__ uint32_t pre[8][32];
  __shared__ uint64_t bas[8][32];
  __shared__ unsigned long long sm[9];
  const unsigned w = threadIdx.x >> 5, lane = lane_id();
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  uint32_t *tab = Ht[w];
  uint64_t cnt = 0;
  for (uint64_t u = gw; u < n; u += nw) {
    const uint64_t ab = doff[u];
    const uint32_t na = (uint32_t)(doff[u + 1] - ab);
    if (na < 2 || na > kTcWarpCap) continue;
    // 2^lg >= 4 na up to the table's kTcHash entries (>= 2 na): load <= 1/4
    // for most vertices, so a miss (most lookups) ends after ~1.4 probes
    const uint32_t lg = min(31 - __clz((int)kTcHash), max(6, 32 - __clz((int)(4 * na - 1))));
    const uint32_t size = 1u << lg, mask = size - 1, shift = 32 - lg;
    for (uint32_t i = lane; i < size; i += 32) tab[i] = kSentinel;
    __syncwarp();
    for (uint32_t i = lane; i < na; i += 32) {
      const uint32_t x = dn[ab + i];
      uint32_t h = (x * 0x9E3779B1u) >> shift;
      while (atomicCAS(tab + h, kSentinel, x) != kSentinel) h = (h + 1) & mask;
    }
    __syncwarp();
    cnt += tc_wedges(doff, dn, dn + ab, na, 0, 32, pre[w], bas[w], TcHash{tab, mask, shift});
    __syncwarp();
  }
  const unsigned long long tot = block_sum((unsigned long long)cnt, sm);
  if (threadIdx.x == 0 && tot) atomicAdd(total, tot);
}

// A CTA per vertex with |N+(u)| > kTcWarpCap (listed in big[]); N+(u) is
// staged in dynamic shared memory when it fits `stage` entries, else read in
// place.  The CTA's warps take interleaved chunks of 32 v's.
__global__ void __launch_bounds__(256) k_tc_block(const uint64_t *__restrict__ doff, const uint32_t *__restrict__ dn,
                                                  const uint32_t *__restrict__ big, const unsigned long long *nbig,
                                                  uint32_t stage, unsigned long long *total) {
  extern __shared__ uint32_t Ablk[];
  __shared__ uint32_t pre[8][32];
  __shared__ uint64_t bas[8][32];
  __shared__ unsigned long long sm[9];
  const unsigned w = threadIdx.x >> 5, nwb = blockDim.x >> 5;
  const uint64_t nb = *nbig;
  uint64_t cnt = 0;
  for (uint64_t k = blockIdx.x; k < nb; k += gridDim.x) {
    const uint32_t u = big[k];
    const uint64_t ab = doff[u];
    const uint32_t na = (uint32_t)(doff[u + 1] - ab);
    const uint32_t *A = dn + ab;
    if (na <= stage) {
      for (uint32_t i = threadIdx.x; i < na; i += blockDim.x) Ablk[i] = dn[ab + i];
      A = Ablk;
    }
    __syncthreads();
    cnt += tc_wedges(doff, dn, A, na, w * 32, nwb * 32, pre[w], bas[w], TcSorted{A, na});
    __syncthreads();
  }
  const unsigned long long tot = block_sum((unsigned long long)cnt, sm);
  if (threadIdx.x == 0 && tot) atomicAdd(total, tot);
}

__global__ void k_tc_big(const uint64_t *__restrict__ doff, uint64_t n, uint32_t *big, unsigned long long *nbig) {
  for (uint64_t base = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) & ~31ull; base < n;
       base += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t u = base + lane_id();
    const bool b = u < n && doff[u + 1] - doff[u] > kTcWarpCap;
    const uint64_t at = warp_append(b, nbig);
    if (b) big[at] = (uint32_t)u;
  }
}

int tc_run(byo_graph *g, uint64_t *count) {
  byo_ctx *ctx = g->ctx;
  const uint64_t n = g->n;
  *count = 0;
  if (n == 0) return BYO_OK;
  uint64_t *keys = nullptr, *tmp = nullptr;
  BYO_TRY(ws(g, WS_TC_OFF, 2 * n + 2, &keys));
  tmp = keys + n + 1;
  launch(ctx, k_tc_rank_keys, dim3(grid_for(ctx, n, 256)), dim3(256), 0, (const uint32_t *)g->d_deg, n, keys);
  uint64_t maxdeg_mask = 0xFFFFFFFFull;  // degree bits
  uint64_t id_mask = sig_mask_for(n) & 0xFFFFFFFFull;
  uint64_t *sorted = nullptr;
  BYO_TRY(sort_u64(ctx, keys, tmp, n, (maxdeg_mask << 32) | id_mask, &sorted));
  uint32_t *rank = nullptr;
  BYO_TRY(ws(g, WS_TC_RANK, n, &rank));
  launch(ctx, k_tc_rank_scatter, dim3(grid_for(ctx, n, 256)), dim3(256), 0, (const uint64_t *)sorted, n,
         rank);
  uint32_t *dcnt = nullptr;
  BYO_TRY(ws(g, WS_TC_CNT, n, &dcnt));
  launch(ctx, k_tc_count, dim3(grid_for(ctx, n * 32, 256, 16)), dim3(256), 0, (const uint64_t *)g->d_off,
         (const uint32_t *)g->d_slots, (const uint32_t *)rank, n, dcnt);
  uint64_t *doff = keys;  // reuse: sorted keys no longer needed
  BYO_TRY(scan_u32_to_u64(ctx, dcnt, n, doff));
  uint64_t *h = nullptr;
  BYO_TRY(pinned(ctx, 4096, (void **)&h));
  BYO_CU(ctx, cudaMemcpyAsync(h, doff + n, 8, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  const uint64_t md = h[0];
  uint32_t *dn = nullptr;
  BYO_TRY(ws(g, WS_TC_NBR, md + 1, &dn));
  launch(ctx, k_tc_fill, dim3(grid_for(ctx, n * 32, 256, 16)), dim3(256), 0, (const uint64_t *)g->d_off,
         (const uint32_t *)g->d_slots, (const uint32_t *)rank, n, (const uint64_t *)doff, dn);
  unsigned long long *d_total = nullptr;
  BYO_TRY(ws(g, WS_MISC, 4, (uint32_t **)&d_total));
  BYO_CU(ctx, cudaMemsetAsync(d_total, 0, 16, ctx->stream));  // total, big count
  uint32_t *big = dcnt;  // reuse: the counts are in doff now
  launch(ctx, k_tc_big, dim3(grid_for(ctx, n, 256)), dim3(256), 0, (const uint64_t *)doff, n, big, d_total + 1);
  launch_t(ctx, "tc_intersect", k_tc_warp, dim3(grid_for(ctx, n * 32, 256, 8)), dim3(256), 0,
           (const uint64_t *)doff, (const uint32_t *)dn, n, d_total);
  const byo_tuning tn = effective_tuning(g);
  const uint32_t stage = tn.tc_stage;
  static int configured = 0;
  const int smem = (int)(stage * 4);
  if (smem > 48 * 1024 && configured < smem) {
    BYO_CU(ctx, cudaFuncSetAttribute(k_tc_block, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    configured = smem;
  }
  launch_t(ctx, "tc_intersect", k_tc_block, dim3(ctx->num_sms), dim3(256), (size_t)smem, (const uint64_t *)doff,
           (const uint32_t *)dn, (const uint32_t *)big, (const unsigned long long *)(d_total + 1), stage, d_total);
  BYO_CU(ctx, cudaMemcpyAsync(h, d_total, 8, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  *count = h[0];
  return check_launch(ctx, "triangle_count");
}

}  // namespace byo

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
// PageRank (PageRank.h:125-193): Jacobi pull with lane groups per vertex,
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
#include <unordered_map>
#include <vector>

#include "device.cuh"
#include "engine.h"
#include "internal.h"
#include "scan.cuh"

namespace byo {

// ================================================================ connectivity

constexpr int kSample = 2;

__device__ __forceinline__ uint32_t ld_parent(const uint32_t *p, uint32_t v) { return __ldcg(p + v); }

// Root of v with path halving; parents only ever point to smaller ids.
__device__ __forceinline__ uint32_t cc_find(uint32_t *p, uint32_t v) {
  uint32_t cur = ld_parent(p, v);
  if (cur == v) return v;
  uint32_t prev = v, next;
  while (cur > (next = ld_parent(p, cur))) {
    p[prev] = next;
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
__global__ void k_cc_sample(const uint64_t *__restrict__ off, const uint32_t *__restrict__ slots,
                            uint32_t *p, uint64_t n) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = off[v], e = off[v + 1];
    int taken = 0;
    for (uint64_t j = b; j < e && taken < kSample; j++) {
      uint32_t u = slots[j];
      if (u == kSentinel) continue;
      taken++;
      cc_link(p, (uint32_t)v, u);
    }
  }
}

__global__ void k_cc_compress(uint32_t *p, uint64_t n) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    p[v] = cc_find(p, (uint32_t)v);
}

// Remaining edges of vertices outside the giant component; GS lanes per
// vertex.  A vertex inside the giant component is skipped entirely: each of
// its neighbours outside it will link the edge from its own side.
template <int GS>
__global__ void __launch_bounds__(256) k_cc_finish(const uint64_t *__restrict__ off,
                                                   const uint32_t *__restrict__ slots, uint32_t *p,
                                                   uint64_t n, uint32_t giant) {
  const unsigned gl = threadIdx.x % GS;
  const uint64_t gid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / GS;
  const uint64_t ng = ((uint64_t)gridDim.x * blockDim.x) / GS;
  for (uint64_t v = gid; v < n; v += ng) {
    if (cc_find(p, (uint32_t)v) == giant) continue;
    const uint64_t b = off[v], e = off[v + 1];
    // skip the first kSample non-gap neighbours: already linked
    uint64_t start = b;
    for (int taken = 0; start < e && taken < kSample; start++)
      if (slots[start] != kSentinel) taken++;
    for (uint64_t j = start + gl; j < e; j += GS) {
      uint32_t u = slots[j];
      if (u == kSentinel) continue;
      cc_link(p, (uint32_t)v, u);
    }
  }
}

__global__ void k_gather_u32(const uint32_t *__restrict__ src, uint64_t n, uint64_t seed, uint32_t cnt,
                             uint32_t *out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
    uint64_t z = seed + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    out[i] = src[(uint32_t)(((z & 0xFFFFFFFFull) * n) >> 32)];
  }
}

int cc_run(byo_graph *g, uint32_t *d_label) {
  byo_ctx *ctx = g->ctx;
  const uint64_t n = g->n;
  if (n == 0) return BYO_OK;
  uint32_t *p = d_label;
  launch(ctx, k_cc_init, dim3(grid_for(ctx, n, 256)), dim3(256), 0, p, n);
  launch(ctx, k_cc_sample, dim3(grid_for(ctx, n, 256)), dim3(256), 0, (const uint64_t *)g->d_off,
         (const uint32_t *)g->d_slots, p, n);
  launch(ctx, k_cc_compress, dim3(grid_for(ctx, n, 256)), dim3(256), 0, p, n);
  // most frequent root among 1024 sampled vertices
  constexpr uint32_t kProbe = 1024;
  uint32_t *probe = nullptr;
  BYO_TRY(ws(g, WS_MISC, kProbe, &probe));
  launch(ctx, k_gather_u32, dim3(4), dim3(256), 0, (const uint32_t *)p, n, (uint64_t)0x5EEDull, kProbe,
         probe);
  uint32_t *h = nullptr;
  BYO_TRY(pinned(ctx, 4096 + kProbe * 4, (void **)&h));
  BYO_CU(ctx, cudaMemcpyAsync(h, probe, kProbe * 4, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  std::unordered_map<uint32_t, uint32_t> freq;
  uint32_t giant = h[0], best = 0;
  for (uint32_t i = 0; i < kProbe; i++) {
    uint32_t c = ++freq[h[i]];
    if (c > best) {
      best = c;
      giant = h[i];
    }
  }
  const double avg = (double)g->m / (double)n;
  const int GS = avg >= 24 ? 16 : avg >= 8 ? 8 : 4;
  const int grid = grid_for(ctx, n * GS, 256, 16);
  if (GS == 16)
    launch_t(ctx, "cc_finish", k_cc_finish<16>, dim3(grid), dim3(256), 0, (const uint64_t *)g->d_off,
           (const uint32_t *)g->d_slots, p, n, giant);
  else if (GS == 8)
    launch_t(ctx, "cc_finish", k_cc_finish<8>, dim3(grid), dim3(256), 0, (const uint64_t *)g->d_off,
           (const uint32_t *)g->d_slots, p, n, giant);
  else
    launch_t(ctx, "cc_finish", k_cc_finish<4>, dim3(grid), dim3(256), 0, (const uint64_t *)g->d_off,
           (const uint32_t *)g->d_slots, p, n, giant);
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
// Vertices are split by slot-range length: light (<= kPrLightMax) vertices are
// packed into tiles of consecutive ids whose ranges total about kPrTile slots;
// medium vertices get a warp each, hubs (> kPrHubMin) a CTA each.  A tile
// never spans a heavier vertex, so its slots are one contiguous run.
constexpr int kPrTile = 4096;
constexpr uint32_t kPrLightMax = 512;
constexpr uint32_t kPrHubMin = 16384;
constexpr int kPrBlock = 256;

struct InLightLen {
  const uint64_t *off;
  __device__ uint64_t operator()(uint64_t v) const {
    uint64_t len = off[v + 1] - off[v];
    return len <= kPrLightMax ? len : 0;
  }
};

// tile starts: v == 0, v heavy, v-1 heavy, or the light prefix crossed a
// multiple of kPrTile between v-1 and v
struct InTileStart {
  const uint64_t *off;
  const uint64_t *pre;
  __device__ uint64_t operator()(uint64_t v) const {
    if (v == 0) return 1;
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

__global__ void k_pr_heavy_lists(const uint64_t *__restrict__ off, uint64_t n, uint32_t *med,
                                 unsigned long long *nmed, uint32_t *hubs, unsigned long long *nhub) {
  // warp-uniform trip count: every lane reaches warp_append
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) & ~31ull; base < n; base += stride) {
    const uint64_t v = base + lane_id();
    uint64_t len = v < n ? off[v + 1] - off[v] : 0;
    bool m = len > kPrLightMax && len <= kPrHubMin, h = len > kPrHubMin;
    uint64_t sm = warp_append(m, nmed);
    if (m) med[sm] = (uint32_t)v;
    uint64_t sh = warp_append(h, nhub);
    if (h) hubs[sh] = (uint32_t)v;
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

// One CTA per light tile: stage p_div[u] of the tile's slots in shared memory
// (coalesced id loads, four independent gathers per thread in flight), then
// one thread per vertex sums its run left to right.
template <bool kComp, typename T>
__global__ void __launch_bounds__(kPrBlock) k_pr_tiles(const uint64_t *__restrict__ off,
                                                       const uint32_t *__restrict__ slots,
                                                       const uint32_t *__restrict__ deg,
                                                       const uint32_t *__restrict__ tstart, uint64_t ntiles,
                                                       const T *__restrict__ pdiv_in,
                                                       const T *__restrict__ p_curr, T *__restrict__ p_next,
                                                       T *__restrict__ pdiv_out, T damping, T added, double *l1) {
  __shared__ T vals[kPrTile + kPrLightMax];
  __shared__ double sm[kPrBlock / 32 + 1];
  double l1loc = 0.0;
  for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const uint32_t v0 = tstart[t], v1 = tstart[t + 1];
    const uint64_t s0 = off[v0], s1 = off[v1];
    if (v1 - v0 == 1 && s1 - s0 > kPrLightMax) continue;  // a heavy vertex: its own kernel
    const uint32_t len = (uint32_t)(s1 - s0);
    for (uint32_t i = threadIdx.x; i < len; i += 4 * kPrBlock) {
      uint32_t u[4];
#pragma unroll
      for (int k = 0; k < 4; k++) {
        uint32_t idx = i + k * kPrBlock;
        u[k] = idx < len ? __ldcs(slots + s0 + idx) : kSentinel;
      }
      T g[4];
#pragma unroll
      for (int k = 0; k < 4; k++) g[k] = u[k] != kSentinel ? pdiv_in[u[k]] : T(0);
#pragma unroll
      for (int k = 0; k < 4; k++) {
        uint32_t idx = i + k * kPrBlock;
        if (idx < len) vals[idx] = g[k];
      }
    }
    __syncthreads();
    for (uint32_t v = v0 + threadIdx.x; v < v1; v += kPrBlock) {
      const uint32_t r0 = (uint32_t)(off[v] - s0), r1 = (uint32_t)(off[v + 1] - s0);
      T s = T(0), c = T(0);
      for (uint32_t r = r0; r < r1; r++) acc_add<kComp>(s, c, vals[r]);
      pr_finish<kComp, T>(v, kComp ? s + c : s, deg, p_curr, p_next, pdiv_out, damping, added, l1loc);
    }
    __syncthreads();
  }
  l1loc = block_sum(l1loc, sm);
  if (threadIdx.x == 0 && l1loc != 0.0) atomicAdd(l1, l1loc);
}

// One warp per medium vertex; four independent loads per lane in flight.
template <bool kComp, typename T>
__global__ void __launch_bounds__(256) k_pr_medium(const uint64_t *__restrict__ off,
                                                   const uint32_t *__restrict__ slots,
                                                   const uint32_t *__restrict__ deg,
                                                   const uint32_t *__restrict__ med,
                                                   const unsigned long long *__restrict__ nmed,
                                                   const T *__restrict__ pdiv_in,
                                                   const T *__restrict__ p_curr, T *__restrict__ p_next,
                                                   T *__restrict__ pdiv_out, T damping, T added, double *l1) {
  __shared__ double sm[9];
  const uint64_t nm = *nmed;
  const unsigned lane = lane_id();
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  double l1loc = 0.0;
  for (uint64_t h = gw; h < nm; h += nw) {
    const uint32_t v = med[h];
    const uint64_t b = off[v], e = off[v + 1];
    T s = T(0), c = T(0);
    for (uint64_t j = b + lane; j < e; j += 128) {
      uint32_t u[4];
#pragma unroll
      for (int k = 0; k < 4; k++) u[k] = j + 32 * k < e ? __ldcs(slots + j + 32 * k) : kSentinel;
      T g[4];
#pragma unroll
      for (int k = 0; k < 4; k++) g[k] = u[k] != kSentinel ? pdiv_in[u[k]] : T(0);
#pragma unroll
      for (int k = 0; k < 4; k++) acc_add<kComp>(s, c, g[k]);
    }
    T tot = group_total<kComp, T, 32>(s, c);
    if (lane == 0) pr_finish<kComp, T>(v, tot, deg, p_curr, p_next, pdiv_out, damping, added, l1loc);
  }
  l1loc = block_sum(l1loc, sm);
  if (threadIdx.x == 0 && l1loc != 0.0) atomicAdd(l1, l1loc);
}

// One CTA per hub; warp partials combined in warp order.
template <bool kComp, typename T>
__global__ void __launch_bounds__(256) k_pr_hubs(const uint64_t *__restrict__ off,
                                                 const uint32_t *__restrict__ slots,
                                                 const uint32_t *__restrict__ deg,
                                                 const uint32_t *__restrict__ hubs,
                                                 const unsigned long long *__restrict__ nhub,
                                                 const T *__restrict__ pdiv_in,
                                                 const T *__restrict__ p_curr, T *__restrict__ p_next,
                                                 T *__restrict__ pdiv_out, T damping, T added, double *l1) {
  __shared__ T ss[8];
  const uint64_t nh = *nhub;
  for (uint64_t h = blockIdx.x; h < nh; h += gridDim.x) {
    const uint32_t v = hubs[h];
    const uint64_t b = off[v], e = off[v + 1];
    T s = T(0), c = T(0);
    for (uint64_t j = b + threadIdx.x; j < e; j += 4 * blockDim.x) {
      uint32_t u[4];
#pragma unroll
      for (int k = 0; k < 4; k++) u[k] = j + blockDim.x * k < e ? __ldcs(slots + j + blockDim.x * k) : kSentinel;
      T g[4];
#pragma unroll
      for (int k = 0; k < 4; k++) g[k] = u[k] != kSentinel ? pdiv_in[u[k]] : T(0);
#pragma unroll
      for (int k = 0; k < 4; k++) acc_add<kComp>(s, c, g[k]);
    }
    T tot = group_total<kComp, T, 32>(s, c);
    if (lane_id() == 0) ss[threadIdx.x >> 5] = tot;
    __syncthreads();
    if (threadIdx.x == 0) {
      T S = T(0), C = T(0);
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) acc_add<kComp>(S, C, ss[w]);
      double l1loc = 0.0;
      pr_finish<kComp, T>(v, kComp ? S + C : S, deg, p_curr, p_next, pdiv_out, damping, added, l1loc);
      atomicAdd(l1, l1loc);
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void k_pr_init(const uint32_t *__restrict__ deg, uint64_t n, T *p_curr, T *pdiv, T one_over_n) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    p_curr[v] = one_over_n;
    pdiv[v] = one_over_n / (T)deg[v];
  }
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
  BYO_TRY(ws(g, WS_PR_A, n, &pa));
  BYO_TRY(ws(g, WS_PR_B, n, &pb));
  BYO_TRY(ws(g, WS_PR_C, n, &da));
  BYO_TRY(ws(g, WS_PR_D, n, &db));
  // plan: light prefix, tile starts, medium and hub lists
  uint64_t *pre = nullptr;
  uint32_t *lists = nullptr;
  BYO_TRY(ws(g, WS_SCAN, n + 1, &pre));
  BYO_TRY(ws(g, WS_BUCKETS, 3 * n + 16, &lists));
  uint32_t *tstart = lists, *med = lists + (n + 2), *hubs = lists + 2 * (n + 2);
  unsigned long long *cnt = (unsigned long long *)(lists + 3 * n + 8 - ((3 * n + 8) & 1));
  double *d_l1 = nullptr;
  BYO_TRY(ws(g, WS_MISC, 4, (uint32_t **)&d_l1));
  const uint64_t *tot = nullptr;
  BYO_TRY(scan_apply(ctx, n, InLightLen{g->d_off}, OutPrefix{pre}, &tot));
  BYO_TRY(scan_apply(ctx, n, InTileStart{g->d_off, pre}, OutTileStart{tstart}, &tot));
  uint64_t *h = nullptr;
  BYO_TRY(pinned(ctx, 4096, (void **)&h));
  BYO_CU(ctx, cudaMemcpyAsync(h, tot, 8, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaMemsetAsync(cnt, 0, 16, ctx->stream));
  launch(ctx, k_pr_heavy_lists, dim3(grid_for(ctx, n + 31, 256)), dim3(256), 0, (const uint64_t *)g->d_off, n,
         med, cnt, hubs, cnt + 1);
  launch(ctx, k_pr_init<T>, dim3(grid_for(ctx, n, 256)), dim3(256), 0, (const uint32_t *)g->d_deg, n, pa, da,
         (T)(1.0 / (double)n));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  const uint64_t ntiles = h[0];
  uint32_t nn = (uint32_t)n;
  BYO_CU(ctx, cudaMemcpyAsync(tstart + ntiles, &nn, 4, cudaMemcpyHostToDevice, ctx->stream));
  const T damping = (T)0.85;
  const T added = (T)((1 - 0.85) * (1 / (double)n));
  const int grid_t = grid_for(ctx, ntiles, 1, 8);
  const int grid_m = ctx->num_sms * 8;
  const int grid_h = ctx->num_sms * 2;
  uint32_t it = 0;
  double L1 = 0.0;
  T *p_curr = pa, *p_next = pb, *pdiv = da, *pdiv_next = db, *last = nullptr;
  double *hl = (double *)h;
  while (it++ < max_iters) {
    BYO_CU(ctx, cudaMemsetAsync(d_l1, 0, 8, ctx->stream));
    launch_t(ctx, "pr_pull", k_pr_tiles<kComp, T>, dim3(grid_t), dim3(kPrBlock), 0, (const uint64_t *)g->d_off,
             (const uint32_t *)g->d_slots, (const uint32_t *)g->d_deg, (const uint32_t *)tstart, ntiles,
             (const T *)pdiv, (const T *)p_curr, p_next, pdiv_next, damping, added, d_l1);
    launch_t(ctx, "pr_pull", k_pr_medium<kComp, T>, dim3(grid_m), dim3(256), 0, (const uint64_t *)g->d_off,
             (const uint32_t *)g->d_slots, (const uint32_t *)g->d_deg, (const uint32_t *)med,
             (const unsigned long long *)cnt, (const T *)pdiv, (const T *)p_curr, p_next, pdiv_next, damping,
             added, d_l1);
    launch_t(ctx, "pr_pull", k_pr_hubs<kComp, T>, dim3(grid_h), dim3(256), 0, (const uint64_t *)g->d_off,
             (const uint32_t *)g->d_slots, (const uint32_t *)g->d_deg, (const uint32_t *)hubs,
             (const unsigned long long *)(cnt + 1), (const T *)pdiv, (const T *)p_curr, p_next, pdiv_next,
             damping, added, d_l1);
    BYO_CU(ctx, cudaMemcpyAsync(hl, d_l1, 8, cudaMemcpyDeviceToHost, ctx->stream));
    BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
    L1 = hl[0];
    std::swap(pdiv, pdiv_next);
    last = p_next;
    if (L1 < eps) break;
    std::swap(p_curr, p_next);
  }
  if (it > max_iters) it = max_iters;
  // the last computed iterate (the reference's final swap would hand back the
  // zeroed previous one when max_iters ends the loop, PageRank.h:181-192)
  launch(ctx, k_to_f64<T>, dim3(grid_for(ctx, n, 256)), dim3(256), 0, (const T *)(last ? last : p_curr), n,
         d_p);
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

// Lane groups per DAG vertex u; for each v in N+(u), the group counts
// |N+(u) cap N+(v)| by binary-searching the elements of the shorter list in
// the longer one.
template <int GS>
__global__ void __launch_bounds__(256) k_tc_intersect(const uint64_t *__restrict__ doff,
                                                      const uint32_t *__restrict__ dn, uint64_t n,
                                                      unsigned long long *total) {
  __shared__ unsigned long long sm[9];
  const unsigned gl = threadIdx.x % GS;
  const uint64_t gid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / GS;
  const uint64_t ng = ((uint64_t)gridDim.x * blockDim.x) / GS;
  unsigned long long cnt = 0;
  for (uint64_t u = gid; u < n; u += ng) {
    const uint64_t ab = doff[u], ae = doff[u + 1];
    for (uint64_t k = ab; k < ae; k++) {
      const uint32_t v = dn[k];
      const uint64_t bb = doff[v], be = doff[v + 1];
      // shorter list S is scanned, longer L searched
      uint64_t sb = ab, se = ae, lb = bb, le = be;
      if (be - bb < ae - ab) {
        sb = bb; se = be; lb = ab; le = ae;
      }
      for (uint64_t j = sb + gl; j < se; j += GS) {
        const uint32_t x = dn[j];
        uint64_t lo = lb, hi = le;
        while (lo < hi) {
          uint64_t mid = (lo + hi) >> 1;
          if (dn[mid] < x) lo = mid + 1; else hi = mid;
        }
        cnt += (lo < le && dn[lo] == x);
      }
    }
  }
  cnt = block_sum(cnt, sm);
  if (threadIdx.x == 0 && cnt) atomicAdd(total, cnt);
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
  BYO_CU(ctx, cudaMemsetAsync(d_total, 0, 8, ctx->stream));
  launch_t(ctx, "tc_intersect", k_tc_intersect<8>, dim3(grid_for(ctx, n * 8, 256, 16)), dim3(256), 0, (const uint64_t *)doff,
         (const uint32_t *)dn, n, d_total);
  BYO_CU(ctx, cudaMemcpyAsync(h, d_total, 8, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  *count = h[0];
  return check_launch(ctx, "triangle_count");
}

}  // namespace byo

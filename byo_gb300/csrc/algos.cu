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
    launch(ctx, k_cc_finish<16>, dim3(grid), dim3(256), 0, (const uint64_t *)g->d_off,
           (const uint32_t *)g->d_slots, p, n, giant);
  else if (GS == 8)
    launch(ctx, k_cc_finish<8>, dim3(grid), dim3(256), 0, (const uint64_t *)g->d_off,
           (const uint32_t *)g->d_slots, p, n, giant);
  else
    launch(ctx, k_cc_finish<4>, dim3(grid), dim3(256), 0, (const uint64_t *)g->d_off,
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

// p_next[v] = damping * sum + added; pdiv_out[v] = p_next[v] / deg[v];
// l1 += |p_curr[v] - p_next[v]| (FP64).  Vertices with degree >= hub_min are
// skipped here and handled by k_pr_hubs.
template <bool kComp, typename T, int GS>
__global__ void __launch_bounds__(256) k_pr_pull(const uint64_t *__restrict__ off,
                                                 const uint32_t *__restrict__ slots,
                                                 const uint32_t *__restrict__ deg,
                                                 const T *__restrict__ pdiv_in,
                                                 const T *__restrict__ p_curr, T *__restrict__ p_next,
                                                 T *__restrict__ pdiv_out, uint64_t n, T damping,
                                                 T added, uint32_t hub_min, double *l1) {
  __shared__ double sm[9];
  const unsigned gl = threadIdx.x % GS;
  const uint64_t gid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / GS;
  const uint64_t ng = ((uint64_t)gridDim.x * blockDim.x) / GS;
  double l1loc = 0.0;
  const uint64_t nround = (n + ng - 1) / ng;
  for (uint64_t r = 0; r < nround; r++) {
    const uint64_t v = gid + r * ng;
    T s = T(0), c = T(0);
    bool mine = v < n;
    uint32_t d = 0;
    if (mine) {
      d = deg[v];
      if (d >= hub_min) mine = false;
    }
    if (mine) {
      const uint64_t b = off[v], e = off[v + 1];
      for (uint64_t j = b + gl; j < e; j += GS) {
        uint32_t u = slots[j];
        if (u != kSentinel) acc_add<kComp>(s, c, pdiv_in[u]);
      }
    }
    T tot = group_total<kComp, T, GS>(s, c);
    if (mine && gl == 0) {
      T p = damping * tot + added;
      p_next[v] = p;
      pdiv_out[v] = p / (T)d;
      l1loc += fabs((double)p_curr[v] - (double)p);
    }
  }
  l1loc = block_sum(l1loc, sm);
  if (threadIdx.x == 0 && l1loc != 0.0) atomicAdd(l1, l1loc);
}

template <bool kComp, typename T>
__global__ void __launch_bounds__(256) k_pr_hubs(const uint64_t *__restrict__ off,
                                                 const uint32_t *__restrict__ slots,
                                                 const uint32_t *__restrict__ deg,
                                                 const uint32_t *__restrict__ hubs, uint64_t nh,
                                                 const T *__restrict__ pdiv_in,
                                                 const T *__restrict__ p_curr, T *__restrict__ p_next,
                                                 T *__restrict__ pdiv_out, T damping, T added,
                                                 double *l1) {
  __shared__ T ss[8], sc[8];
  for (uint64_t h = blockIdx.x; h < nh; h += gridDim.x) {
    const uint32_t v = hubs[h];
    const uint64_t b = off[v], e = off[v + 1];
    T s = T(0), c = T(0);
    for (uint64_t j = b + threadIdx.x; j < e; j += blockDim.x) {
      uint32_t u = slots[j];
      if (u != kSentinel) acc_add<kComp>(s, c, pdiv_in[u]);
    }
    T tot = group_total<kComp, T, 32>(s, c);
    // group_total leaves the warp total in every lane; combine warps in order
    if (lane_id() == 0) {
      ss[threadIdx.x >> 5] = tot;
      sc[threadIdx.x >> 5] = T(0);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      T S = T(0), C = T(0);
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) acc_add<kComp>(S, C, ss[w]);
      T t = kComp ? S + C : S;
      T p = damping * t + added;
      p_next[v] = p;
      pdiv_out[v] = p / (T)deg[v];
      atomicAdd(l1, fabs((double)p_curr[v] - (double)p));
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

__global__ void k_collect_hubs(const uint32_t *__restrict__ deg, uint64_t n, uint32_t hub_min,
                               uint32_t *hubs, unsigned long long *cnt) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    bool h = deg[v] >= hub_min;
    uint64_t s = warp_append(h, cnt);
    if (h) hubs[s] = (uint32_t)v;
  }
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
  // hub list: vertices of degree >= hub_min, one CTA each
  const uint32_t hub_min = 4096;
  uint32_t *hubs = nullptr;
  BYO_TRY(ws(g, WS_BUCKETS, n + 4, &hubs));
  // counter in the trailing 8-byte-aligned word
  unsigned long long *d_cnt = (unsigned long long *)(hubs + ((n + 1) & ~1ull));
  double *d_l1 = nullptr;
  BYO_TRY(ws(g, WS_MISC, 4, (uint32_t **)&d_l1));
  BYO_CU(ctx, cudaMemsetAsync(d_cnt, 0, 8, ctx->stream));
  launch(ctx, k_collect_hubs, dim3(grid_for(ctx, n, 256)), dim3(256), 0, (const uint32_t *)g->d_deg, n,
         hub_min, hubs, d_cnt);
  double *h = nullptr;
  BYO_TRY(pinned(ctx, 4096, (void **)&h));
  BYO_CU(ctx, cudaMemcpyAsync(h, d_cnt, 8, cudaMemcpyDeviceToHost, ctx->stream));
  launch(ctx, k_pr_init<T>, dim3(grid_for(ctx, n, 256)), dim3(256), 0, (const uint32_t *)g->d_deg, n, pa,
         da, (T)(1.0 / (double)n));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  const uint64_t nh = ((uint64_t *)h)[0];
  const T damping = (T)0.85;
  const T added = (T)((1 - 0.85) * (1 / (double)n));
  const double avg = (double)g->m / (double)n;
  const int GS = avg >= 24 ? 16 : avg >= 8 ? 8 : 4;
  const int grid = grid_for(ctx, n * GS, 256, 8);
  uint32_t it = 0;
  double L1 = 0.0;
  T *p_curr = pa, *p_next = pb, *pdiv = da, *pdiv_next = db, *last = nullptr;
  while (it++ < max_iters) {
    BYO_CU(ctx, cudaMemsetAsync(d_l1, 0, 8, ctx->stream));
#define PR_CASE(G)                                                                                   \
  launch(ctx, k_pr_pull<kComp, T, G>, dim3(grid), dim3(256), 0, (const uint64_t *)g->d_off,          \
         (const uint32_t *)g->d_slots, (const uint32_t *)g->d_deg, (const T *)pdiv, (const T *)p_curr, \
         p_next, pdiv_next, n, damping, added, hub_min, d_l1)
    if (GS == 16)
      PR_CASE(16);
    else if (GS == 8)
      PR_CASE(8);
    else
      PR_CASE(4);
#undef PR_CASE
    if (nh)
      launch(ctx, k_pr_hubs<kComp, T>, dim3((unsigned)std::min<uint64_t>(nh, ctx->num_sms * 4)), dim3(256),
             0, (const uint64_t *)g->d_off, (const uint32_t *)g->d_slots, (const uint32_t *)g->d_deg,
             (const uint32_t *)hubs, nh, (const T *)pdiv, (const T *)p_curr, p_next, pdiv_next, damping,
             added, d_l1);
    BYO_CU(ctx, cudaMemcpyAsync(h, d_l1, 8, cudaMemcpyDeviceToHost, ctx->stream));
    BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
    L1 = h[0];
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
  launch(ctx, k_tc_intersect<8>, dim3(grid_for(ctx, n * 8, 256, 16)), dim3(256), 0, (const uint64_t *)doff,
         (const uint32_t *)dn, n, d_total);
  BYO_CU(ctx, cudaMemcpyAsync(h, d_total, 8, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  *count = h[0];
  return check_launch(ctx, "triangle_count");
}

}  // namespace byo

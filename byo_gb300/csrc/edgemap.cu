// edgemap.cu -- edgeMap over the device functors other than BFS_F, and
// vertexMap / vertexFilter.
//
// The reference's edgeMap (gbbs/edge_map_data.h:254-315) takes any struct
// with update / updateAtomic / cond; a GPU kernel cannot call a host lambda,
// so the functors are a closed set of device structs, each mirroring one
// GBBS functor:
//   LabelF    BFS_ComponentLabel_F (benchmarks/Connectivity/BFSCC/Connectivity.h:31-50)
//   PrF       PR_F                 (benchmarks/PageRank/PageRank.h:33-50)
//   PrDeltaF  delta::PR_Delta_F    (benchmarks/PageRank/PageRank.h:200-226)
// BFS_F keeps the traversal engine of engine.cu.
//
// Rounds:
//   sparse (edgeMapSparse, gbbs/edge_map_blocked.h:18-92) and blocked: a warp
//     per frontier vertex walks its neighbour run with coalesced loads and
//     applies cond + updateAtomic; a vertex enters the output once (its bit is
//     claimed by atomicOr, the winner appends it by warp ballot).
//   dense (edgeMapDense, gbbs/edge_map_data.h:47-175): every vertex whose
//     cond holds scans its neighbours in order and applies update (one writer
//     per vertex) to those in the frontier, leaving at the first !cond.  A
//     lane takes a vertex of <= kDenseShort slots; longer runs go to a warp
//     that loads and tests 32 neighbours at a time and applies the updates in
//     order (for PR_F / PR_Delta_F: lanes gather the values, one lane adds them
//     left to right, so sums are bit-identical to a sequential scan).
//   dense forward (edgeMapDenseForward, gbbs/edge_map_data.h:180-247): the
//     frontier's members push with updateAtomic, as the sparse round does.
// The output is a list and a bitmap kept together (the engine's Frontier).
//
// Arithmetic that feeds parity with the FP64 oracle uses explicitly rounded
// operations (__dadd_rn, __dmul_rn, __ddiv_rn): no fused multiply-add, so
// every result equals the oracle's separately rounded C expression.
#include "device.cuh"
#include "engine.h"
#include "internal.h"

namespace byo {

namespace {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kDenseShort = 64;  // slots a lane scans alone in a dense round

struct LabelF {
  uint32_t *P;
  uint32_t src;
  __device__ bool cond(uint32_t d) const { return *(volatile uint32_t *)(P + d) == kNone; }
  __device__ bool update(uint32_t, uint32_t d) const {
    if (P[d] != src) {
      P[d] = src;
      return true;
    }
    return false;
  }
  __device__ bool updateAtomic(uint32_t, uint32_t d) const { return atomicCAS(P + d, kNone, src) == kNone; }
};

struct PrF {
  const double *pc;
  double *pn;
  const uint32_t *deg;
  __device__ double value(uint32_t s) const { return __ddiv_rn(pc[s], (double)deg[s]); }
  __device__ bool cond(uint32_t) const { return true; }
  __device__ bool update(uint32_t s, uint32_t d) const {
    pn[d] = __dadd_rn(pn[d], value(s));
    return true;
  }
  __device__ bool updateAtomic(uint32_t s, uint32_t d) const {
    atomicAdd(pn + d, value(s));
    return true;
  }
};

struct PrDeltaF {
  const double *delta;  // [2n]: delta, delta / degree
  double *ngh;
  __device__ double value(uint32_t s) const { return delta[2 * (uint64_t)s + 1]; }
  __device__ bool cond(uint32_t) const { return true; }
  __device__ bool update(uint32_t s, uint32_t d) const {
    const double old = ngh[d];
    ngh[d] = __dadd_rn(old, value(s));
    return old == 0.0;
  }
  __device__ bool updateAtomic(uint32_t s, uint32_t d) const {
    unsigned long long *a = reinterpret_cast<unsigned long long *>(ngh + d);
    const double x = value(s);
    unsigned long long old = *(volatile unsigned long long *)a, seen;
    do {
      seen = old;
      old = atomicCAS(a, seen, __double_as_longlong(__dadd_rn(__longlong_as_double(seen), x)));
    } while (old != seen);
    return __longlong_as_double(seen) == 0.0;
  }
};

// Output of a round: the bit of v claimed once, the winner appends v.
__device__ __forceinline__ void emit_out(bool want, uint32_t v, uint32_t *out_list, uint32_t *out_bits,
                                         const uint32_t *deg, unsigned long long *cnt, uint64_t &outdeg) {
  bool emit = false;
  if (want) {
    const uint32_t bit = 1u << (v & 31);
    emit = !(atomicOr(out_bits + (v >> 5), bit) & bit);
  }
  const uint64_t slot = warp_append(emit, cnt);
  if (emit) {
    out_list[slot] = v;
    outdeg += deg[v];
  }
}

template <class F>
__global__ void __launch_bounds__(256) k_em_push(const uint64_t *__restrict__ off, const uint32_t *__restrict__ slots,
                                                 const uint32_t *__restrict__ deg, F f,
                                                 const uint32_t *__restrict__ list, uint64_t size, int output,
                                                 uint32_t *out_list, uint32_t *out_bits, unsigned long long *cnt) {
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  uint64_t outdeg = 0;
  for (uint64_t i = gw; i < size; i += nw) {
    const uint32_t u = list[i];
    const uint64_t b = off[u], e = off[u + 1];
    for (uint64_t base = b; base < e; base += 32) {
      const uint64_t j = base + lane_id();
      bool hit = false;
      uint32_t v = 0;
      if (j < e) {
        v = slots[j];
        if (v != kSentinel && f.cond(v)) hit = f.updateAtomic(u, v);
      }
      emit_out(hit && output, v, out_list, out_bits, deg, cnt, outdeg);
    }
  }
  outdeg = warp_sum(outdeg);
  if (lane_id() == 0 && outdeg) atomicAdd(cnt + 1, (unsigned long long)outdeg);
}

template <class F>
__global__ void __launch_bounds__(256) k_em_pull(const uint64_t *__restrict__ off, const uint32_t *__restrict__ slots,
                                                 const uint32_t *__restrict__ deg, F f, const uint32_t *__restrict__ fb,
                                                 uint64_t n, int output, uint32_t *out_list, uint32_t *out_bits,
                                                 unsigned long long *cnt, uint32_t *defer) {
  const uint64_t W = (n + 31) / 32;
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  uint64_t outdeg = 0;
  for (uint64_t w = gw; w < W; w += nw) {
    const uint64_t v = w * 32 + lane_id();
    bool marked = false, lng = false;
    if (v < n) {
      const uint64_t b = off[v], e = off[v + 1];
      if (e - b > kDenseShort) {
        lng = true;
      } else if (f.cond((uint32_t)v)) {
        for (uint64_t j = b; j < e; j++) {
          const uint32_t u = slots[j];
          if (u == kSentinel) continue;
          if (test_bit(fb, u) && f.update(u, (uint32_t)v)) marked = true;
          if (!f.cond((uint32_t)v)) break;
        }
      }
    }
    const uint64_t slot = warp_append(lng, cnt + 2);
    if (lng) defer[slot] = (uint32_t)v;
    marked = marked && output;
    const unsigned m = __ballot_sync(kFull, marked);
    if (lane_id() == 0 && m) atomicOr(out_bits + w, m);
    const uint64_t s2 = warp_append(marked, cnt);
    if (marked) {
      out_list[s2] = (uint32_t)v;
      outdeg += deg[v];
    }
  }
  outdeg = warp_sum(outdeg);
  if (lane_id() == 0 && outdeg) atomicAdd(cnt + 1, (unsigned long long)outdeg);
}

// A long run in order, a warp at a time: returns whether any update marked v
// (warp-uniform).  Generic form: lane 0 applies the updates one by one.
template <class F>
__device__ __forceinline__ bool warp_pull_run(const F &f, uint32_t v, const uint32_t *slots, uint64_t b, uint64_t e,
                                              const uint32_t *fb) {
  bool marked = false;
  for (uint64_t base = b; base < e; base += 32) {
    const uint64_t j = base + lane_id();
    const uint32_t u = j < e ? slots[j] : kSentinel;
    unsigned in = __ballot_sync(kFull, u != kSentinel && test_bit(fb, u));
    bool stop = false;
    while (in && !stop) {
      const int k = __ffs(in) - 1;
      in &= in - 1;
      const uint32_t uk = __shfl_sync(kFull, u, k);
      int r = 0, c = 1;
      if (lane_id() == 0) {
        r = f.update(uk, v) ? 1 : 0;
        c = f.cond(v) ? 1 : 0;
      }
      r = __shfl_sync(kFull, r, 0);
      c = __shfl_sync(kFull, c, 0);
      marked |= r != 0;
      stop = !c;
    }
    if (stop) break;
  }
  return marked;
}

// Sums (PR_F, PR_Delta_F): lanes gather 32 values, lane 0 adds them in order.
template <class F>
__device__ __forceinline__ bool warp_pull_sum(double *acc_at, bool zero_marks, const F &f, const uint32_t *slots,
                                              uint64_t b, uint64_t e, const uint32_t *fb) {
  double acc = 0.0;
  bool marked = false;
  if (lane_id() == 0) acc = *acc_at;
  for (uint64_t base = b; base < e; base += 32) {
    const uint64_t j = base + lane_id();
    const uint32_t u = j < e ? slots[j] : kSentinel;
    const bool in = u != kSentinel && test_bit(fb, u);
    const double x = in ? f.value(u) : 0.0;
    unsigned m = __ballot_sync(kFull, in);
    while (m) {
      const int k = __ffs(m) - 1;
      m &= m - 1;
      const double xk = __shfl_sync(kFull, x, k);
      if (lane_id() == 0) {
        marked |= zero_marks ? acc == 0.0 : true;
        acc = __dadd_rn(acc, xk);
      }
    }
  }
  if (lane_id() == 0) *acc_at = acc;
  return __shfl_sync(kFull, marked ? 1 : 0, 0) != 0;
}

__device__ __forceinline__ bool warp_pull(const LabelF &f, uint32_t v, const uint32_t *slots, uint64_t b, uint64_t e,
                                          const uint32_t *fb) {
  return warp_pull_run(f, v, slots, b, e, fb);
}
__device__ __forceinline__ bool warp_pull(const PrF &f, uint32_t v, const uint32_t *slots, uint64_t b, uint64_t e,
                                          const uint32_t *fb) {
  return warp_pull_sum(f.pn + v, false, f, slots, b, e, fb);
}
__device__ __forceinline__ bool warp_pull(const PrDeltaF &f, uint32_t v, const uint32_t *slots, uint64_t b,
                                          uint64_t e, const uint32_t *fb) {
  return warp_pull_sum(f.ngh + v, true, f, slots, b, e, fb);
}

template <class F>
__global__ void __launch_bounds__(256) k_em_pull_long(const uint64_t *__restrict__ off,
                                                      const uint32_t *__restrict__ slots,
                                                      const uint32_t *__restrict__ deg, F f,
                                                      const uint32_t *__restrict__ fb, int output,
                                                      uint32_t *out_list, uint32_t *out_bits, unsigned long long *cnt,
                                                      const uint32_t *__restrict__ defer) {
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t nd = cnt[2];
  uint64_t outdeg = 0;
  for (uint64_t i = gw; i < nd; i += nw) {
    const uint32_t v = defer[i];
    bool marked = false;
    if (__shfl_sync(kFull, f.cond(v) ? 1 : 0, 0)) marked = warp_pull(f, v, slots, off[v], off[v + 1], fb);
    const bool want = lane_id() == 0 && marked && output;
    emit_out(want, v, out_list, out_bits, deg, cnt, outdeg);
  }
  outdeg = warp_sum(outdeg);
  if (lane_id() == 0 && outdeg) atomicAdd(cnt + 1, (unsigned long long)outdeg);
}

// ---------------------------------------------------------------- frontier forms

__global__ void k_bits_to_list(const uint32_t *__restrict__ bits, uint64_t n, const uint32_t *__restrict__ deg,
                               uint32_t *list, unsigned long long *cnt) {
  const uint64_t W = (n + 31) / 32;
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  uint64_t outdeg = 0;
  for (uint64_t w = gw; w < W; w += nw) {
    const uint64_t v = w * 32 + lane_id();
    const bool in = v < n && ((bits[w] >> lane_id()) & 1u);
    const uint64_t slot = warp_append(in, cnt);
    if (in) {
      list[slot] = (uint32_t)v;
      outdeg += deg[v];
    }
  }
  outdeg = warp_sum(outdeg);
  if (lane_id() == 0 && outdeg) atomicAdd(cnt + 1, (unsigned long long)outdeg);
}

// bits[w] = src[w] (or all ones) with the bits of ids >= n cleared
__global__ void k_bits_copy(const uint32_t *__restrict__ src, uint64_t n, uint32_t *bits) {
  const uint64_t W = (n + 31) / 32;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < W; w += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t x = src ? src[w] : 0xFFFFFFFFu;
    if (w == W - 1 && (n & 31)) x &= (1u << (n & 31)) - 1u;
    bits[w] = x;
  }
}

// ---------------------------------------------------------------- vertex functions

struct VOp {
  int kind;
  double *a, *b, *c;
  double damping, eps2, added, one_over_n;
  const uint32_t *deg;
};

// PR_Vertex_F (PageRank.h:53-68), PR_Vertex_Reset (:71-78),
// delta::PR_Vertex_F_FirstRound (:252-281), delta::PR_Vertex_F (:294-318)
__device__ __forceinline__ bool vop_apply(const VOp &o, uint32_t i) {
  switch (o.kind) {
    case BYO_VOP_PR_UPDATE:
      o.a[i] = __dadd_rn(__dmul_rn(o.damping, o.a[i]), o.added);
      return true;
    case BYO_VOP_ZERO:
      o.a[i] = 0.0;
      return true;
    case BYO_VOP_PR_DELTA_FIRST: {
      const double pre = __dadd_rn(__dmul_rn(o.damping, o.c[i]), o.added);
      const double p = __dadd_rn(o.a[i], pre);
      o.a[i] = p;
      const double nd = __dsub_rn(pre, o.one_over_n);
      o.b[2 * (uint64_t)i] = nd;
      o.b[2 * (uint64_t)i + 1] = __ddiv_rn(nd, (double)o.deg[i]);
      return nd > __dmul_rn(o.eps2, p);
    }
    case BYO_VOP_PR_DELTA: {
      const double nd = __dmul_rn(o.c[i], o.damping);
      o.b[2 * (uint64_t)i] = nd;
      o.b[2 * (uint64_t)i + 1] = __ddiv_rn(nd, (double)o.deg[i]);
      if (fabs(nd) > __dmul_rn(o.eps2, o.a[i])) {
        o.a[i] = __dadd_rn(o.a[i], nd);
        return true;
      }
      return false;
    }
    default:
      return false;
  }
}

__global__ void __launch_bounds__(256) k_vertex_op(VOp o, const uint32_t *__restrict__ list, uint64_t size,
                                                   int filter, uint32_t *out_list, uint32_t *out_bits,
                                                   unsigned long long *cnt) {
  uint64_t outdeg = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x; i0 < size; i0 += stride) {
    const uint64_t i = i0 + threadIdx.x;
    bool keep = false;
    uint32_t v = 0;
    if (i < size) {
      v = list[i];
      keep = vop_apply(o, v);
    }
    if (filter) {
      keep = keep && i < size;
      if (keep) atomicOr(out_bits + (v >> 5), 1u << (v & 31));
      const uint64_t slot = warp_append(keep, cnt);
      if (keep) {
        out_list[slot] = v;
        outdeg += o.deg[v];
      }
    }
  }
  if (filter) {
    outdeg = warp_sum(outdeg);
    if (lane_id() == 0 && outdeg) atomicAdd(cnt + 1, (unsigned long long)outdeg);
  }
}

// Sum of |a[i] - b[i]| in 4096-vertex chunks (each summed in order), then
// the chunks in order: the oracle's reduction order, so the value is the
// oracle's to the last bit on the same inputs.
constexpr uint64_t kL1Chunk = 4096;
__global__ void k_l1_chunks(const double *__restrict__ a, const double *__restrict__ b, uint64_t n, double *part) {
  const uint64_t nch = (n + kL1Chunk - 1) / kL1Chunk;
  for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < nch; c += (uint64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    const uint64_t hi = (c + 1) * kL1Chunk < n ? (c + 1) * kL1Chunk : n;
    for (uint64_t i = c * kL1Chunk; i < hi; i++) acc = __dadd_rn(acc, fabs(__dsub_rn(a[i], b[i])));
    part[c] = acc;
  }
}
__global__ void k_l1_total(const double *__restrict__ part, uint64_t nch, double *out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double s = 0.0;
  for (uint64_t c = 0; c < nch; c++) s = __dadd_rn(s, part[c]);
  *out = s;
}

__global__ void k_fill_f64(double *a, uint64_t n, double x) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    a[i] = x;
}

template <class F>
int run_round(byo_graph *g, const F &f, Frontier &in, Frontier &out, int mode, bool output,
              unsigned long long *cnt) {
  byo_ctx *ctx = g->ctx;
  const int block = 256;
  if (mode == MODE_PULL) {
    BYO_TRY(ensure_bits(g, in));
    uint32_t *defer = nullptr;
    BYO_TRY(ws(g, WS_DEFER, g->n + 1, &defer));
    const uint64_t W = (g->n + 31) / 32;
    launch(ctx, k_em_pull<F>, dim3(grid_for(ctx, W * 32, block)), dim3(block), 0, (const uint64_t *)g->d_off,
           (const uint32_t *)g->d_slots, (const uint32_t *)g->d_deg, f, (const uint32_t *)in.bits, g->n,
           output ? 1 : 0, out.list, out.bits, cnt, defer);
    launch(ctx, k_em_pull_long<F>, dim3(grid_for(ctx, W * 32, block)), dim3(block), 0, (const uint64_t *)g->d_off,
           (const uint32_t *)g->d_slots, (const uint32_t *)g->d_deg, f, (const uint32_t *)in.bits, output ? 1 : 0,
           out.list, out.bits, cnt, (const uint32_t *)defer);
  } else {  // sparse, blocked and dense forward: updateAtomic from the members
    BYO_TRY(ensure_list(g, in));
    if (in.size)
      launch(ctx, k_em_push<F>, dim3(grid_for(ctx, in.size * 32, block)), dim3(block), 0,
             (const uint64_t *)g->d_off, (const uint32_t *)g->d_slots, (const uint32_t *)g->d_deg, f,
             (const uint32_t *)in.list, in.size, output ? 1 : 0, out.list, out.bits, cnt);
  }
  return check_launch(ctx, "edge_map");
}

}  // namespace

int ensure_list(byo_graph *g, Frontier &f) {
  if (f.has_list) return BYO_OK;
  byo_ctx *ctx = g->ctx;
  unsigned long long *cnt = nullptr;
  BYO_TRY(ws(g, WS_STATS, 4, (uint64_t **)&cnt));
  BYO_CU(ctx, cudaMemsetAsync(cnt, 0, 16, ctx->stream));
  const uint64_t W = (g->n + 31) / 32;
  launch(ctx, k_bits_to_list, dim3(grid_for(ctx, W * 32, 256)), dim3(256), 0, (const uint32_t *)f.bits, g->n,
         (const uint32_t *)g->d_deg, f.list, cnt);
  unsigned long long h[2] = {0, 0};
  BYO_CU(ctx, cudaMemcpyAsync(h, cnt, 16, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  f.size = h[0];
  f.outdeg = h[1];
  f.has_list = true;
  return check_launch(ctx, "frontier list");
}

int frontier_from_bits(byo_graph *g, const uint32_t *d_bits, Frontier &f) {
  byo_ctx *ctx = g->ctx;
  const uint64_t W = (g->n + 31) / 32;
  launch(ctx, k_bits_copy, dim3(grid_for(ctx, W, 256)), dim3(256), 0, d_bits, g->n, f.bits);
  f.has_bits = true;
  f.has_list = false;
  f.dense = true;
  BYO_TRY(ensure_list(g, f));
  return BYO_OK;
}

int generic_edge_map(byo_graph *g, const FunctorArgs &fa, Frontier &in, Frontier &out, int mode, bool output) {
  byo_ctx *ctx = g->ctx;
  unsigned long long *cnt = nullptr;
  BYO_TRY(ws(g, WS_STATS, 4, (uint64_t **)&cnt));
  BYO_CU(ctx, cudaMemsetAsync(cnt, 0, 32, ctx->stream));
  switch (fa.kind) {
    case BYO_F_BFS_LABEL: BYO_TRY(run_round(g, LabelF{fa.parents, fa.src}, in, out, mode, output, cnt)); break;
    case BYO_F_PR: BYO_TRY(run_round(g, PrF{fa.p_curr, fa.p_next, g->d_deg}, in, out, mode, output, cnt)); break;
    case BYO_F_PR_DELTA: BYO_TRY(run_round(g, PrDeltaF{fa.delta, fa.ngh}, in, out, mode, output, cnt)); break;
    default: return set_error(ctx, BYO_EINVAL, "edge_map: unknown functor kind");
  }
  unsigned long long h[2] = {0, 0};
  BYO_CU(ctx, cudaMemcpyAsync(h, cnt, 16, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  out.size = output ? h[0] : 0;
  out.outdeg = output ? h[1] : 0;
  out.has_list = out.has_bits = true;
  out.dense = mode == MODE_PULL || mode == MODE_DENSE_FWD;
  return BYO_OK;
}

int vertex_op_run(byo_graph *g, const VertexOpArgs &op, Frontier &in, Frontier *out) {
  byo_ctx *ctx = g->ctx;
  BYO_TRY(ensure_list(g, in));
  VOp o;
  o.kind = op.kind;
  o.a = op.a;
  o.b = op.b;
  o.c = op.c;
  o.damping = op.damping;
  o.eps2 = op.eps2;
  o.one_over_n = 1.0 / (double)g->n;
  o.added = (1.0 - op.damping) * o.one_over_n;
  o.deg = g->d_deg;
  unsigned long long *cnt = nullptr;
  BYO_TRY(ws(g, WS_STATS, 4, (uint64_t **)&cnt));
  BYO_CU(ctx, cudaMemsetAsync(cnt, 0, 16, ctx->stream));
  if (in.size)
    launch(ctx, k_vertex_op, dim3(grid_for(ctx, in.size, 256)), dim3(256), 0, o, (const uint32_t *)in.list,
           in.size, out ? 1 : 0, out ? out->list : nullptr, out ? out->bits : nullptr, cnt);
  BYO_TRY(check_launch(ctx, "vertex_map"));
  if (out) {
    unsigned long long h[2] = {0, 0};
    BYO_CU(ctx, cudaMemcpyAsync(h, cnt, 16, cudaMemcpyDeviceToHost, ctx->stream));
    BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
    out->size = h[0];
    out->outdeg = h[1];
    out->has_list = out->has_bits = true;
    out->dense = false;
  }
  return BYO_OK;
}

int l1_diff(byo_graph *g, const double *a, const double *b, double *d_part, double *h_out) {
  byo_ctx *ctx = g->ctx;
  const uint64_t nch = (g->n + kL1Chunk - 1) / kL1Chunk;
  launch(ctx, k_l1_chunks, dim3(grid_for(ctx, nch, 128)), dim3(128), 0, a, b, g->n, d_part);
  launch(ctx, k_l1_total, dim3(1), dim3(32), 0, (const double *)d_part, nch, d_part + nch);
  BYO_CU(ctx, cudaMemcpyAsync(h_out, d_part + nch, 8, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  return check_launch(ctx, "l1");
}

// PageRank_edgeMap (benchmarks/PageRank/PageRank.h:80-123) through the
// generic edgeMap: p_curr = 1/n, frontier = every vertex; each iteration
// edgeMap(PR_F, threshold 0, no_output) (always dense), vertexMap(PR_Vertex_F),
// L1 between the iterates, stop below eps; reset p_curr and swap.  Returns
// the last computed iterate (the reference's final swap would hand back the
// zeroed one when max_iters ends the loop).
int pagerank_edgemap_run(byo_graph *g, double eps, uint32_t max_iters, double *d_p, uint32_t *iters_out,
                         double *l1_out) {
  byo_ctx *ctx = g->ctx;
  const uint64_t n = g->n;
  const uint64_t W = (n + 31) / 32;
  const uint64_t nch = (n + kL1Chunk - 1) / kL1Chunk;
  double *pa = nullptr, *pb = nullptr, *part = nullptr;
  BYO_TRY(ws(g, WS_PR_A, n + 1, &pa));
  BYO_TRY(ws(g, WS_PR_B, n + 1, &pb));
  BYO_TRY(ws(g, WS_PR_C, nch + 2, &part));
  uint32_t *flist = nullptr, *fbits = nullptr;
  BYO_TRY(ws(g, WS_FRONT_LIST_A, n + 1, &flist));
  BYO_TRY(ws(g, WS_FRONT_BITS_A, W + 1, &fbits));
  Frontier all;
  all.list = flist;
  all.bits = fbits;
  BYO_TRY(frontier_from_bits(g, nullptr, all));
  Frontier none;  // no_output rounds write nothing
  launch(ctx, k_fill_f64, dim3(grid_for(ctx, n, 256)), dim3(256), 0, pa, n, 1.0 / (double)n);
  BYO_CU(ctx, cudaMemsetAsync(pb, 0, n * 8, ctx->stream));
  double *pc = pa, *pn = pb;
  uint32_t it = 0;
  double L1 = 0.0;
  while (it++ < max_iters) {
    FunctorArgs f{};
    f.kind = BYO_F_PR;
    f.p_curr = pc;
    f.p_next = pn;
    BYO_TRY(generic_edge_map(g, f, all, none, MODE_PULL, false));
    VertexOpArgs vf{BYO_VOP_PR_UPDATE, pn, nullptr, nullptr, 0.85, 0.0};
    BYO_TRY(vertex_op_run(g, vf, all, nullptr));
    BYO_TRY(l1_diff(g, pc, pn, part, &L1));
    if (L1 < eps) break;
    VertexOpArgs rz{BYO_VOP_ZERO, pc, nullptr, nullptr, 0.0, 0.0};
    BYO_TRY(vertex_op_run(g, rz, all, nullptr));
    std::swap(pc, pn);
  }
  if (it > max_iters) {
    it = max_iters;
    std::swap(pc, pn);  // the last computed iterate, not the zeroed one
  }
  BYO_CU(ctx, cudaMemcpyAsync(d_p, pn, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
  if (iters_out) *iters_out = it;
  if (l1_out) *l1_out = L1;
  return check_launch(ctx, "pagerank_edgemap");
}

}  // namespace byo

// prdelta.cu -- PageRankDelta (benchmarks/PageRank/PageRank.h:340-398).
//
// Per round: nghSum[v] = sum of delta[u] / deg(u) over v's neighbours u in
// the frontier, then a filter over every vertex updates p, delta and the next
// frontier (PR_Vertex_F_FirstRound :271-290 in the first round, PR_Vertex_F
// :307-323 after).  sparse_or_dense (:231-269) decides how nghSum is formed;
// both branches compute the same sum and differ only in the order of the
// additions, so here the choice is a speed choice:
//   pull  the frontier as a bitmap; a thread sums a vertex of up to kPrdLight
//         slots left to right (the order of the restatement in the oracle), a
//         warp sums a heavier one.
//   push  the frontier as a list; a warp per frontier vertex adds its
//         delta / deg into each neighbour's nghSum with FP64 atomics (the
//         reference's PR_Delta_F::updateAtomic CAS loop).
// The filter's arithmetic uses explicitly rounded operations so that no
// multiply-add is contracted.  The L1 norm of the deltas is reduced per block
// and the block partials are added in block order.
#include <algorithm>

#include "device.cuh"
#include "internal.h"

namespace byo {

constexpr int kPrdBlock = 256;
constexpr uint32_t kPrdLight = 32;

struct PrdStats {
  unsigned long long count;   // |next frontier|
  unsigned long long outdeg;  // degree sum of the next frontier
  unsigned long long nheavy;  // vertices above kPrdLight slots (built once)
  double l1;
};

__global__ void k_prd_init(const uint64_t *__restrict__ off, const uint32_t *__restrict__ deg, uint64_t n, double *p,
                           double *delta, double *dod, double *ngh, uint32_t *fbits, uint32_t *heavy, PrdStats *st) {
  const double one_over_n = 1.0 / (double)n;
  for (uint64_t base = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) & ~31ull; base < n;
       base += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = base + lane_id();
    bool hv = false;
    if (i < n) {
      p[i] = 0.0;
      delta[i] = one_over_n;
      dod[i] = __ddiv_rn(one_over_n, (double)deg[i]);  // inf for degree 0, never read
      ngh[i] = 0.0;
      hv = off[i + 1] - off[i] > kPrdLight;
    }
    const unsigned all = __ballot_sync(kFull, i < n);
    if (lane_id() == 0) fbits[i >> 5] = all;
    const uint64_t at = warp_append(hv, &st->nheavy);
    if (hv) heavy[at] = (uint32_t)i;
  }
}

// nghSum of every light vertex, left to right over its slots
__global__ void __launch_bounds__(kPrdBlock) k_prd_pull_light(const uint64_t *__restrict__ off,
                                                              const uint32_t *__restrict__ slots, uint64_t n,
                                                              const uint32_t *__restrict__ fbits,
                                                              const double *__restrict__ dod, double *ngh) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = off[v], e = off[v + 1];
    if (e - b > kPrdLight) continue;
    double s = 0.0;
    for (uint64_t j = b; j < e; j++) {
      const uint32_t u = slots[j];
      if (u != kSentinel && test_bit(fbits, u)) s = __dadd_rn(s, dod[u]);
    }
    ngh[v] = s;
  }
}

// nghSum of every heavy vertex, a warp each
__global__ void __launch_bounds__(kPrdBlock) k_prd_pull_heavy(const uint64_t *__restrict__ off,
                                                              const uint32_t *__restrict__ slots,
                                                              const uint32_t *__restrict__ heavy,
                                                              const PrdStats *__restrict__ st,
                                                              const uint32_t *__restrict__ fbits,
                                                              const double *__restrict__ dod, double *ngh) {
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t nh = st->nheavy;
  for (uint64_t h = gw; h < nh; h += nw) {
    const uint32_t v = heavy[h];
    double s = 0.0;
    for (uint64_t j = off[v] + lane_id(); j < off[v + 1]; j += 32) {
      const uint32_t u = slots[j];
      if (u != kSentinel && test_bit(fbits, u)) s = __dadd_rn(s, dod[u]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = __dadd_rn(s, __shfl_xor_sync(kFull, s, o));
    if (lane_id() == 0) ngh[v] = s;
  }
}

// nghSum by push from a frontier list, a warp per frontier vertex
__global__ void __launch_bounds__(kPrdBlock) k_prd_push(const uint64_t *__restrict__ off,
                                                        const uint32_t *__restrict__ slots,
                                                        const uint32_t *__restrict__ flist, uint64_t fsize,
                                                        const double *__restrict__ dod, double *ngh) {
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t i = gw; i < fsize; i += nw) {
    const uint32_t u = flist[i];
    const double x = dod[u];
    for (uint64_t j = off[u] + lane_id(); j < off[u + 1]; j += 32) {
      const uint32_t v = slots[j];
      if (v != kSentinel) atomicAdd(ngh + v, x);
    }
  }
}

// vertexFilter over all vertices; writes the next frontier (bits and list),
// its size and degree sum, and this block's sum of |delta| to part[block].
template <bool kFirst>
__global__ void __launch_bounds__(kPrdBlock) k_prd_filter(const uint32_t *__restrict__ deg, uint64_t n, double *p,
                                                          double *delta, double *dod, double *ngh,
                                                          uint32_t *nbits, uint32_t *nlist, PrdStats *st,
                                                          double *part, double local_eps) {
  __shared__ double sm[kPrdBlock / 32 + 1];
  const double damping = 0.85, one_over_n = 1.0 / (double)n;
  const double added = __dmul_rn(1.0 - damping, one_over_n);
  double l1 = 0.0;
  unsigned long long dsum = 0;
  for (uint64_t base = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) & ~31ull; base < n;
       base += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = base + lane_id();
    bool act = false;
    if (i < n) {
      const uint32_t d = deg[i];
      const double s = ngh[i];
      double nd;
      if (kFirst) {
        const double pre = __dadd_rn(__dmul_rn(damping, s), added);
        const double pi = __dadd_rn(p[i], pre);
        p[i] = pi;
        nd = __dsub_rn(pre, one_over_n);
        act = nd > __dmul_rn(local_eps, pi);
      } else {
        nd = __dmul_rn(s, damping);
        const double pi = p[i];
        if (fabs(nd) > __dmul_rn(local_eps, pi)) {
          p[i] = __dadd_rn(pi, nd);
          act = true;
        }
      }
      delta[i] = nd;
      dod[i] = __ddiv_rn(nd, (double)d);
      ngh[i] = 0.0;
      l1 = __dadd_rn(l1, fabs(nd));
      if (act) dsum += d;
    }
    const unsigned m = __ballot_sync(kFull, act);
    if (lane_id() == 0 && base / 32 < (n + 31) / 32) nbits[base >> 5] = m;
    const uint64_t at = warp_append(act, &st->count);
    if (act) nlist[at] = (uint32_t)i;
  }
  dsum = warp_sum(dsum);
  if (lane_id() == 0 && dsum) atomicAdd(&st->outdeg, dsum);
  // this block's |delta| sum, a fixed tree
  const unsigned w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) l1 = __dadd_rn(l1, __shfl_xor_sync(kFull, l1, o));
  if (lane_id() == 0) sm[w] = l1;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < kPrdBlock / 32; k++) t = __dadd_rn(t, sm[k]);
    part[blockIdx.x] = t;
  }
}

// One block of 256 threads: strided partial sums, then a fixed tree.
__global__ void __launch_bounds__(256) k_prd_l1(const double *__restrict__ part, uint32_t nparts, PrdStats *st) {
  __shared__ double sm[256];
  double t = 0.0;
  for (uint32_t k = threadIdx.x; k < nparts; k += 256) t = __dadd_rn(t, part[k]);
  sm[threadIdx.x] = t;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sm[threadIdx.x] = __dadd_rn(sm[threadIdx.x], sm[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) st->l1 = sm[0];
}

int pagerank_delta_run(byo_graph *g, double eps, double local_eps, uint32_t max_iters, double *d_p,
                       uint32_t *rounds_out, double *l1_out) {
  byo_ctx *ctx = g->ctx;
  const uint64_t n = g->n;
  if (rounds_out) *rounds_out = 0;
  if (l1_out) *l1_out = 0;
  if (n == 0) return BYO_OK;
  const uint64_t W = (n + 31) / 32;
  double *delta, *dod, *ngh, *part;
  uint32_t *fa, *fb, *la, *lb, *heavy;
  PrdStats *st;
  BYO_TRY(ws(g, WS_PR_A, 3 * n + 1, &delta));
  dod = delta + n;
  ngh = dod + n;
  BYO_TRY(ws(g, WS_FRONT_BITS_A, W + 1, &fa));
  BYO_TRY(ws(g, WS_FRONT_BITS_B, W + 1, &fb));
  BYO_TRY(ws(g, WS_FRONT_LIST_A, n + 1, &la));
  BYO_TRY(ws(g, WS_FRONT_LIST_B, n + 1, &lb));
  BYO_TRY(ws(g, WS_DEFER, n + 1, &heavy));
  const int fgrid = grid_for(ctx, n, kPrdBlock, 8);
  BYO_TRY(ws(g, WS_PR_B, (uint64_t)fgrid + 1, &part));
  BYO_TRY(ws(g, WS_STATS, sizeof(PrdStats) / 8 + 1, (uint64_t **)&st));
  BYO_CU(ctx, cudaMemsetAsync(st, 0, sizeof(PrdStats), ctx->stream));
  launch(ctx, k_prd_init, dim3(grid_for(ctx, n, 256, 8)), dim3(256), 0, (const uint64_t *)g->d_off,
         (const uint32_t *)g->d_deg, n, d_p, delta, dod, ngh, fa, heavy, st);
  PrdStats *h = nullptr;
  BYO_TRY(pinned(ctx, sizeof(PrdStats), (void **)&h));
  uint64_t fsize = n, fdeg = g->m;
  bool have_list = false;  // the first frontier (all vertices) has only its bitmap
  uint32_t round = 0;
  double L1 = 0;
  while (round++ < max_iters) {
    // sparse_or_dense (PageRank.h:231-269) with edgeMap's threshold M/2
    const bool dense = !have_list || fsize > n / 5 || fsize + fdeg > g->m / 2;
    if (dense) {
      launch_t(ctx, "pr_delta", k_prd_pull_light, dim3(grid_for(ctx, n, kPrdBlock, 8)), dim3(kPrdBlock), 0,
               (const uint64_t *)g->d_off, (const uint32_t *)g->d_slots, n, (const uint32_t *)fa,
               (const double *)dod, ngh);
      launch_t(ctx, "pr_delta", k_prd_pull_heavy, dim3(ctx->num_sms * 8), dim3(kPrdBlock), 0,
               (const uint64_t *)g->d_off, (const uint32_t *)g->d_slots, (const uint32_t *)heavy,
               (const PrdStats *)st, (const uint32_t *)fa, (const double *)dod, ngh);
    } else if (fsize) {
      launch_t(ctx, "pr_delta", k_prd_push, dim3(grid_for(ctx, fsize * 32, kPrdBlock, 8)), dim3(kPrdBlock), 0,
               (const uint64_t *)g->d_off, (const uint32_t *)g->d_slots, (const uint32_t *)la, fsize,
               (const double *)dod, ngh);
    }
    BYO_CU(ctx, cudaMemsetAsync(st, 0, 16, ctx->stream));  // count, outdeg
    if (round == 1)
      launch(ctx, k_prd_filter<true>, dim3(fgrid), dim3(kPrdBlock), 0, (const uint32_t *)g->d_deg, n, d_p, delta,
             dod, ngh, fb, lb, st, part, local_eps);
    else
      launch(ctx, k_prd_filter<false>, dim3(fgrid), dim3(kPrdBlock), 0, (const uint32_t *)g->d_deg, n, d_p, delta,
             dod, ngh, fb, lb, st, part, local_eps);
    launch(ctx, k_prd_l1, dim3(1), dim3(256), 0, (const double *)part, (uint32_t)fgrid, st);
    BYO_CU(ctx, cudaMemcpyAsync(h, st, sizeof(PrdStats), cudaMemcpyDeviceToHost, ctx->stream));
    BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
    L1 = h->l1;
    if (L1 < eps) break;
    fsize = h->count;
    fdeg = h->outdeg;
    have_list = true;
    std::swap(fa, fb);
    std::swap(la, lb);
  }
  if (round > max_iters) round = max_iters;
  if (rounds_out) *rounds_out = round;
  if (l1_out) *l1_out = L1;
  return check_launch(ctx, "pagerank_delta");
}

}  // namespace byo

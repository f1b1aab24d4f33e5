// pcsr.cu -- the Packed CSR container (BYO_CONTAINER_PCSR): the layout of
// the reference's PCSR target (benchmarks/run_structures/run_pcsr.cc:24-99;
// its PCSR class lives in the un-vendored Packed-Memory-Array submodule and
// follows the published Packed CSR of Wheatman & Xu, HPEC 2018).
//
// One packed array holds, in vertex order, a sentinel for every vertex
// followed by its sorted neighbours.  The array is cut into leaves of kPL
// slots, each left-packed with its slack at the end, and kept within density
// bounds the way a packed-memory array is: a leaf that would overflow has the
// smallest aligned window of leaves around it redistributed evenly, and the
// whole array is laid out again when even the root is too dense (or, after a
// remove, too sparse).  A slot holds a neighbour id or kSentinel: a vertex's
// sentinel slot reads kSentinel too, and one bit per slot (head) marks the
// sentinels.  vbeg[v] is the slot of v's sentinel and is the container's
// d_off: v's slot range [vbeg[v], vbeg[v+1]) is its sentinel, its neighbours
// and gaps, so the gapped view needs no rebuild after an update.  4 bytes per
// slot and a bit, against the PMA container's 8 (src and dst per slot).
//
// Elements are ordered by a composite key: (v << 33) for v's sentinel and
// (v << 33) | (w + 1) for the edge (v, w).  Every leaf keeps the vertex that
// owns its first element (lv) and a routing separator (sep): every element of
// leaf j lies in [sep[j], sep[j+1]).  The owner of any element is lv plus the
// sentinels before it in the leaf, so leaves decode independently.
//
// A batch is validated and sorted on the device and routed to leaves by sep
// (batch keys compared as composite keys, duplicates skipped by the merge); a
// warp per touched leaf decodes it into shared memory, ranks each batch key in
// it and scatters the merged sequence back in place when it fits, moving the
// sentinels' vbeg with them and the degrees by atomics.  A leaf that would
// overflow leaves its merged sequence in an overflow area for the windowed
// redistribution.
#include <algorithm>
#include <cmath>

#include "device.cuh"
#include "internal.h"

namespace byo {

constexpr uint32_t kPL = 512;       // slots per leaf
constexpr uint32_t kPW = kPL / 32;  // head words per leaf
constexpr double kPBuild = 0.70;    // density of a fresh layout
constexpr double kPRootMax = 0.90;  // upper density bound at the root (1.0 at a leaf)
constexpr double kPRootMin = 0.25;  // a remove below this lays the array out smaller
constexpr uint64_t kCkMask = (1ull << 33) - 1;
constexpr uint32_t kNoWindow = 0xFFFFFFFFu;
constexpr int kPcsrWarps = 4;  // warps per CTA of the merge (24.6 KB of shared memory, 8 CTAs per SM)

struct Pcsr {
  uint64_t NL = 0;
  int H = 0;
  uint32_t *slots = nullptr, *head = nullptr, *cnt = nullptr, *lv = nullptr;
  uint64_t *sep = nullptr;
  DevBuf keys_a, keys_b, bstart, rcount, rpre, marks, win, staging, ovf, ovf_off, misc;
  uint64_t rebuilds = 0, windows = 0;
};

__host__ __device__ __forceinline__ uint64_t ck_sent(uint64_t v) { return v << 33; }
__host__ __device__ __forceinline__ uint64_t ck_edge(uint64_t v, uint64_t w) { return (v << 33) | (w + 1); }
__device__ __forceinline__ bool ck_is_sent(uint64_t k) { return (k & kCkMask) == 0; }
// composite key of a batch key src << 32 | dst (order preserving)
__device__ __forceinline__ uint64_t ck_of(uint64_t k) { return ck_edge(k >> 32, k & 0xFFFFFFFFull); }

__host__ __device__ __forceinline__ double pcsr_bound(int h, int H) {
  return H == 0 ? kPRootMax : 1.0 - (1.0 - kPRootMax) * (double)h / (double)H;
}

static int ceil_log2_u64(uint64_t x) {
  int h = 0;
  while ((1ull << h) < x) h++;
  return h;
}

static uint64_t pcsr_leaves_for(uint64_t elems) {
  const uint64_t nl = (uint64_t)std::ceil((double)elems / (kPBuild * kPL));
  return nl ? nl : 1;
}

// ---------------------------------------------------------------- decode / encode

// Sentinel counts of leaf j's head words, one word per lane (lanes >= kPW
// hold 0): the word, its exclusive prefix and whether slot 0 is a sentinel.
struct HeadScan {
  uint32_t word, before, first;
};

__device__ __forceinline__ HeadScan head_scan(const uint32_t *__restrict__ head, uint64_t j) {
  const unsigned lane = lane_id();
  const uint32_t hw = lane < kPW ? head[j * kPW + lane] : 0u;
  const uint32_t pc = __popc(hw);
  const uint32_t incl = warp_inclusive_scan(pc);
  return HeadScan{hw, incl - pc, __shfl_sync(kFull, hw, 0) & 1u};
}

// Owner and sentinel bit of slot i of a leaf from its head scan; every lane
// of the warp calls it (the shuffles read word i / 32).
__device__ __forceinline__ uint64_t slot_owner(const HeadScan &hs, uint32_t lv0, uint32_t i, bool &sent) {
  const uint32_t w = (i >> 5) & 31u;
  const uint32_t word = __shfl_sync(kFull, hs.word, w);
  const uint32_t before = __shfl_sync(kFull, hs.before, w);
  sent = (word >> (i & 31)) & 1u;
  const uint32_t s_incl = before + __popc(word & (0xFFFFFFFFu >> (31 - (i & 31))));
  return (uint64_t)lv0 + s_incl - hs.first;
}

// Composite keys of leaf j's c elements into A; a warp.
__device__ __forceinline__ void pcsr_decode_leaf(const uint32_t *__restrict__ slots, const uint32_t *__restrict__ head,
                                                 uint64_t j, uint32_t c, uint32_t lv0, uint64_t *A) {
  const HeadScan hs = head_scan(head, j);
  for (uint32_t base = 0; base < c; base += 256) {
    uint32_t x[8];  // eight loads per lane in flight
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const uint32_t i = base + 32 * q + lane_id();
      x[q] = i < c ? slots[j * kPL + i] : kSentinel;
    }
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const uint32_t i = base + 32 * q + lane_id();
      bool sent;
      const uint64_t owner = slot_owner(hs, lv0, i, sent);
      if (i < c) A[i] = sent ? ck_sent(owner) : ck_edge(owner, x[q]);
    }
  }
}

// Writes n_el composite keys E[0..) into leaf j (left-packed, the rest gaps):
// slots, head words, cnt, lv and the vbeg of every sentinel; a warp.  The
// separator is the caller's.
__device__ __forceinline__ void pcsr_encode_leaf(uint32_t *slots, uint32_t *head, uint32_t *cnt, uint32_t *lv,
                                                 uint64_t *vbeg, uint64_t j, const uint64_t *E, uint32_t n_el) {
  const unsigned lane = lane_id();
  for (uint32_t base = 0; base < kPL; base += 32) {
    const uint32_t i = base + lane;
    bool s = false;
    uint32_t val = kSentinel;
    if (i < n_el) {
      const uint64_t k = E[i];
      s = ck_is_sent(k);
      if (s) vbeg[k >> 33] = j * kPL + i;
      else val = (uint32_t)((k & kCkMask) - 1);
    }
    slots[j * kPL + i] = val;
    const unsigned b = __ballot_sync(kFull, s);
    if (lane == 0) head[j * kPW + (base >> 5)] = b;
  }
  if (lane == 0) {
    cnt[j] = n_el;
    lv[j] = n_el ? (uint32_t)(E[0] >> 33) : 0u;
  }
}

// ---------------------------------------------------------------- build

// Elements of a CSR (keys src << 32 | dst, sorted; off its offsets): v's
// sentinel at off[v] + v, edge i of source u at i + u + 1.
__global__ void k_pcsr_elems(const uint64_t *__restrict__ keys, uint64_t m, const uint64_t *__restrict__ off,
                             uint64_t n, uint64_t *out) {
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, nthr = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t v = tid; v < n; v += nthr) out[off[v] + v] = ck_sent(v);
  for (uint64_t i = tid; i < m; i += nthr) {
    const uint64_t k = keys[i], u = k >> 32;
    out[i + u + 1] = ck_edge(u, k & 0xFFFFFFFFull);
  }
}

// Each window's staged elements spread evenly over its leaves; a warp per
// leaf.  Window mode (all = 0): leaf j with level h = lvl[j] belongs to the
// aligned window [a, e) of 2^h leaves, whose elements are
// stage[rpre[a] .. rpre[e]); its first leaf keeps its separator.  Layout mode
// (all = 1): one window over all NL leaves holding stage[0 .. total).
__global__ void __launch_bounds__(256) k_pcsr_spread(const uint64_t *__restrict__ stage, const uint64_t *__restrict__ rpre,
                                                     const uint32_t *__restrict__ lvl, uint64_t NL, int all,
                                                     uint64_t total, uint32_t *slots, uint32_t *head, uint32_t *cnt,
                                                     uint32_t *lv, uint64_t *sep, uint64_t *vbeg) {
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t j = gw; j < NL; j += nw) {
    uint64_t a = 0, e = NL, s0 = 0, T = total;
    if (!all) {
      const uint32_t h = lvl[j];
      if (h == kNoWindow) continue;
      a = (j >> h) << h;
      e = a + (1ull << h);
      if (e > NL) e = NL;
      s0 = rpre[a];
      T = rpre[e] - s0;
    }
    const uint64_t k = j - a, width = e - a;
    const uint64_t lo = T * k / width, hi = T * (k + 1) / width;
    pcsr_encode_leaf(slots, head, cnt, lv, vbeg, j, stage + s0 + lo, (uint32_t)(hi - lo));
    if (lane_id() == 0) {
      if (all && k == 0) {
        sep[j] = 0;
      } else if (k > 0) {
        uint64_t s = ~0ull;  // an empty leaf takes the next element's key
        if (hi > lo) s = stage[s0 + lo];
        else if (hi < T) s = stage[s0 + hi];
        else if (!all && e < NL) s = sep[e];  // the next window's first leaf keeps its separator
        sep[j] = s;
      }
    }
    __syncwarp();
  }
}

static int pcsr_alloc(byo_ctx *ctx, Pcsr *p, uint64_t NL) {
  uint32_t *slots = nullptr, *head = nullptr, *cnt = nullptr, *lv = nullptr;
  uint64_t *sep = nullptr;
  cudaError_t e = cudaMalloc(&slots, NL * kPL * 4);
  if (e == cudaSuccess) e = cudaMalloc(&head, NL * kPW * 4);
  if (e == cudaSuccess) e = cudaMalloc(&cnt, NL * 4);
  if (e == cudaSuccess) e = cudaMalloc(&lv, NL * 4);
  if (e == cudaSuccess) e = cudaMalloc(&sep, (NL + 1) * 8);
  if (e != cudaSuccess) {
    cudaGetLastError();
    cudaFree(slots);
    cudaFree(head);
    cudaFree(cnt);
    cudaFree(lv);
    cudaFree(sep);
    return set_error(ctx, BYO_ENOMEM, "pcsr: leaves", e);
  }
  cudaFree(p->slots);
  cudaFree(p->head);
  cudaFree(p->cnt);
  cudaFree(p->lv);
  cudaFree(p->sep);
  p->slots = slots;
  p->head = head;
  p->cnt = cnt;
  p->lv = lv;
  p->sep = sep;
  p->NL = NL;
  p->H = ceil_log2_u64(NL);
  return BYO_OK;
}

// Lays the E sorted elements in `elems` out over NL new leaves.
static int pcsr_layout(byo_graph *g, const uint64_t *elems, uint64_t E, uint64_t NL) {
  byo_ctx *ctx = g->ctx;
  Pcsr *p = g->pcsr;
  BYO_TRY(pcsr_alloc(ctx, p, NL));
  g->d_slots = p->slots;
  g->nslots = NL * kPL;
  launch(ctx, k_pcsr_spread, dim3(grid_for(ctx, NL * 32, 256)), dim3(256), 0, elems, (const uint64_t *)nullptr,
         (const uint32_t *)nullptr, NL, 1, E, p->slots, p->head, p->cnt, p->lv, p->sep, g->d_off);
  uint64_t *h = nullptr;
  BYO_TRY(pinned(ctx, 4096, (void **)&h));
  h[0] = NL * kPL;
  BYO_CU(ctx, cudaMemcpyAsync(g->d_off + g->n, h, 8, cudaMemcpyHostToDevice, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));  // the pinned word is reused
  return check_launch(ctx, "pcsr_layout");
}

int pcsr_build(byo_graph *g, const uint64_t *d_keys, uint64_t m) {
  byo_ctx *ctx = g->ctx;
  if (g->n >= (1ull << 31)) return set_error(ctx, BYO_EINVAL, "pcsr: n must be below 2^31");
  g->pcsr = new Pcsr();
  Pcsr *p = g->pcsr;
  const uint64_t n = g->n, E = n + m;
  BYO_TRY(offsets_from_keys(ctx, d_keys, m, n, g->d_off));  // the CSR's offsets give the element ranks
  BYO_TRY(degrees_from_offsets(ctx, g->d_off, n, g->d_deg));
  BYO_TRY(ensure(ctx, p->staging, (E ? E : 1) * 8));
  uint64_t *el = (uint64_t *)p->staging.p;
  launch(ctx, k_pcsr_elems, dim3(grid_for(ctx, std::max(n, m), 256)), dim3(256), 0, d_keys, m,
         (const uint64_t *)g->d_off, n, el);
  return pcsr_layout(g, el, E, pcsr_leaves_for(E));
}

void pcsr_destroy(Pcsr *p) {
  if (!p) return;
  cudaFree(p->slots);
  cudaFree(p->head);
  cudaFree(p->cnt);
  cudaFree(p->lv);
  cudaFree(p->sep);
  for (DevBuf *b : {&p->keys_a, &p->keys_b, &p->bstart, &p->rcount, &p->rpre, &p->marks, &p->win,
                    &p->staging, &p->ovf, &p->ovf_off, &p->misc})
    free_buf(*b);
  delete p;
}

uint64_t pcsr_leaf_slots() { return kPL; }

// ---------------------------------------------------------------- snapshot

// The compact CSR of the contents: the edge element of global rank e
// (epre[j] + its index in leaf j) owned by u goes to out[e - u - 1], since
// u's sentinel has rank u + offc[u] and its k-th edge rank u + offc[u] + 1 + k.
__global__ void __launch_bounds__(256) k_pcsr_compact(const uint32_t *__restrict__ slots,
                                                      const uint32_t *__restrict__ head,
                                                      const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ lv,
                                                      const uint64_t *__restrict__ epre, uint64_t NL, uint64_t m,
                                                      uint32_t *out) {
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t j = gw; j < NL; j += nw) {
    const uint32_t c = cnt[j];
    if (!c) continue;
    const HeadScan hs = head_scan(head, j);
    const uint64_t e0 = epre[j];
    const uint32_t l0 = lv[j];
    // eight streaming loads per lane in flight before the stores
    for (uint32_t base = 0; base < c; base += 256) {
      uint32_t x[8];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const uint32_t i = base + 32 * q + lane_id();
        x[q] = i < c ? __ldcs(slots + j * kPL + i) : kSentinel;
      }
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const uint32_t i = base + 32 * q + lane_id();
        bool sent;
        const uint64_t owner = slot_owner(hs, l0, i, sent);
        const uint64_t at = e0 + i - owner - 1;
        if (i < c && !sent && at < m) out[at] = x[q];
      }
    }
  }
}

int pcsr_compact(byo_graph *g, uint32_t *out) {
  byo_ctx *ctx = g->ctx;
  Pcsr *p = g->pcsr;
  BYO_TRY(ensure(ctx, p->rpre, (p->NL + 1) * 8));
  uint64_t *epre = (uint64_t *)p->rpre.p;
  BYO_TRY(scan_u32_to_u64(ctx, p->cnt, p->NL, epre));
  launch_t(ctx, "pcsr_compact", k_pcsr_compact, dim3(grid_for(ctx, p->NL * 32, 256, 16)), dim3(256), 0,
           (const uint32_t *)p->slots, (const uint32_t *)p->head, (const uint32_t *)p->cnt, (const uint32_t *)p->lv,
           (const uint64_t *)epre, p->NL, g->m, out);
  return check_launch(ctx, "pcsr_compact");
}

// ---------------------------------------------------------------- update

// flags[0]: a key with src or dst >= n; flags[1]: `sorted` input not
// strictly increasing.
__global__ void k_pcsr_check(const uint64_t *__restrict__ keys, uint64_t b, uint64_t n, int sorted,
                             unsigned int *flags) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < b; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[i];
    if ((k >> 32) >= n || (k & 0xFFFFFFFFull) >= n) atomicOr(flags, 1u);
    if (sorted && i > 0 && keys[i - 1] >= k) atomicOr(flags + 1, 1u);
  }
}

// bstart[j] = first batch key (sorted src << 32 | dst) whose composite key is
// >= sep[j]; bstart[0] = 0, bstart[NL] = b.  A batch the check flagged (a key
// >= n, or a "sorted" batch that is not) is routed to no leaf, so the merge
// changes nothing; the host rejects it after the merge.
__global__ void k_pcsr_route(const uint64_t *__restrict__ sep, uint64_t NL, const uint64_t *__restrict__ keys,
                             uint64_t b, const unsigned int *bad, uint64_t *bstart) {
  const bool drop = bad[0] || bad[1];
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j <= NL; j += (uint64_t)gridDim.x * blockDim.x) {
    if (drop) {
      bstart[j] = 0;
      continue;
    }
    if (j == 0 || j == NL) {
      bstart[j] = j ? b : 0;
      continue;
    }
    const uint64_t s = sep[j];
    uint64_t lo = 0, hi = b;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (ck_of(keys[mid]) < s) lo = mid + 1;
      else hi = mid;
    }
    bstart[j] = lo;
  }
}

// Rank of x in A[0..c) (lower bound).
__device__ __forceinline__ uint32_t rank_in(const uint64_t *A, uint32_t c, uint64_t x) {
  uint32_t l = 0, hi = c;
  while (l < hi) {
    const uint32_t mid = (l + hi) >> 1;
    if (A[mid] < x) l = mid + 1;
    else hi = mid;
  }
  return l;
}

// Leaf of every key of a sorted batch: the last leaf whose separator is <= its
// composite key (as k_pcsr_route assigns them).  Nothing when the batch
// failed validation (flags[0] | flags[1]).
__global__ void k_pcsr_leafof(const uint64_t *__restrict__ sep, uint64_t NL, const uint64_t *__restrict__ keys,
                              uint64_t b, const unsigned int *flags, uint32_t *leaf) {
  if (flags[0] | flags[1]) return;
  for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < b; q += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t x = ck_of(keys[q]);
    uint64_t lo = 0, len = NL;
    while (len > 1) {
      const uint64_t half = len >> 1;
      if (sep[lo + half] <= x) lo += half;
      len -= half;
    }
    leaf[q] = (uint32_t)lo;
  }
}

// The segment list of a sorted batch from its keys' leaves: one entry per
// leaf with keys, (leaf, b0 << 32 | b1), in any order.
__global__ void k_pcsr_segs(const uint32_t *__restrict__ leaf, uint64_t b, const unsigned int *flags, uint64_t *seg,
                            unsigned long long *nseg) {
  if (flags[0] | flags[1]) return;
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, nthr = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = tid & ~31ull; base < b; base += nthr) {
    const uint64_t q = base + lane_id();
    const uint32_t j = q < b ? leaf[q] : 0u;
    const bool start = q < b && (q == 0 || leaf[q - 1] != j);
    uint64_t b1 = b;
    if (start) {  // the first key past q on a later leaf
      uint64_t l = q + 1, h = b;
      while (l < h) {
        const uint64_t mid = (l + h) >> 1;
        if (leaf[mid] <= j) l = mid + 1;
        else h = mid;
      }
      b1 = l;
    }
    const uint64_t at = warp_append(start, nseg);
    if (start) {
      seg[2 * at] = j;
      seg[2 * at + 1] = q << 32 | b1;
    }
  }
}

// rcount of the listed leaves from the merge's segment list.
__global__ void k_pcsr_seg_counts(const uint64_t *__restrict__ seg, const unsigned long long *nseg, uint32_t *rcount) {
  const uint64_t ns = *nseg;
  for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < ns; q += (uint64_t)gridDim.x * blockDim.x)
    rcount[seg[2 * q] & 0xFFFFFFFFull] = (uint32_t)(seg[2 * q] >> 32);
}

// Where one merged element goes: in place (its slot, the sentinel bit in the
// warp's head words H, vbeg for a sentinel, lv for position 0) or, for a leaf
// that overflows, its composite key in the overflow area.
struct MergeOut {
  uint32_t *slots;
  uint64_t *vbeg;
  uint32_t *lv;
  uint32_t *H;
  uint64_t j;
  uint64_t *ovf;  // non-null: the leaf overflows
};

__device__ __forceinline__ void merge_put(const MergeOut &o, uint32_t pos, uint64_t k) {
  if (o.ovf) {
    o.ovf[pos] = k;
    return;
  }
  const uint64_t at = o.j * kPL + pos;
  if (ck_is_sent(k)) {
    o.slots[at] = kSentinel;
    o.vbeg[k >> 33] = at;
    atomicOr(o.H + (pos >> 5), 1u << (pos & 31));
  } else {
    o.slots[at] = (uint32_t)((k & kCkMask) - 1);
  }
  if (pos == 0) o.lv[o.j] = (uint32_t)(k >> 33);
}

// A warp per leaf with batch keys (sorted src << 32 | dst; a key equal to its
// predecessor is skipped, so the batch needs no separate deduplication): the
// leaf is decoded into A (shared), each batch key ranked in A, and every
// merged element written straight to its position -- in place, the leaf's
// own slots, when the result fits, else to the overflow area.  Positions come
// from ranks:
//   insert: A[i] moves by the kept batch keys of rank <= i (a scan of D, the
//           kept keys per rank); kept key x of rank l lands at l + the kept
//           keys before it, written while ranking when the leaf cannot
//           overflow (c + batch keys <= kPL)
//   remove: A[i] moves back by the removed keys before it, and the slots a
//           remove frees at the end become gaps.
// Slots and sentinel bits past max(old, new count) are gaps already.
// kList: the leaves with keys come from a segment list (seg[2q] = leaf,
// seg[2q + 1] = b0 << 32 | b1, *nseg entries) instead of bstart over every
// leaf, and a leaf's count after the merge goes to the high half of seg[2q]
// instead of rcount.
// ctr: [0] overflow cursor, [1] overflowing leaves, [2] change of the edge
// count, [3] leaves merged, [4] elements they held.
template <bool kList>
__global__ void __launch_bounds__(32 * kPcsrWarps, 8) k_pcsr_merge(
    uint32_t *slots, uint32_t *head, uint32_t *cnt, uint32_t *lv, uint64_t NL, const uint64_t *__restrict__ keys,
    const uint64_t *__restrict__ bstart, uint64_t *seg, const unsigned long long *nseg, int insert, uint32_t *rcount,
    uint64_t *ovf, uint64_t *ovf_off, unsigned long long *ctr, uint32_t *deg, uint64_t *vbeg) {
  __shared__ uint64_t As[kPcsrWarps][kPL];
  __shared__ uint32_t Ds[kPcsrWarps][kPL + 1];
  __shared__ uint32_t Hs[kPcsrWarps][kPW];
  const unsigned w = threadIdx.x >> 5, lane = lane_id();
  uint64_t *A = As[w];
  uint32_t *D = Ds[w];
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  long long dsum = 0;
  unsigned long long nleaves = 0, nentries = 0;
  const uint64_t nwork = kList ? *nseg : NL;
  // the next work item's leaf, batch range, count and first owner are loaded
  // while this one merges (a leaf is listed once, and only the warp merging
  // it writes its cnt and lv)
  uint64_t nj = 0, nb0 = 0, nb1 = 0;
  uint32_t ncnt = 0, nlv = 0;
  auto fetch = [&](uint64_t q) {
    if (kList) {
      nj = seg[2 * q];
      const uint64_t r = seg[2 * q + 1];
      nb0 = r >> 32;
      nb1 = r & 0xFFFFFFFFull;
    } else {
      nj = q;
      nb0 = bstart[q];
      nb1 = bstart[q + 1];
    }
    ncnt = cnt[nj];
    nlv = lv[nj];
  };
  if (gw < nwork) fetch(gw);
  for (uint64_t q = gw; q < nwork; q += nw) {
    const uint64_t j = nj, b0 = nb0, b1 = nb1;
    const uint32_t c = min(ncnt, kPL), lv0 = nlv;
    if (q + nw < nwork) fetch(q + nw);
    if (b0 == b1) {
      if (lane == 0) rcount[j] = c;
      continue;
    }
    nleaves++;
    nentries += c;
    // the first round of batch keys is in flight with the leaf's loads
    uint64_t xn = b0 + lane < b1 ? keys[b0 + lane] : 0;
    pcsr_decode_leaf(slots, head, j, c, lv0, A);
    for (uint32_t i = lane; i <= c; i += 32) D[i] = 0;
    if (lane < kPW) Hs[w][lane] = 0;
    __syncwarp();
    MergeOut o{slots, vbeg, lv, Hs[w], j, nullptr};
    const bool direct = insert && c + (b1 - b0) <= kPL;
    uint32_t changed = 0;
    uint64_t prev_last = 0;  // the previous round's last key
    for (uint64_t t0 = b0; t0 < b1; t0 += 32) {
      const uint64_t t = t0 + lane;
      bool act = false;
      uint32_t l = 0;
      uint64_t x = 0;
      const uint64_t k = xn;
      // the next round's key loads while this round ranks
      xn = t + 32 < b1 ? keys[t + 32] : 0;
      uint64_t before = __shfl_up_sync(kFull, k, 1);
      if (lane == 0) before = prev_last;
      prev_last = __shfl_sync(kFull, k, 31);
      if (t < b1 && !(t > b0 && before == k)) {
        x = ck_of(k);
        l = rank_in(A, c, x);
        const bool present = l < c && A[l] == x;
        act = insert ? !present : present;
        if (act) {
          if (insert) atomicAdd(D + l, 1u);
          else D[l] = 1u;
          atomicAdd(deg + (x >> 33), insert ? 1u : 0xFFFFFFFFu);
        }
      }
      const unsigned ma = __ballot_sync(kFull, act);
      if (direct && act) merge_put(o, l + changed + __popc(ma & lanemask_lt()), x);
      changed += __popc(ma);
    }
    __syncwarp();
    const uint32_t r = insert ? c + changed : c - changed;
    dsum += insert ? (long long)changed : -(long long)changed;
    if (r > kPL) {
      unsigned long long at = 0;
      if (lane == 0) {
        at = atomicAdd(&ctr[0], (unsigned long long)r);
        atomicAdd(&ctr[1], 1ull);
        ovf_off[j] = at;
      }
      at = __shfl_sync(kFull, at, 0);
      o.ovf = ovf + at;
    }
    if (insert) {
      uint32_t carry = 0;
      for (uint32_t i0 = 0; i0 <= c; i0 += 32) {
        const uint32_t i = i0 + lane;
        const uint32_t inc = warp_inclusive_scan(i <= c ? D[i] : 0u) + carry;
        if (i < c) merge_put(o, i + inc, A[i]);
        carry = __shfl_sync(kFull, inc, 31);
      }
      if (!direct) {
        uint32_t kept_before = 0;
        for (uint64_t t0 = b0; t0 < b1; t0 += 32) {
          const uint64_t t = t0 + lane;
          bool keep = false;
          uint32_t l = 0;
          uint64_t x = 0;
          if (t < b1 && !(t > b0 && keys[t - 1] == keys[t])) {
            x = ck_of(keys[t]);
            l = rank_in(A, c, x);
            keep = !(l < c && A[l] == x);
          }
          const unsigned mk = __ballot_sync(kFull, keep);
          if (keep) merge_put(o, l + kept_before + __popc(mk & lanemask_lt()), x);
          kept_before += __popc(mk);
        }
      }
    } else {
      uint32_t removed = 0;
      for (uint32_t i0 = 0; i0 < c; i0 += 32) {
        const uint32_t i = i0 + lane;
        const bool gone = i < c && D[i];
        const unsigned mg = __ballot_sync(kFull, gone);
        if (i < c && !gone) merge_put(o, i - removed - __popc(mg & lanemask_lt()), A[i]);
        removed += __popc(mg);
      }
    }
    __syncwarp();
    if (!o.ovf) {
      // in place; the separator stays (every key routed here is >= it)
      for (uint32_t i = r + lane; i < c; i += 32) slots[j * kPL + i] = kSentinel;
      if (lane < (max(c, r) + 31) / 32) head[j * kPW + lane] = Hs[w][lane];
      if (lane == 0) {
        cnt[j] = r;
        if (r == 0) lv[j] = 0;
      }
    }
    if (lane == 0) {
      if (kList) seg[2 * q] = j | (uint64_t)r << 32;
      else rcount[j] = r;
    }
    __syncwarp();
  }
  if (lane == 0) {
    if (dsum) atomicAdd(&ctr[2], (unsigned long long)dsum);
    if (nleaves) {
      atomicAdd(&ctr[3], nleaves);
      atomicAdd(&ctr[4], nentries);
    }
  }
}

// For each overflowing leaf the smallest aligned window within its density
// bound: marks[h * NL + index] = 1; *grow when even the root is too dense.
__global__ void k_pcsr_windows(const uint32_t *__restrict__ rcount, const uint64_t *__restrict__ rpre, uint64_t NL,
                               int H, uint8_t *marks, unsigned int *grow) {
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < NL; j += (uint64_t)gridDim.x * blockDim.x) {
    if (rcount[j] <= kPL) continue;
    bool found = false;
    for (int h = 1; h <= H && !found; h++) {
      const uint64_t a = (j >> h) << h;
      uint64_t e = a + (1ull << h);
      if (e > NL) e = NL;
      if ((double)(rpre[e] - rpre[a]) <= pcsr_bound(h, H) * (double)(e - a) * kPL) {
        marks[(uint64_t)h * NL + (j >> h)] = 1;
        found = true;
      }
    }
    if (!found) atomicOr(grow, 1u);
  }
}

// Level of every leaf's window: the highest marked ancestor (kNoWindow if none).
__global__ void k_pcsr_cover(const uint8_t *__restrict__ marks, uint64_t NL, int H, uint32_t *lvl) {
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < NL; j += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t code = kNoWindow;
    for (int h = H; h >= 1; h--)
      if (marks[(uint64_t)h * NL + (j >> h)]) {
        code = (uint32_t)h;
        break;
      }
    lvl[j] = code;
  }
}

// The elements of every leaf in a window (every leaf when lvl is null) as
// composite keys at stage[rpre[j] ...]: from the overflow area for a leaf
// that overflowed, decoded from the leaf otherwise.  A warp per leaf.
__global__ void __launch_bounds__(256) k_pcsr_gather(const uint32_t *__restrict__ slots,
                                                     const uint32_t *__restrict__ head,
                                                     const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ lv,
                                                     const uint32_t *__restrict__ rcount,
                                                     const uint64_t *__restrict__ rpre, const uint64_t *__restrict__ ovf,
                                                     const uint64_t *__restrict__ ovf_off,
                                                     const uint32_t *__restrict__ lvl, uint64_t NL, uint64_t *stage) {
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t j = gw; j < NL; j += nw) {
    if (lvl && lvl[j] == kNoWindow) continue;
    const uint32_t r = rcount[j];
    uint64_t *out = stage + rpre[j];
    if (r > kPL) {
      const uint64_t *src = ovf + ovf_off[j];
      for (uint32_t i = lane_id(); i < r; i += 32) out[i] = src[i];
    } else {
      pcsr_decode_leaf(slots, head, j, r, lv[j], out);
    }
  }
}

int pcsr_update(byo_graph *g, const uint64_t *d_keys_in, uint64_t count, int sorted, int insert,
                uint64_t *changed) {
  byo_ctx *ctx = g->ctx;
  Pcsr *p = g->pcsr;
  if (!p) return set_error(ctx, BYO_ENOTSUP, "not a PCSR container");
  g->version++;  // any snapshot of the contents is stale from here on
  const uint64_t n = g->n, m_before = g->m;
  // 1. validate on the device, sort (duplicates stay: the merge skips them).
  // No sort indexes out of bounds by key, and the segment kernels or the
  // routing drop an invalid batch (the merge then has no work), so the
  // validation is read after the single synchronisation of the update.  A
  // batch of at most one key per leaf takes the segment list (only its own
  // leaves are visited).
  const uint64_t NL = p->NL;
  const bool small = !sorted && count <= sort_small_max();
  const bool list = count <= NL && count < (1ull << 32);
  BYO_TRY(ensure(ctx, p->keys_a, count * 8));
  BYO_TRY(ensure(ctx, p->keys_b, count * 8));
  BYO_TRY(ensure(ctx, p->misc, 128));
  uint64_t *ka = (uint64_t *)p->keys_a.p, *kb = (uint64_t *)p->keys_b.p;
  // misc: [0..4] merge counters, [5] segments, [6..7] the small sort's bounds,
  // then flags [0] range, [1] order, [2] grow
  unsigned long long *ctr = (unsigned long long *)p->misc.p;
  unsigned int *flags = (unsigned int *)(ctr + 8);
  BYO_CU(ctx, cudaMemsetAsync(p->misc.p, 0, 128, ctx->stream));
  launch(ctx, k_pcsr_check, dim3(grid_for(ctx, count, 256)), dim3(256), 0, d_keys_in, count, n, sorted, flags);
  uint64_t *h = nullptr;
  BYO_TRY(pinned(ctx, 4096, (void **)&h));
  const unsigned int *hf = (const unsigned int *)(h + 8);
  const uint64_t *batch = d_keys_in;
  uint64_t b = count;
  if (small) {
    BYO_TRY(sort_small_keys(ctx, d_keys_in, count, ka, ctr + 6));
    batch = ka;
  } else if (!sorted) {
    BYO_TRY(sort_bucketed(ctx, d_keys_in, count, n, ka, kb));
    batch = ka;
  }
  // 2. route and merge (bstart doubles as the segment list)
  const uint64_t list_words = list ? 2 * std::min<uint64_t>(count, NL) + 2 : 0;
  BYO_TRY(ensure(ctx, p->bstart, std::max<uint64_t>(NL + 1, list_words) * 8));
  BYO_TRY(ensure(ctx, p->rcount, NL * 4));
  BYO_TRY(ensure(ctx, p->rpre, (NL + 1) * 8));
  BYO_TRY(ensure(ctx, p->ovf, (n + m_before + b + 1) * 8));  // the merged leaves hold at most every element
  BYO_TRY(ensure(ctx, p->ovf_off, NL * 8));
  uint64_t *bstart = (uint64_t *)p->bstart.p, *rpre = (uint64_t *)p->rpre.p;
  uint32_t *rcount = (uint32_t *)p->rcount.p;
  if (list) {
    uint32_t *leaf = reinterpret_cast<uint32_t *>(kb);  // free once the batch is sorted
    launch(ctx, k_pcsr_leafof, dim3(grid_for(ctx, b, 256)), dim3(256), 0, (const uint64_t *)p->sep, NL, batch, b,
           (const unsigned int *)flags, leaf);
    launch(ctx, k_pcsr_segs, dim3(grid_for(ctx, b, 256)), dim3(256), 0, (const uint32_t *)leaf, b,
           (const unsigned int *)flags, bstart, ctr + 5);
    launch_t(ctx, "pcsr_merge", k_pcsr_merge<true>, dim3(grid_for(ctx, b * 32, 32 * kPcsrWarps, 8)),
             dim3(32 * kPcsrWarps), 0, p->slots, p->head, p->cnt, p->lv, NL, batch, (const uint64_t *)nullptr,
             bstart, (const unsigned long long *)(ctr + 5), insert, rcount, (uint64_t *)p->ovf.p,
             (uint64_t *)p->ovf_off.p, ctr, g->d_deg, g->d_off);
  } else {
    launch(ctx, k_pcsr_route, dim3(grid_for(ctx, NL + 1, 256)), dim3(256), 0, (const uint64_t *)p->sep, NL, batch,
           b, (const unsigned int *)flags, bstart);
    launch_t(ctx, "pcsr_merge", k_pcsr_merge<false>, dim3(grid_for(ctx, NL * 32, 32 * kPcsrWarps, 8)),
             dim3(32 * kPcsrWarps), 0, p->slots, p->head, p->cnt, p->lv, NL, batch, (const uint64_t *)bstart,
             (uint64_t *)nullptr, (const unsigned long long *)nullptr, insert, rcount, (uint64_t *)p->ovf.p,
             (uint64_t *)p->ovf_off.p, ctr, g->d_deg, g->d_off);
  }
  BYO_CU(ctx, cudaMemcpyAsync(h, ctr, 80, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaMemcpyAsync(h + 8, flags, 16, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  if (hf[0]) return set_error(ctx, BYO_EINVAL, "update key with src or dst >= n");
  if (hf[1]) return set_error(ctx, BYO_EINVAL, "sorted batch not increasing");
  const uint64_t novf = h[1], merged_leaves = h[3], merged_entries = h[4];
  const uint64_t m_after = (uint64_t)((long long)m_before + (long long)h[2]);
  g->m = m_after;
  const uint64_t ch = insert ? m_after - m_before : m_before - m_after;
  if (changed) *changed = ch;
  const uint64_t total = n + m_after;
  const bool shrink = !insert && NL > 1 && (double)total < kPRootMin * (double)NL * kPL;
  g->upd = UpdateStats{b, ch, merged_leaves, merged_entries, (novf || shrink) ? 2u : 0u};
  if (novf == 0 && !shrink) return check_launch(ctx, "pcsr_update");
  // 3. redistribution: windows over the counts after the merge, or a new
  // layout when the root is out of bounds
  if (list) {  // counts of every leaf: unlisted ones keep theirs
    BYO_CU(ctx, cudaMemcpyAsync(rcount, p->cnt, NL * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    launch(ctx, k_pcsr_seg_counts, dim3(grid_for(ctx, b, 256)), dim3(256), 0, (const uint64_t *)bstart,
           (const unsigned long long *)(ctr + 5), rcount);
  }
  BYO_TRY(scan_u32_to_u64(ctx, rcount, NL, rpre));
  BYO_TRY(ensure(ctx, p->staging, (total ? total : 1) * 8));
  BYO_TRY(ensure(ctx, p->win, NL * 4));
  uint64_t *stg = (uint64_t *)p->staging.p;
  uint32_t *lvl = (uint32_t *)p->win.p;
  bool rebuild = shrink || (double)total > kPRootMax * (double)NL * kPL;
  if (!rebuild) {
    BYO_TRY(ensure(ctx, p->marks, (uint64_t)(p->H + 1) * NL));
    uint8_t *marks = (uint8_t *)p->marks.p;
    BYO_CU(ctx, cudaMemsetAsync(marks, 0, (uint64_t)(p->H + 1) * NL, ctx->stream));
    launch(ctx, k_pcsr_windows, dim3(grid_for(ctx, NL, 256)), dim3(256), 0, (const uint32_t *)rcount,
           (const uint64_t *)rpre, NL, p->H, marks, flags + 2);
    BYO_CU(ctx, cudaMemcpyAsync(h + 8, flags, 16, cudaMemcpyDeviceToHost, ctx->stream));
    BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
    rebuild = hf[2] != 0;
    if (!rebuild)
      launch(ctx, k_pcsr_cover, dim3(grid_for(ctx, NL, 256)), dim3(256), 0, (const uint8_t *)marks, NL, p->H, lvl);
  }
  launch(ctx, k_pcsr_gather, dim3(grid_for(ctx, NL * 32, 256, 16)), dim3(256), 0, (const uint32_t *)p->slots,
         (const uint32_t *)p->head, (const uint32_t *)p->cnt, (const uint32_t *)p->lv, (const uint32_t *)rcount,
         (const uint64_t *)rpre, (const uint64_t *)p->ovf.p, (const uint64_t *)p->ovf_off.p,
         rebuild ? (const uint32_t *)nullptr : (const uint32_t *)lvl, NL, stg);
  BYO_TRY(check_launch(ctx, "pcsr_gather"));
  if (rebuild) {
    p->rebuilds++;
    return pcsr_layout(g, stg, total, pcsr_leaves_for(total));
  }
  p->windows++;
  launch_t(ctx, "pcsr_redistribute", k_pcsr_spread, dim3(grid_for(ctx, NL * 32, 256, 16)), dim3(256), 0,
           (const uint64_t *)stg, (const uint64_t *)rpre, (const uint32_t *)lvl, NL, 0, total, p->slots, p->head,
           p->cnt, p->lv, p->sep, g->d_off);
  return check_launch(ctx, "pcsr_update");
}

}  // namespace byo

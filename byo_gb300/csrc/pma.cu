// pma.cu -- packed-memory-array graph container on the device, the GB300
// counterpart of PMA_graph / CPMA (benchmarks/run_structures/run_single_pma.cc:
// 39-141; the CPMA itself lives in the un-vendored Packed-Memory-Array
// submodule).  Its observable contract is the sorted set of (src,dst) keys
// with insert = union and remove = difference after sort+unique of the batch
// (Graph::insert_batch / remove_batch, gbbs/graph.h:3071-3124).
//
// Layout in HBM (structure of arrays, leaves of kLeaf slots):
//   dst[NL*kLeaf], src[NL*kLeaf]  the keys (src<<32|dst) of leaf i sorted and
//                                 left-packed in [i*kLeaf, i*kLeaf+cnt[i]);
//                                 the rest of the leaf holds kSentinel
//   cnt[NL]                       elements per leaf
//   sep[NL]                       routing separators: leaf i holds keys in
//                                 [sep[i], sep[i+1]); sep[0] = 0
// `dst` is the graph's traversal slot array: vertex v's slot range
// [off[v], off[v+1]) holds its neighbours in order plus the gaps at the ends of
// the leaves it spans, so BFS / CC / PageRank run on the PMA unchanged.
//
// A batch update (keys already sorted and unique):
//   route     batch segment of every leaf (binary search of sep[i])
//   count     per leaf, how many batch keys are new (insert) / present (remove)
//   windows   an overflowing leaf takes the smallest aligned window of 2^h
//             leaves whose density after the update is within the bound for
//             height h (1.0 at a leaf down to kRootMax at the root); nested
//             windows resolve to the outermost; none fits -> grow
//   merge     one CTA per leaf with work: the leaf is staged in shared memory,
//             every output element's position is computed by rank (binary
//             searches, no serial merge), and written in place or, for a leaf
//             inside a window, to a staging buffer
//   spread    one CTA per windowed leaf copies its even share of the window's
//             elements back and resets its separator
//   view      off[v] / deg[v] for every vertex by binary search
// Bytes per update: 16 per batch key (sort passes excluded) + 16 per slot of
// every leaf touched (read + write of src and dst), twice for windowed leaves.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "device.cuh"
#include "gridsync.cuh"
#include "internal.h"
#include "msbfs.cuh"
#include "scan.cuh"

namespace byo {

constexpr uint32_t kLeafLg = 9;
constexpr uint32_t kLeaf = 1u << kLeafLg;
constexpr int kPmaBlock = 256;
constexpr double kBuildDensity = 0.70;
constexpr double kRootMax = 0.90;
constexpr double kRootMin = 0.25;  // below this after a remove: rebuild smaller

struct Pma {
  uint64_t NL = 0;        // leaves
  int H = 0;              // ceil(log2 NL)
  uint32_t *src = nullptr, *dst = nullptr, *cnt = nullptr;
  uint64_t *sep = nullptr;
  // update scratch
  DevBuf keys_a, keys_b;  // batch copies for sort / unique
  DevBuf bstart;          // uint64[NL+1]
  DevBuf rcount;          // uint32[NL] elements after the update
  DevBuf rpre;            // uint64[NL+1]
  DevBuf win;             // uint32[NL]   window code per leaf (or kNoWin)
  DevBuf marks;           // uint8[2*NL]  marked windows per (level,index)
  DevBuf staging;         // uint64[...]  windowed elements
  DevBuf misc;            // flags / counters
  DevBuf epre;            // uint64[NL+1] element prefix for the view
  DevBuf ovf, ovf_off;    // overflow area of the optimistic merge, per-leaf offsets
  DevBuf vrange, vchunks; // view rebuild: vertex range per leaf, chunks of the long ranges
  uint64_t rebuilds = 0, windows = 0;
};

constexpr uint32_t kNoWin = 0xFFFFFFFFu;

__device__ __forceinline__ uint64_t slot_key(const uint32_t *src, const uint32_t *dst, uint64_t s) {
  return ((uint64_t)src[s] << 32) | dst[s];
}

__host__ __device__ __forceinline__ double upper_bound_density(int h, int H) {
  return H == 0 ? kRootMax : 1.0 - (1.0 - kRootMax) * (double)h / (double)H;
}

// last leaf i with sep[i] <= key
__device__ __forceinline__ uint64_t route(const uint64_t *sep, uint64_t NL, uint64_t key) {
  uint64_t lo = 0, hi = NL;
  while (hi - lo > 1) {
    uint64_t mid = (lo + hi) >> 1;
    if (sep[mid] <= key) lo = mid; else hi = mid;
  }
  return lo;
}

// ---------------------------------------------------------------- batch preparation

__global__ void k_key_bounds(const uint64_t *__restrict__ keys, uint64_t cnt, unsigned long long *out) {
  uint64_t ms = 0, md = 0;
  const uint64_t nthr = (uint64_t)gridDim.x * blockDim.x;
  // four loads per thread in flight
  for (uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i0 < cnt; i0 += 4 * nthr) {
    uint64_t k[4];
#pragma unroll
    for (int q = 0; q < 4; q++) k[q] = i0 + q * nthr < cnt ? keys[i0 + q * nthr] : 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      ms = ms > (k[q] >> 32) ? ms : (k[q] >> 32);
      md = md > (k[q] & 0xFFFFFFFFull) ? md : (k[q] & 0xFFFFFFFFull);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    uint64_t a = __shfl_xor_sync(kFull, ms, o), b = __shfl_xor_sync(kFull, md, o);
    ms = ms > a ? ms : a;
    md = md > b ? md : b;
  }
  if (lane_id() == 0) {
    atomicMax(out, (unsigned long long)ms);
    atomicMax(out + 1, (unsigned long long)md);
  }
}

// strictly increasing check for callers that pass sorted = 1
__global__ void k_check_sorted(const uint64_t *__restrict__ keys, uint64_t cnt, unsigned int *bad) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x + 1; i < cnt;
       i += (uint64_t)gridDim.x * blockDim.x)
    if (keys[i] <= keys[i - 1]) atomicOr(bad, 1u);
}

// ---------------------------------------------------------------- routing / counting

// bounds (optional): the batch's largest src and dst, and *unsorted; a batch
// with a key >= n, or a "sorted" batch that is not, is routed to no leaf (the
// merge then changes nothing and the host rejects it after the merge).
__global__ void k_pma_route(const uint64_t *__restrict__ sep, uint64_t NL, const uint64_t *__restrict__ keys,
                            uint64_t b, uint64_t *bstart, const unsigned long long *bounds, uint64_t n,
                            const unsigned int *unsorted) {
  const bool drop = bounds && (bounds[0] >= n || bounds[1] >= n || *unsorted);
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i <= NL;
       i += (uint64_t)gridDim.x * blockDim.x) {
    if (drop) {
      bstart[i] = 0;
      continue;
    }
    if (i == NL) {
      bstart[NL] = b;
      continue;
    }
    const uint64_t s = sep[i];
    uint64_t lo = 0, hi = b;  // first index with keys >= s
    while (lo < hi) {
      uint64_t mid = (lo + hi) >> 1;
      if (keys[mid] < s) lo = mid + 1; else hi = mid;
    }
    bstart[i] = i == 0 ? 0 : lo;
  }
}

// rcount[i] = elements of leaf i after the update.  One warp per leaf; the
// leaf's keys are staged in the warp's shared memory, then every batch key of
// the leaf's segment is looked up there.
constexpr int kPmaWarps = 8;
__global__ void __launch_bounds__(32 * kPmaWarps) k_pma_count(const uint32_t *__restrict__ src,
                                                             const uint32_t *__restrict__ dst,
                                                             const uint32_t *__restrict__ cnt, uint64_t NL,
                                                             const uint64_t *__restrict__ keys,
                                                             const uint64_t *__restrict__ bstart, int insert,
                                                             uint32_t *rcount) {
  __shared__ uint64_t As[kPmaWarps][kLeaf];
  uint64_t *A = As[threadIdx.x >> 5];
  const unsigned lane = lane_id();
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t i = gw; i < NL; i += nw) {
    const uint64_t b0 = bstart[i], b1 = bstart[i + 1];
    const uint32_t c = cnt[i];
    if (b0 == b1) {
      if (lane == 0) rcount[i] = c;
      continue;
    }
    for (uint32_t e = lane; e < c; e += 32) A[e] = slot_key(src, dst, i * kLeaf + e);
    __syncwarp();
    uint64_t present = 0;
    for (uint64_t k = b0 + lane; k < b1; k += 32) {
      const uint64_t x = keys[k];
      uint32_t lo = 0, hi = c;
      while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (A[mid] < x) lo = mid + 1; else hi = mid;
      }
      present += (lo < c && A[lo] == x);
    }
    present = warp_sum(present);
    if (lane == 0) {
      const uint64_t r = insert ? (uint64_t)c + (b1 - b0) - present : (uint64_t)c - present;
      rcount[i] = (uint32_t)(r > 0xFFFFFFFFull ? 0xFFFFFFFFull : r);
    }
    __syncwarp();
  }
}

struct InCount32 {
  const uint32_t *p;
  __device__ uint64_t operator()(uint64_t i) const { return p[i]; }
};

// ---------------------------------------------------------------- windows

// For each overflowing leaf: the smallest aligned window whose density after
// the update is within bound; marks[(h, idx)] = 1.  Sets *grow when even the
// root is too dense.
__global__ void k_pma_windows(const uint32_t *__restrict__ rcount, const uint64_t *__restrict__ rpre,
                              uint64_t NL, int H, uint8_t *marks, unsigned int *grow, unsigned int *any) {
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < NL;
       j += (uint64_t)gridDim.x * blockDim.x) {
    if (rcount[j] <= kLeaf) continue;
    atomicOr(any, 1u);
    bool found = false;
    for (int h = 1; h <= H; h++) {
      uint64_t a = (j >> h) << h, e = a + (1ull << h);
      if (e > NL) e = NL;
      double tot = (double)(rpre[e] - rpre[a]);
      if (tot <= upper_bound_density(h, H) * (double)(e - a) * kLeaf) {
        // level h occupies marks[(2^h-ish) offset]: index by level base = h*NL
        marks[(uint64_t)h * NL + (j >> h)] = 1;
        found = true;
        break;
      }
    }
    if (!found) atomicOr(grow, 1u);
  }
}

// Window of every leaf: the highest marked ancestor; code = h << 27 | start
// leaf index is recovered from j and h.
__global__ void k_pma_cover(const uint8_t *__restrict__ marks, uint64_t NL, int H, uint32_t *win) {
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < NL;
       j += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t code = kNoWin;
    for (int h = H; h >= 1; h--)
      if (marks[(uint64_t)h * NL + (j >> h)]) {
        code = (uint32_t)h;
        break;
      }
    win[j] = code;
  }
}

// ---------------------------------------------------------------- merge

// One warp per leaf with work.  Leaf A (<= kLeaf keys) and, when it has at
// most kSegCap keys, batch segment B are staged in the warp's shared memory
// (longer segments are read from global memory).  Every output position comes
// from ranks, no serial merge:
//   insert: pos(A[i]) = i + lb_B(A[i]) - PA[i]
//           pos(B[k]) = k - PA[lb_A(B[k])] + lb_A(B[k])   for B[k] not in A
//           (PA[i] = number of A[0..i) also present in B)
//   remove: pos(A[i]) = i - PA[i] for A[i] not in B
// Lane l owns A[16l .. 16l+16): one binary search in B gives lb_B and the
// presence bit, a warp scan of the presence counts gives PA.  Output goes in
// place (leaf not in a window) or to staging[rpre[leaf]...].
constexpr uint32_t kSegCap = 256;
constexpr int kMergeWarps = 4;
constexpr int kOwn = kLeaf / 32;

__global__ void __launch_bounds__(32 * kMergeWarps) k_pma_merge(uint32_t *src, uint32_t *dst, uint32_t *cnt,
                                                               uint64_t NL, const uint64_t *__restrict__ keys,
                                                               const uint64_t *__restrict__ bstart,
                                                               const uint32_t *__restrict__ win,
                                                               const uint64_t *__restrict__ rpre,
                                                               uint64_t *staging, int insert, int all_windowed) {
  __shared__ uint64_t As[kMergeWarps][kLeaf];
  __shared__ uint64_t Bsh[kMergeWarps][kSegCap];
  __shared__ uint32_t PAs[kMergeWarps][kLeaf + 1];
  const unsigned w = threadIdx.x >> 5, lane = lane_id();
  uint64_t *A = As[w];
  uint32_t *PA = PAs[w];
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t j = gw; j < NL; j += nw) {
    const uint64_t b0 = bstart[j], b1 = bstart[j + 1];
    const bool windowed = all_windowed || win[j] != kNoWin;
    if (b0 == b1 && !windowed) continue;
    const uint32_t c = cnt[j];
    const uint64_t nb = b1 - b0;
    const bool bsm = nb <= kSegCap;
    const uint64_t *B = bsm ? Bsh[w] : keys + b0;
    const uint64_t base = j * kLeaf;
    for (uint32_t e = lane; e < c; e += 32) A[e] = slot_key(src, dst, base + e);
    if (bsm)
      for (uint32_t k = lane; k < nb; k += 32) Bsh[w][k] = keys[b0 + k];
    __syncwarp();
    uint32_t lb[kOwn];
    uint32_t hits = 0;
#pragma unroll
    for (int q = 0; q < kOwn; q++) {
      const uint32_t i = lane * kOwn + q;
      lb[q] = 0;
      if (i < c) {
        const uint64_t x = A[i];
        uint64_t lo = 0, hi = nb;
        while (lo < hi) {
          const uint64_t mid = (lo + hi) >> 1;
          if (B[mid] < x) lo = mid + 1; else hi = mid;
        }
        lb[q] = (uint32_t)lo;
        if (lo < nb && B[lo] == x) hits |= 1u << q;
      }
    }
    const uint32_t mine = __popc(hits);
    const uint32_t incl = warp_inclusive_scan(mine);
    const uint32_t tot = __shfl_sync(kFull, incl, 31);
    uint32_t run = incl - mine;
#pragma unroll
    for (int q = 0; q < kOwn; q++) {
      PA[lane * kOwn + q] = run;
      run += (hits >> q) & 1u;
    }
    if (lane == 31) PA[kLeaf] = tot;
    __syncwarp();
    const uint64_t r = insert ? (uint64_t)c + nb - tot : (uint64_t)c - tot;
    uint64_t *ostage = windowed ? staging + rpre[j] : nullptr;
    auto put = [&](uint64_t pos, uint64_t key) {
      if (ostage) {
        ostage[pos] = key;
      } else {
        src[base + pos] = (uint32_t)(key >> 32);
        dst[base + pos] = (uint32_t)key;
      }
    };
    // A elements (each lane its own run: positions increase along it)
#pragma unroll
    for (int q = 0; q < kOwn; q++) {
      const uint32_t i = lane * kOwn + q;
      if (i < c) {
        const uint32_t pa = PA[i];
        if (insert) put(i + lb[q] - pa, A[i]);
        else if (!((hits >> q) & 1u)) put(i - pa, A[i]);
      }
    }
    if (insert) {
      for (uint64_t k = lane; k < nb; k += 32) {
        const uint64_t x = B[k];
        uint32_t lo = 0, hi = c;  // lb_A(x)
        while (lo < hi) {
          const uint32_t mid = (lo + hi) >> 1;
          if (A[mid] < x) lo = mid + 1; else hi = mid;
        }
        if (lo < c && A[lo] == x) continue;  // already present
        put(k - PA[lo] + lo, x);
      }
    }
    if (!windowed) {
      for (uint64_t p = r + lane; p < c; p += 32) {
        src[base + p] = kSentinel;
        dst[base + p] = kSentinel;
      }
      if (lane == 0) cnt[j] = (uint32_t)r;
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- view refresh after a small merge
//
// After an in-place merge of the segment list, off[v] changes only for the
// vertices v whose key (v, 0) routes to a merged leaf j, i.e. v in
// [ceil(sep[j] / 2^32), ceil(sep[j+1] / 2^32)).  Of those, only v in
// (min(s0, L), U] can change, where s0 is the smallest src of the batch keys
// merged into j, L the smaller and U the larger of the leaf's last src before
// and after the merge (U also >= the largest batch src): below that the
// prefix counts are unchanged, above it every vertex starts at the next leaf
// either way.  The merging warp refreshes that range itself, up to
// kViewWarpMax vertices, as a merge of the vertex sequence [a, e) with the
// leaf's src list (staged in shared memory), each lane taking one diagonal
// band of the merge path, so that off[v] = the leaf position of the first key
// with src >= v.  A longer range (a key for a vertex far past the leaf's last
// key moves every vertex between them) is cut into chunks of kViewChunk
// vertices that k_pma_view_chunks fills with the whole grid.
constexpr uint32_t kViewChunk = 1024, kViewThreads = 256, kViewWarpMax = 1u << 10;

__device__ __forceinline__ uint64_t ceil_src(uint64_t key) { return (key >> 32) + ((key & 0xFFFFFFFFull) != 0); }

// The offsets of vertices [a, e) of leaf j (c keys, src list ls): a warp
// stages the src list in Y and fills the range as a merge of the vertex
// sequence with it, each lane taking one diagonal band of the merge path.
// off[v] = the leaf position of the first key with src >= v, or the next
// leaf's start when there is none.
__device__ __forceinline__ void leaf_fill_warp(const uint32_t *ls, uint32_t c, uint64_t a, uint64_t e, uint64_t j,
                                               uint32_t *Y, uint64_t *off) {
  const unsigned lane = lane_id();
  for (uint32_t i = lane; i < c; i += 32) Y[i] = ls[i];
  __syncwarp();
  // keys with src in [a, e): positions [p0, p1)
  uint32_t p0 = 0, p1 = c;
  {
    uint32_t hi = c;
    while (p0 < hi) {
      const uint32_t mid = (p0 + hi) >> 1;
      if (Y[mid] < a) p0 = mid + 1; else hi = mid;
    }
    uint32_t lo = p0;
    while (lo < p1) {
      const uint32_t mid = (lo + p1) >> 1;
      if (Y[mid] < e) lo = mid + 1; else p1 = mid;
    }
  }
  const uint32_t nx = (uint32_t)(e - a), ny = p1 - p0, T = nx + ny, per = (T + 31) / 32;
  const uint32_t d0 = lane * per < T ? lane * per : T, d1 = d0 + per < T ? d0 + per : T;
  // vertices among the first d0 merged (a vertex v goes before a key with src >= v)
  uint32_t lo = d0 > ny ? d0 - ny : 0, hi = d0 < nx ? d0 : nx;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a + mid <= Y[p0 + d0 - mid - 1]) lo = mid + 1; else hi = mid;
  }
  uint32_t i = lo, k = d0 - lo;
  const uint64_t base = j * kLeaf, next = (j + 1) * kLeaf;
  for (uint32_t d = d0; d < d1; d++) {
    if (i < nx && (k >= ny || a + i <= Y[p0 + k])) {
      const uint32_t pos = p0 + k;
      off[a + i] = pos < c ? base + pos : next;
      i++;
    } else {
      k++;
    }
  }
}

// The warp's part for merged leaf j (c keys now, old_last the src of its last
// key before the merge or 0xFFFFFFFF if it was empty) and segment q.
__device__ __forceinline__ void view_refresh_warp(const uint32_t *src, const uint64_t *__restrict__ sep, uint64_t NL,
                                                  uint64_t n, uint64_t j, uint32_t c, uint32_t old_last,
                                                  uint64_t smin, uint64_t smax, uint32_t *Y, uint64_t *off,
                                                  uint64_t q, uint64_t *vrange, uint64_t *chunks,
                                                  unsigned long long *nchunks) {
  const unsigned lane = lane_id();
  const uint32_t *ls = src + j * kLeaf;
  const uint64_t vlo = j == 0 ? 0 : min(ceil_src(sep[j]), n + 1);
  const uint64_t vhi = j + 1 == NL ? n + 1 : min(ceil_src(sep[j + 1]), n + 1);
  const bool had = old_last != 0xFFFFFFFFu, has = c != 0;
  const uint64_t new_last = has ? ls[c - 1] : 0;
  // L + 1 and U + 1 with "no keys" as vlo - 1
  const uint64_t l1 = !had || !has ? vlo : min((uint64_t)old_last, new_last) + 1;
  uint64_t u1 = smax + 1;
  if (had) u1 = max(u1, (uint64_t)old_last + 1);
  if (has) u1 = max(u1, new_last + 1);
  const uint64_t a = max(vlo, min(smin, l1)), e = max(a, min(vhi, u1));
  if (e - a > kViewWarpMax) {
    if (lane == 0) {
      vrange[2 * q] = a;
      vrange[2 * q + 1] = e;
      const uint64_t nch = (e - a + kViewChunk - 1) / kViewChunk;
      const uint64_t at = atomicAdd(nchunks, (unsigned long long)nch);
      for (uint64_t t = 0; t < nch; t++) chunks[at + t] = q << 32 | t;
    }
    return;
  }
  if (e == a) return;
  leaf_fill_warp(ls, c, a, e, j, Y, off);
}


// ---------------------------------------------------------------- optimistic merge
// One warp per leaf with a batch segment.  The leaf (A) and, when short, the
// segment (B) are staged in the warp's shared memory.  The result's size is
// counted first; then the merged sequence of A and B (ties: A first) is
// produced 32 positions per round, a lane per position found on the merge
// path, and the kept keys are packed by a ballot and written with
// consecutive stores.
//   insert keeps every A, and B[j] unless it equals the A element before it
//   or the B element before it (B may hold duplicates: it is sorted, not
//   deduplicated);
//   remove keeps A[i] unless it equals the B element it is compared with.
// When the result fits the leaf it is written in place; otherwise it goes to
// the overflow area (ovf) and the leaf is redistributed afterwards.
constexpr int kOptWarps = 6;
constexpr uint32_t kOptSeg = 256;

__device__ __forceinline__ uint64_t bval(const uint64_t *B, uint64_t j) { return B[j]; }

// The leaves with work come from a segment list (seg[2q] = leaf,
// seg[2q + 1] = b0 << 32 | b1, *nseg entries); the count after the merge goes
// to the high half of seg[2q].  When deg is given, every key that enters or
// leaves adjusts deg[src].  When off is given, a leaf merged in place also
// refreshes the view offsets around it (view_refresh_warp).  Batches of more
// keys than leaves take k_pma_merge_rank instead.
struct ViewOut {
  const uint64_t *sep;
  uint64_t n;
  uint64_t *off, *range, *chunks;
  unsigned long long *nchunks;
};

// One leaf (work item q) merged by the calling warp, with Aw / Bw its staging
// in shared memory (kLeaf and kOptSeg keys); returns the change of the leaf's
// key count.
__device__ __forceinline__ long long merge_leaf(uint64_t q, uint32_t *src, uint32_t *dst, uint32_t *cnt, uint64_t NL,
                                                const uint64_t *__restrict__ keys, uint64_t *seg, int insert,
                                                uint64_t *ovf,
                                                uint64_t *ovf_off, unsigned long long *ctr, uint32_t *deg,
                                                const ViewOut &view, uint64_t *Aw, uint64_t *Bw, uint64_t &tleaves,
                                                uint64_t &tentries) {
  const unsigned lane = lane_id();
  const uint64_t *A = Aw;
  {
    const uint64_t j = seg[2 * q] & 0xFFFFFFFFull;
    const uint64_t b0 = seg[2 * q + 1] >> 32, b1 = seg[2 * q + 1] & 0xFFFFFFFFull;
    const uint32_t c = cnt[j];
    // the leaf's last src before the merge, for the view refresh
    const uint32_t old_last = view.off && c ? src[j * kLeaf + c - 1] : 0xFFFFFFFFu;
    if (b0 == b1) {
      if (lane == 0) seg[2 * q] = j | (uint64_t)c << 32;
      return 0;
    }
    const uint64_t nb = b1 - b0;
    tleaves += 1;  // a leaf the merge rewrites, and the keys it held
    tentries += c;
    const uint64_t *B = nb <= kOptSeg ? Bw : keys + b0;
    const uint64_t base = j * kLeaf;
    // The s leaf keys below the first batch key keep their slots: the merge
    // reads and writes only the rest.  s by two rounds of lane-parallel
    // probes: every stride-th key, then the keys of the one stride that holds
    // the boundary.
    uint32_t s = 0;
    if (c) {
      const uint64_t first = keys[b0];
      const uint32_t stride = (c + 31) / 32;  // <= kLeaf / 32
      const uint32_t ps = lane * stride;
      const uint32_t t = __popc(__ballot_sync(kFull, ps < c && slot_key(src, dst, base + ps) < first));
      if (t) {
        const uint32_t p0 = (t - 1) * stride + 1, pe = t * stride < c ? t * stride : c;
        const uint32_t pp = p0 + lane;
        s = p0 + __popc(__ballot_sync(kFull, pp < pe && slot_key(src, dst, base + pp) < first));
      }
    }
    const uint32_t ca = c - s;  // the leaf keys that take part in the merge
    for (uint32_t e = lane; e < ca; e += 32) Aw[e] = slot_key(src, dst, base + s + e);
    if (nb <= kOptSeg)
      for (uint32_t k = lane; k < nb; k += 32) Bw[k] = keys[b0 + k];
    __syncwarp();
    // The result's size first: the batch keys that are dropped (insert: equal
    // to the key before them in B or present in A; remove: present in A,
    // counted once) by one binary search of each batch key in A.
    uint32_t drops = 0;
    for (uint32_t t = lane; t < nb; t += 32) {
      const uint64_t x = bval(B, t);
      const bool dup = t > 0 && bval(B, t - 1) == x;
      uint32_t l = 0, h = ca;
      while (l < h) {
        const uint32_t mid = (l + h) >> 1;
        if (A[mid] < x) l = mid + 1; else h = mid;
      }
      const bool found = l < ca && A[l] == x;
      drops += insert ? (dup || found) : (!dup && found);
    }
    drops = warp_sum(drops);
    const uint32_t r = s + (insert ? ca + (uint32_t)nb - drops : ca - drops);
    uint32_t *osrc = nullptr, *odst = nullptr;
    uint64_t *ostage = nullptr;
    if (r <= kLeaf) {
      osrc = src + base + s;
      odst = dst + base + s;
    } else {
      unsigned long long at = 0;
      if (lane == 0) {
        at = atomicAdd(&ctr[0], (unsigned long long)r);
        atomicAdd(&ctr[1], 1ull);
        ovf_off[j] = at;
      }
      at = __shfl_sync(kFull, at, 0);
      for (uint32_t e = lane; e < s; e += 32) ovf[at + e] = slot_key(src, dst, base + e);
      ostage = ovf + at + s;
    }
    // The merged sequence 32 positions at a time, a lane per position: the
    // lane finds its position's split (i A and k B keys before it) on the
    // merge path -- within 32 of its split one round earlier -- takes the
    // smaller head (A first on ties) and keeps it by the rule above; a ballot
    // then packs the kept keys, so the warp writes them with consecutive
    // stores.  A and B are in shared memory, so writing the leaf in place is
    // safe.
    const uint32_t T = ca + (uint32_t)nb, nb32 = (uint32_t)nb;
    uint32_t wpos = 0, split = 0;
    for (uint32_t c0 = 0; c0 < T; c0 += 32) {
      const uint32_t d = c0 + lane;
      bool kept = false;
      uint64_t x = 0;
      if (d < T) {
        uint32_t lo = d > nb32 ? d - nb32 : 0, hi = d < ca ? d : ca;
        lo = lo > split ? lo : split;
        hi = hi < split + 32 ? hi : split + 32;
        while (lo < hi) {
          const uint32_t mid = (lo + hi) >> 1;
          if (A[mid] <= bval(B, d - mid - 1)) lo = mid + 1; else hi = mid;
        }
        split = lo;
        const uint32_t i = lo, k = d - lo;
        const uint64_t a = i < ca ? A[i] : ~0ull, bk = k < nb32 ? bval(B, k) : ~0ull;
        const bool takeA = i < ca && a <= bk;
        x = takeA ? a : bk;
        const uint64_t lastA = i > 0 ? A[i - 1] : ~0ull, lastB = k > 0 ? bval(B, k - 1) : ~0ull;
        kept = insert ? (takeA || (x != lastA && x != lastB)) : (takeA && bk != a);
        if (deg && takeA != kept)  // a key left (A dropped) or entered (B kept)
          atomicAdd(deg + (x >> 32), takeA ? 0xFFFFFFFFu : 1u);
      }
      const unsigned m = __ballot_sync(kFull, kept);
      const uint32_t p = wpos + __popc(m & lanemask_lt());
      if (kept && s + p < r) {  // never past the counted size (the counts agree)
        if (ostage) {
          ostage[p] = x;
        } else {
          osrc[p] = (uint32_t)(x >> 32);
          odst[p] = (uint32_t)x;
        }
      }
      wpos += __popc(m);
    }
    if (!ostage) {
      for (uint32_t t = r + lane; t < c; t += 32) {
        src[base + t] = kSentinel;
        dst[base + t] = kSentinel;
      }
      if (lane == 0) cnt[j] = r;
    }
    if (lane == 0) seg[2 * q] = j | (uint64_t)r << 32;
    __syncwarp();  // the leaf's new contents (and A's last reads) are done warp-wide
    if (view.off && !ostage)
      view_refresh_warp(src, view.sep, NL, view.n, j, r, old_last, keys[b0] >> 32, keys[b1 - 1] >> 32,
                        reinterpret_cast<uint32_t *>(Aw), view.off, q, view.range, view.chunks, view.nchunks);
    __syncwarp();
    return (long long)r - (long long)c;
  }
}

__global__ void __launch_bounds__(32 * kOptWarps) k_pma_merge_opt(
    uint32_t *src, uint32_t *dst, uint32_t *cnt, uint64_t NL, const uint64_t *__restrict__ keys, uint64_t *seg,
    const unsigned long long *nseg, int insert, uint64_t *ovf, uint64_t *ovf_off,
    unsigned long long *ctr /* [0] overflow cursor, [1] leaves overflowed */, long long *delta, uint32_t *deg,
    ViewOut view) {
  __shared__ uint64_t As[kOptWarps][kLeaf];
  __shared__ uint64_t Bsh[kOptWarps][kOptSeg];
  const unsigned w = threadIdx.x >> 5;
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  long long dsum = 0;
  uint64_t tleaves = 0, tentries = 0;
  const uint64_t nwork = *nseg;
  for (uint64_t q = gw; q < nwork; q += nw)
    dsum += merge_leaf(q, src, dst, cnt, NL, keys, seg, insert, ovf, ovf_off, ctr, deg, view, As[w], Bsh[w], tleaves,
                       tentries);
  if (lane_id() == 0 && dsum) atomicAdd((unsigned long long *)delta, (unsigned long long)dsum);
  if (lane_id() == 0 && tleaves) {  // ctr[5], ctr[6]: touched leaves and the keys they held
    atomicAdd(&ctr[5], (unsigned long long)tleaves);
    atomicAdd(&ctr[6], (unsigned long long)tentries);
  }
}

// ---------------------------------------------------------------- rank merge (large batches)
// A warp per leaf with batch keys, every output position from ranks instead
// of the merge path: the leaf's keys staged in shared memory (A), each batch
// key ranked in A by a binary search (a key equal to its predecessor in the
// batch is skipped), and every element written straight to its slot:
//   insert: A[i] moves by the kept batch keys of rank <= i (a warp scan of D,
//           the kept keys per rank); kept key x of rank l lands at l + the
//           kept keys before it, written while ranking when the leaf cannot
//           overflow (c + batch keys <= kLeaf)
//   remove: A[i] moves back by the removed keys before it; the slots freed
//           at the end become gaps.
// A leaf whose result does not fit goes whole to the overflow area.
// ctr: [0] overflow cursor, [1] overflowing leaves, [5] leaves merged, [6]
// the keys they held; *delta the change of the key count.
constexpr int kRankWarps = 4;

struct RankOut {
  uint32_t *src, *dst;
  uint64_t base;
  uint64_t *ovf;  // non-null: the leaf overflows
};

__device__ __forceinline__ void rank_put(const RankOut &o, uint32_t pos, uint64_t k) {
  if (o.ovf) {
    o.ovf[pos] = k;
  } else {
    o.src[o.base + pos] = (uint32_t)(k >> 32);
    o.dst[o.base + pos] = (uint32_t)k;
  }
}

__device__ __forceinline__ uint32_t rank_of(const uint64_t *A, uint32_t c, uint64_t x) {
  uint32_t l = 0, hi = c;
  while (l < hi) {
    const uint32_t mid = (l + hi) >> 1;
    if (A[mid] < x) l = mid + 1;
    else hi = mid;
  }
  return l;
}

__global__ void __launch_bounds__(32 * kRankWarps, 8) k_pma_merge_rank(
    uint32_t *src, uint32_t *dst, uint32_t *cnt, uint64_t NL, const uint64_t *__restrict__ keys,
    const uint64_t *__restrict__ bstart, int insert, uint32_t *rcount, uint64_t *ovf, uint64_t *ovf_off,
    unsigned long long *ctr, long long *delta) {
  __shared__ uint64_t As[kRankWarps][kLeaf];
  __shared__ uint32_t Ds[kRankWarps][kLeaf + 1];
  const unsigned w = threadIdx.x >> 5, lane = lane_id();
  uint64_t *A = As[w];
  uint32_t *D = Ds[w];
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  long long dsum = 0;
  unsigned long long nleaves = 0, nentries = 0;
  // the next leaf's batch range and count are loaded while this one merges
  // (cnt[j] is written only by the warp that merges leaf j)
  uint64_t nb0 = 0, nb1 = 0;
  uint32_t ncnt = 0;
  if (gw < NL) {
    nb0 = bstart[gw];
    nb1 = bstart[gw + 1];
    ncnt = cnt[gw];
  }
  for (uint64_t j = gw; j < NL; j += nw) {
    const uint64_t b0 = nb0, b1 = nb1;
    const uint32_t c = min(ncnt, kLeaf);
    if (j + nw < NL) {
      nb0 = bstart[j + nw];
      nb1 = bstart[j + nw + 1];
      ncnt = cnt[j + nw];
    }
    if (b0 == b1) {
      if (lane == 0) rcount[j] = c;
      continue;
    }
    nleaves++;
    nentries += c;
    const uint64_t base = j * kLeaf;
    // the first round of batch keys is in flight with the leaf's loads
    uint64_t xn = b0 + lane < b1 ? keys[b0 + lane] : 0;
    for (uint32_t e0 = 0; e0 < c; e0 += 256) {  // eight loads of each array per lane in flight
      uint32_t hs[8], ds[8];
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const uint32_t e = e0 + 32 * u + lane;
        hs[u] = e < c ? src[base + e] : 0u;
        ds[u] = e < c ? dst[base + e] : 0u;
      }
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const uint32_t e = e0 + 32 * u + lane;
        if (e < c) A[e] = (uint64_t)hs[u] << 32 | ds[u];
      }
    }
    for (uint32_t i = lane; i <= c; i += 32) D[i] = 0;
    __syncwarp();
    RankOut o{src, dst, base, nullptr};
    const bool direct = insert && c + (b1 - b0) <= kLeaf;
    uint32_t changed = 0;
    uint64_t prev_last = 0;  // the previous round's last key
    for (uint64_t t0 = b0; t0 < b1; t0 += 32) {
      const uint64_t t = t0 + lane;
      bool act = false;
      uint32_t l = 0;
      const uint64_t x = xn;
      // the next round's key loads while this round ranks
      xn = t + 32 < b1 ? keys[t + 32] : 0;
      uint64_t before = __shfl_up_sync(kFull, x, 1);
      if (lane == 0) before = prev_last;
      prev_last = __shfl_sync(kFull, x, 31);
      if (t < b1) {
        if (!(t > b0 && before == x)) {
          l = rank_of(A, c, x);
          const bool present = l < c && A[l] == x;
          act = insert ? !present : present;
          if (act) {
            if (insert) atomicAdd(D + l, 1u);
            else D[l] = 1u;
          }
        }
      }
      const unsigned ma = __ballot_sync(kFull, act);
      if (direct && act) rank_put(o, l + changed + __popc(ma & lanemask_lt()), x);
      changed += __popc(ma);
    }
    __syncwarp();
    const uint32_t r = insert ? c + changed : c - changed;
    dsum += insert ? (long long)changed : -(long long)changed;
    if (r > kLeaf) {
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
        if (i < c) rank_put(o, i + inc, A[i]);
        carry = __shfl_sync(kFull, inc, 31);
      }
      if (!direct) {
        uint32_t kept_before = 0;
        for (uint64_t t0 = b0; t0 < b1; t0 += 32) {
          const uint64_t t = t0 + lane;
          bool keep = false;
          uint32_t l = 0;
          uint64_t x = 0;
          if (t < b1) {
            x = keys[t];
            if (!(t > b0 && keys[t - 1] == x)) {
              l = rank_of(A, c, x);
              keep = !(l < c && A[l] == x);
            }
          }
          const unsigned mk = __ballot_sync(kFull, keep);
          if (keep) rank_put(o, l + kept_before + __popc(mk & lanemask_lt()), x);
          kept_before += __popc(mk);
        }
      }
    } else {
      uint32_t removed = 0;
      for (uint32_t i0 = 0; i0 < c; i0 += 32) {
        const uint32_t i = i0 + lane;
        const bool gone = i < c && D[i];
        const unsigned mg = __ballot_sync(kFull, gone);
        if (i < c && !gone) rank_put(o, i - removed - __popc(mg & lanemask_lt()), A[i]);
        removed += __popc(mg);
      }
    }
    if (!o.ovf) {
      for (uint32_t i = r + lane; i < c; i += 32) {
        src[base + i] = kSentinel;
        dst[base + i] = kSentinel;
      }
      if (lane == 0) cnt[j] = r;
    }
    if (lane == 0) rcount[j] = r;
    __syncwarp();
  }
  if (lane == 0) {
    if (dsum) atomicAdd((unsigned long long *)delta, (unsigned long long)dsum);
    if (nleaves) {
      atomicAdd(&ctr[5], nleaves);
      atomicAdd(&ctr[6], nentries);
    }
  }
}

// Copies the current contents of every leaf in a window (all leaves when
// `all`) to staging[rpre[leaf] ...]: from the overflow area for a leaf that
// overflowed, from the leaf itself otherwise.
__global__ void k_pma_gather(const uint32_t *__restrict__ src, const uint32_t *__restrict__ dst,
                             const uint32_t *__restrict__ rcount, const uint32_t *__restrict__ cnt, uint64_t NL,
                             const uint32_t *__restrict__ win, int all, const uint64_t *__restrict__ rpre,
                             const uint64_t *__restrict__ ovf, const uint64_t *__restrict__ ovf_off,
                             uint64_t *staging) {
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t j = gw; j < NL; j += nw) {
    if (!all && win[j] == kNoWin) continue;
    const uint32_t r = rcount[j];
    uint64_t *out = staging + rpre[j];
    if (r > kLeaf || r != cnt[j]) {  // overflowed: its merge result is in ovf
      const uint64_t *in = ovf + ovf_off[j];
      for (uint32_t e = lane_id(); e < r; e += 32) out[e] = in[e];
    } else {
      for (uint32_t e = lane_id(); e < r; e += 32) out[e] = slot_key(src, dst, j * kLeaf + e);
    }
  }
}

// One CTA per leaf of a window: its even share of the window's staged
// elements.  The window of leaf j starts at a = (j >> h) << h (or 0 for the
// whole-array rebuild); elements [rpre[a], rpre[e]) are in staging at the same
// offsets.  Destination arrays may be new ones (grow / shrink).
__global__ void __launch_bounds__(kPmaBlock) k_pma_spread(const uint64_t *__restrict__ staging,
                                                         const uint64_t *__restrict__ rpre,
                                                         const uint32_t *__restrict__ win, uint64_t NL_src,
                                                         uint32_t *dsrc, uint32_t *ddst, uint32_t *dcnt,
                                                         uint64_t *dsep, uint64_t NL_dst, int all,
                                                         const uint64_t *__restrict__ old_sep) {
  for (uint64_t j = blockIdx.x; j < NL_dst; j += gridDim.x) {
    uint64_t a, e, s0, T, k, width;
    if (all) {
      a = 0;
      e = NL_dst;
      s0 = 0;
      T = rpre[NL_src];
    } else {
      const uint32_t h = win[j];
      if (h == kNoWin) continue;
      a = (j >> h) << h;
      e = a + (1ull << h);
      if (e > NL_dst) e = NL_dst;
      s0 = rpre[a];
      T = rpre[e] - s0;
    }
    width = e - a;
    k = j - a;
    const uint64_t lo = (T * k) / width, hi = (T * (k + 1)) / width;
    const uint64_t base = j * kLeaf;
    for (uint64_t p = threadIdx.x; p < kLeaf; p += kPmaBlock) {
      if (lo + p < hi) {
        const uint64_t key = staging[s0 + lo + p];
        dsrc[base + p] = (uint32_t)(key >> 32);
        ddst[base + p] = (uint32_t)key;
      } else {
        dsrc[base + p] = kSentinel;
        ddst[base + p] = kSentinel;
      }
    }
    if (threadIdx.x == 0) {
      dcnt[j] = (uint32_t)(hi - lo);
      if (k == 0) {
        if (all) dsep[j] = 0;  // window start keeps its separator otherwise
      } else if (hi > lo) {
        dsep[j] = staging[s0 + lo];
      } else {
        // empty leaf: route nothing here; take the next separator
        uint64_t nxt = ~0ull;
        if (hi < T) nxt = staging[s0 + hi];
        else if (!all && e < NL_src) nxt = old_sep[e];
        dsep[j] = nxt;
      }
    }
  }
}

// ---------------------------------------------------------------- graph view

__global__ void k_pma_deg(const uint64_t *__restrict__ elem, uint64_t n, uint32_t *deg) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    deg[v] = (uint32_t)(elem[v + 1] - elem[v]);
}

// export: element e of leaf i -> out[epre[i] + e]
__global__ void k_pma_export(const uint32_t *__restrict__ src, const uint32_t *__restrict__ dst,
                             const uint32_t *__restrict__ cnt, const uint64_t *__restrict__ epre, uint64_t NL,
                             uint64_t *out) {
  for (uint64_t i = blockIdx.x; i < NL; i += gridDim.x) {
    const uint32_t c = cnt[i];
    for (uint32_t e = threadIdx.x; e < c; e += blockDim.x) out[epre[i] + e] = slot_key(src, dst, i * kLeaf + e);
  }
}

// Leaves with work for a small sorted batch: key q starts a segment when it
// routes to another leaf than key q-1; the segment ends at the first key >=
// sep[leaf + 1].  seg[2s] = leaf, seg[2s + 1] = b0 << 32 | b1 (b < 2^32).
// With `bounds` set (a batch not yet validated on the host), a batch with a
// src or dst >= n or flagged unsorted yields no segments, so the merge after
// it changes nothing and the host reports the error once it reads the flags.
// The segment list, warps striding over the keys (first key tid0 & ~31,
// stride `stride` threads).
__device__ __forceinline__ void segments_range(const uint64_t *__restrict__ sep, uint64_t NL,
                                               const uint64_t *__restrict__ keys, uint64_t b, uint64_t *seg,
                                               unsigned long long *nseg, uint64_t tid0, uint64_t stride) {
  const unsigned lane = lane_id();
  for (uint64_t base = tid0 & ~31ull; base < b; base += stride) {
    const uint64_t q = base + lane;
    // the leaf of key q, and lane 0 also that of key base - 1, in one search
    // loop whose trip count depends only on NL (the two searches overlap)
    const uint64_t kq = q < b ? keys[q] : ~0ull;
    const uint64_t kp = lane == 0 && base > 0 ? keys[base - 1] : 0;
    uint64_t lo = 0, lp = 0, len = NL;
    while (len > 1) {
      const uint64_t half = len >> 1;
      if (sep[lo + half] <= kq) lo += half;
      if (lane == 0 && sep[lp + half] <= kp) lp += half;
      len -= half;
    }
    const uint64_t j = lo;
    uint64_t jprev = __shfl_up_sync(kFull, j, 1);
    if (lane == 0) jprev = base > 0 ? lp : ~0ull;
    const bool start = q < b && j != jprev;
    // a segment ends at the next start in the warp, else past the warp
    const unsigned starts = __ballot_sync(kFull, start);
    const unsigned later = lane == 31 ? 0u : starts >> (lane + 1) << (lane + 1);
    uint64_t b1 = b;  // also when j is the last leaf
    if (start && later) {
      b1 = base + (uint64_t)__ffs(later) - 1;
    } else if (start && base + 32 < b && j + 1 < NL) {
      const uint64_t lim = sep[j + 1];
      uint64_t l = base + 32, h = b;
      while (l < h) {
        const uint64_t mid = (l + h) >> 1;
        if (keys[mid] < lim) l = mid + 1; else h = mid;
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

__global__ void k_pma_segments(const uint64_t *__restrict__ sep, uint64_t NL, const uint64_t *__restrict__ keys,
                               uint64_t b, uint64_t *seg, unsigned long long *nseg,
                               const unsigned long long *bounds, uint64_t n, const unsigned int *unsorted) {
  if (bounds && (bounds[0] >= n || bounds[1] >= n || *unsorted)) return;
  segments_range(sep, NL, keys, b, seg, nseg, blockIdx.x * (uint64_t)blockDim.x + threadIdx.x,
                 (uint64_t)gridDim.x * blockDim.x);
}

// One block of 1024 threads sorts up to kSmallSort keys (a bitonic network
// over P = 1024 K keys, padded with ~0) and reports the largest src and dst
// in bounds[0], bounds[1].  The keys live in registers: lane l of warp w holds
// keys w*32K + 32k + l (k < K).  Compare-exchanges over a stride below 32 are
// lane shuffles, strides from 32 to 32K - 1 pair registers of one thread, and
// only the strides that cross warps go through shared memory.
constexpr uint32_t kSmallSort = 4096;

template <int K, int M>
__device__ __forceinline__ void sort_regs_cx(uint64_t (&x)[K], uint32_t ibase, uint32_t size) {
#pragma unroll
  for (int k = 0; k < K; k++) {
    if ((k & M) == 0 && (k | M) < K) {
      const bool up = ((ibase + 32u * k) & size) == 0;
      const uint64_t a = x[k], b = x[k | M];
      const bool sw = (a > b) == up;
      x[k] = sw ? b : a;
      x[k | M] = sw ? a : b;
    }
  }
}

// The sort by a block of 1024 threads with s (1024 K keys) and red (64 words)
// in shared memory.
template <int K>
__device__ __forceinline__ void sort_small_block(const uint64_t *__restrict__ in, uint32_t count, uint64_t *out,
                                                 unsigned long long *bounds, uint64_t *s, uint64_t (*red)[32]) {
  constexpr uint32_t P = 1024u * K, kWarpSpan = 32u * K;
  const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
  const uint32_t ibase = w * kWarpSpan + lane;
  uint64_t x[K];
  uint64_t ms = 0, md = 0;
#pragma unroll
  for (int k = 0; k < K; k++) {
    const uint32_t i = ibase + 32u * k;
    x[k] = i < count ? in[i] : ~0ull;
    if (i < count) {
      ms = ms > (x[k] >> 32) ? ms : (x[k] >> 32);
      md = md > (x[k] & 0xFFFFFFFFull) ? md : (x[k] & 0xFFFFFFFFull);
    }
  }
  for (uint32_t size = 2; size <= P; size <<= 1) {
    uint32_t stride = size >> 1;
    if (stride >= kWarpSpan) {
      __syncthreads();  // every warp has read back the previous round
#pragma unroll
      for (int k = 0; k < K; k++) s[ibase + 32u * k] = x[k];
      __syncthreads();
      for (; stride >= kWarpSpan; stride >>= 1) {
        for (uint32_t t = threadIdx.x; t < P / 2; t += blockDim.x) {
          const uint32_t i = 2 * t - (t & (stride - 1)), j = i + stride;
          const bool up = (i & size) == 0;
          const uint64_t a = s[i], b = s[j];
          if ((a > b) == up) {
            s[i] = b;
            s[j] = a;
          }
        }
        __syncthreads();
      }
#pragma unroll
      for (int k = 0; k < K; k++) x[k] = s[ibase + 32u * k];
    }
    for (; stride >= 32; stride >>= 1) {
      if (stride == 32) sort_regs_cx<K, 1>(x, ibase, size);
      else sort_regs_cx<K, 2>(x, ibase, size);  // stride 64 < kWarpSpan: K == 4
    }
    for (; stride > 0; stride >>= 1) {
      const bool lower = (lane & stride) == 0;
#pragma unroll
      for (int k = 0; k < K; k++) {
        const uint64_t y = __shfl_xor_sync(kFull, x[k], stride);
        const bool up = ((ibase + 32u * k) & size) == 0;
        const bool take_min = lower == up;
        x[k] = take_min ? (x[k] < y ? x[k] : y) : (x[k] < y ? y : x[k]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < K; k++) {
    const uint32_t i = ibase + 32u * k;
    if (i < count) out[i] = x[k];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const uint64_t a = __shfl_xor_sync(kFull, ms, o), b = __shfl_xor_sync(kFull, md, o);
    ms = ms > a ? ms : a;
    md = md > b ? md : b;
  }
  if (lane == 0) {
    red[0][w] = ms;
    red[1][w] = md;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (uint32_t v = 1; v < 32; v++) {
      ms = ms > red[0][v] ? ms : red[0][v];
      md = md > red[1][v] ? md : red[1][v];
    }
    bounds[0] = ms;
    bounds[1] = md;
  }
}

template <int K>
__global__ void __launch_bounds__(1024) k_sort_small(const uint64_t *__restrict__ in, uint32_t count, uint64_t *out,
                                                     unsigned long long *bounds) {
  __shared__ uint64_t s[1024u * K];
  __shared__ uint64_t red[2][32];
  sort_small_block<K>(in, count, out, bounds, s, red);
}

uint64_t sort_small_max() { return kSmallSort; }

int sort_small_keys(byo_ctx *ctx, const uint64_t *in, uint64_t count, uint64_t *out, unsigned long long *bounds) {
  if (count > kSmallSort) return set_error(ctx, BYO_EINVAL, "small sort: more than 4096 keys");
  if (count <= 1024)
    launch(ctx, k_sort_small<1>, dim3(1), dim3(1024), 0, in, (uint32_t)count, out, bounds);
  else if (count <= 2048)
    launch(ctx, k_sort_small<2>, dim3(1), dim3(1024), 0, in, (uint32_t)count, out, bounds);
  else
    launch(ctx, k_sort_small<4>, dim3(1), dim3(1024), 0, in, (uint32_t)count, out, bounds);
  return BYO_OK;
}


// A block per chunk of a long range; the leaf's src list is staged in shared
// memory and each thread fills kViewChunk / kViewThreads vertices a block
// width apart, each by its own binary search.  Nothing to do when a leaf
// overflowed or the update shrinks: the windowed path rebuilds the whole view.
// seg null: chunk q is of leaf q (the full view, which also writes
// elem[v] = epre[leaf] + position); ctr null: no overflow check.
__global__ void __launch_bounds__(kViewThreads)
    k_pma_view_chunks(const uint32_t *__restrict__ src, const uint32_t *__restrict__ cnt,
                      const uint64_t *__restrict__ seg, const uint64_t *__restrict__ range,
                      const uint64_t *__restrict__ chunks, const unsigned long long *nchunks, uint64_t *off,
                      const unsigned long long *ctr, uint64_t m_before, double shrink_below,
                      const uint64_t *__restrict__ epre, uint64_t *elem) {
  __shared__ uint32_t Y[kLeaf];
  if (ctr && (ctr[1] || (double)((long long)m_before + (long long)ctr[2]) < shrink_below)) return;
  const uint64_t nc = *nchunks;
  constexpr uint32_t kPer = kViewChunk / kViewThreads;
  for (uint64_t i = blockIdx.x; i < nc; i += gridDim.x) {
    const uint64_t ch = chunks[i];
    const uint64_t q = ch >> 32, t = ch & 0xFFFFFFFFull;
    const uint64_t j = seg ? seg[2 * q] & 0xFFFFFFFFull : q;
    const uint64_t e = range[2 * q + 1];
    const uint64_t v0 = range[2 * q] + t * kViewChunk + threadIdx.x;
    const uint32_t c = cnt[j];
    __syncthreads();  // the previous chunk's searches are done with Y
    for (uint32_t k = threadIdx.x; k < c; k += kViewThreads) Y[k] = src[j * kLeaf + k];
    __syncthreads();
#pragma unroll
    for (uint32_t k = 0; k < kPer; k++) {
      const uint64_t v = v0 + (uint64_t)k * kViewThreads;
      if (v >= e) break;
      uint32_t lo = 0, hi = c;
      while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (Y[mid] < v) lo = mid + 1; else hi = mid;
      }
      off[v] = lo < c ? j * kLeaf + lo : (j + 1) * kLeaf;
      if (elem) elem[v] = epre[j] + lo;
    }
  }
}

// The whole view: a warp per leaf fills its vertex range [ceil(sep[j] /
// 2^32), ceil(sep[j+1] / 2^32)) (the ranges of all leaves cover [0, n]),
// 32 vertices per round, a lane per vertex with a binary search in the leaf
// (its lines shared by the warp in L1) that starts where the lane's previous
// vertex ended; ranges above kViewWarpMax vertices go to the chunk list.
constexpr int kViewWarps = 8;
__global__ void __launch_bounds__(32 * kViewWarps)
    k_pma_view_leaves(const uint32_t *__restrict__ src, const uint32_t *__restrict__ cnt,
                      const uint64_t *__restrict__ sep, const uint64_t *__restrict__ epre, uint64_t NL, uint64_t n,
                      uint64_t *off, uint64_t *elem, uint64_t *range, uint64_t *chunks,
                      unsigned long long *nchunks) {
  const unsigned lane = lane_id();
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t j = gw; j < NL; j += nw) {
    const uint64_t vlo = j == 0 ? 0 : min(ceil_src(sep[j]), n + 1);
    const uint64_t vhi = j + 1 == NL ? n + 1 : min(ceil_src(sep[j + 1]), n + 1);
    if (vhi - vlo > kViewWarpMax) {
      if (lane == 0) {
        range[2 * j] = vlo;
        range[2 * j + 1] = vhi;
        const uint64_t nch = (vhi - vlo + kViewChunk - 1) / kViewChunk;
        const uint64_t at = atomicAdd(nchunks, (unsigned long long)nch);
        for (uint64_t t = 0; t < nch; t++) chunks[at + t] = j << 32 | t;
      }
      continue;
    }
    if (vhi == vlo) continue;
    const uint32_t c = cnt[j];
    const uint32_t *ls = src + j * kLeaf;
    const uint64_t eb = epre[j], base = j * kLeaf, next = (j + 1) * kLeaf;
    uint32_t from = 0;
    for (uint64_t v0 = vlo; v0 < vhi; v0 += 32) {
      const uint64_t v = v0 + lane;
      if (v >= vhi) break;
      uint32_t lo = from, hi = c;
      while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(ls + mid) < v) lo = mid + 1; else hi = mid;
      }
      from = lo;
      off[v] = lo < c ? base + lo : next;
      elem[v] = eb + lo;
    }
  }
}

// rcount after a list-mode merge: the counts of every leaf (copied from cnt
// beforehand), then the merged leaves' counts from the segment list.
__global__ void k_pma_seg_counts(const uint64_t *__restrict__ seg, const unsigned long long *nseg,
                                 uint32_t *rcount) {
  const uint64_t ns = *nseg;
  for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < ns; q += (uint64_t)gridDim.x * blockDim.x)
    rcount[seg[2 * q] & 0xFFFFFFFFull] = (uint32_t)(seg[2 * q] >> 32);
}

// One warp per leaf: its cnt keys (packed at the leaf's start) go to
// out[epre[leaf] ...].
__global__ void k_pma_compact(const uint32_t *__restrict__ dst, const uint32_t *__restrict__ cnt,
                              const uint64_t *__restrict__ epre, uint64_t NL, uint32_t *out) {
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t i = gw; i < NL; i += nw) {
    const uint32_t c = cnt[i];
    const uint64_t o = epre[i];
    // eight loads per lane in flight before the stores
    for (uint32_t e0 = lane_id(); e0 < c; e0 += 256) {
      uint32_t x[8];
#pragma unroll
      for (int q = 0; q < 8; q++)
        if (e0 + 32 * q < c) x[q] = __ldcs(dst + i * kLeaf + e0 + 32 * q);
#pragma unroll
      for (int q = 0; q < 8; q++)
        if (e0 + 32 * q < c) out[o + e0 + 32 * q] = x[q];
    }
  }
}

// ---------------------------------------------------------------- host side

static int pma_alloc(byo_ctx *ctx, uint64_t NL, uint32_t **src, uint32_t **dst, uint32_t **cnt, uint64_t **sep) {
  cudaError_t e;
  *src = *dst = *cnt = nullptr;
  *sep = nullptr;
  if ((e = cudaMalloc(src, NL * kLeaf * 4)) != cudaSuccess ||
      (e = cudaMalloc(dst, NL * kLeaf * 4)) != cudaSuccess || (e = cudaMalloc(cnt, NL * 4)) != cudaSuccess ||
      (e = cudaMalloc(sep, NL * 8)) != cudaSuccess) {
    cudaGetLastError();
    if (*src) cudaFree(*src);
    if (*dst) cudaFree(*dst);
    if (*cnt) cudaFree(*cnt);
    if (*sep) cudaFree(*sep);
    *src = *dst = *cnt = nullptr;
    *sep = nullptr;
    return set_error(ctx, BYO_ENOMEM, "pma arrays", e);
  }
  return BYO_OK;
}

static void pma_free_arrays(Pma *p) {
  if (p->src) cudaFree(p->src);
  if (p->dst) cudaFree(p->dst);
  if (p->cnt) cudaFree(p->cnt);
  if (p->sep) cudaFree(p->sep);
  p->src = p->dst = p->cnt = nullptr;
  p->sep = nullptr;
}

static int ceil_log2(uint64_t x) {
  int h = 0;
  while ((1ull << h) < x) h++;
  return h;
}

static uint64_t leaves_for(uint64_t m) {
  uint64_t NL = (uint64_t)std::ceil((double)m / (kBuildDensity * kLeaf));
  return NL < 1 ? 1 : NL;
}

// Recomputes the traversal view (off, deg, nslots) from the leaves, with no
// host synchronisation: m, the element count the leaves hold, is known to the
// caller, and the pass over long vertex ranges reads its chunk count on the
// device (it exits at once when there are none).
static int pma_view(byo_graph *g, uint64_t m) {
  byo_ctx *ctx = g->ctx;
  Pma *p = g->pma;
  uint64_t *epre = nullptr, *elem = nullptr;
  BYO_TRY(ensure(ctx, p->epre, (p->NL + 1) * 8));
  epre = (uint64_t *)p->epre.p;
  BYO_TRY(scan_u32_to_u64(ctx, p->cnt, p->NL, epre));
  BYO_TRY(ws(g, WS_SCAN, g->n + 2, &elem));
  BYO_TRY(ensure(ctx, p->vrange, 2 * p->NL * 8));
  BYO_TRY(ensure(ctx, p->vchunks, ((g->n + 1) / kViewChunk + p->NL + 1) * 8 + 8));
  unsigned long long *nch = reinterpret_cast<unsigned long long *>(p->vchunks.p);
  uint64_t *chunks = reinterpret_cast<uint64_t *>(p->vchunks.p) + 1;
  BYO_CU(ctx, cudaMemsetAsync(nch, 0, 8, ctx->stream));
  launch_t(ctx, "pma_view", k_pma_view_leaves, dim3(grid_for(ctx, p->NL * 32, 32 * kViewWarps, 8)), dim3(32 * kViewWarps), 0,
         (const uint32_t *)p->src, (const uint32_t *)p->cnt, (const uint64_t *)p->sep, (const uint64_t *)epre, p->NL,
         g->n, g->d_off, elem, (uint64_t *)p->vrange.p, chunks, nch);
  g->m = m;
  launch_t(ctx, "pma_view", k_pma_view_chunks, dim3(grid_for(ctx, (g->n + 1) / kViewChunk + 1, 1, 8)),
           dim3(kViewThreads), 0, (const uint32_t *)p->src, (const uint32_t *)p->cnt, (const uint64_t *)nullptr,
           (const uint64_t *)p->vrange.p, (const uint64_t *)chunks, (const unsigned long long *)nch, g->d_off,
           (const unsigned long long *)nullptr, (uint64_t)0, 0.0, (const uint64_t *)epre, elem);
  launch(ctx, k_pma_deg, dim3(grid_for(ctx, g->n, 256)), dim3(256), 0, (const uint64_t *)elem, g->n, g->d_deg);
  g->d_slots = p->dst;
  g->nslots = p->NL * kLeaf;
  return check_launch(ctx, "pma_view");
}

// Lays `m` sorted unique keys (device) evenly over NL new leaves.
static int pma_layout(byo_graph *g, const uint64_t *d_keys, uint64_t m, uint64_t NL) {
  byo_ctx *ctx = g->ctx;
  Pma *p = g->pma;
  uint32_t *s, *d, *c;
  uint64_t *sp;
  BYO_TRY(pma_alloc(ctx, NL, &s, &d, &c, &sp));
  // rpre for the "all" spread: only rpre[NL_src] = m is read
  uint64_t *rp = nullptr;
  BYO_TRY(ensure(ctx, p->rpre, 16));
  rp = (uint64_t *)p->rpre.p;
  BYO_CU(ctx, cudaMemcpyAsync(rp, &m, 8, cudaMemcpyHostToDevice, ctx->stream));
  launch(ctx, k_pma_spread, dim3(grid_for(ctx, NL, 1, 16)), dim3(kPmaBlock), 0, d_keys, (const uint64_t *)rp,
         (const uint32_t *)nullptr, (uint64_t)0, s, d, c, sp, NL, 1, (const uint64_t *)nullptr);
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  pma_free_arrays(p);
  p->src = s;
  p->dst = d;
  p->cnt = c;
  p->sep = sp;
  p->NL = NL;
  p->H = ceil_log2(NL);
  return pma_view(g, m);
}

int pma_build(byo_graph *g, const uint64_t *d_keys, uint64_t m) {
  Pma *p = new Pma();
  g->pma = p;
  return pma_layout(g, d_keys, m, leaves_for(m));
}

void pma_destroy(Pma *p) {
  if (!p) return;
  pma_free_arrays(p);
  for (DevBuf *b : {&p->keys_a, &p->keys_b, &p->bstart, &p->rcount, &p->rpre, &p->win, &p->marks, &p->staging,
                    &p->misc, &p->epre, &p->ovf, &p->ovf_off, &p->vrange, &p->vchunks})
    free_buf(*b);
  delete p;
}

int pma_export_keys(byo_graph *g, uint64_t *d_keys_out) {
  byo_ctx *ctx = g->ctx;
  Pma *p = g->pma;
  BYO_TRY(ensure(ctx, p->epre, (p->NL + 1) * 8));
  BYO_TRY(scan_u32_to_u64(ctx, p->cnt, p->NL, (uint64_t *)p->epre.p));
  launch(ctx, k_pma_export, dim3(grid_for(ctx, p->NL, 1, 16)), dim3(256), 0, (const uint32_t *)p->src,
         (const uint32_t *)p->dst, (const uint32_t *)p->cnt, (const uint64_t *)p->epre.p, p->NL, d_keys_out);
  return check_launch(ctx, "pma_export");
}

// Full rebuild: every leaf merged into staging, then laid out over NL_new
// leaves (grow, shrink, or the "rebuild" update strategy).
static int pma_rebuild(byo_graph *g, const uint64_t *keys, const uint64_t *bstart, const uint64_t *rpre,
                       uint64_t total, int insert) {
  byo_ctx *ctx = g->ctx;
  Pma *p = g->pma;
  BYO_TRY(ensure(ctx, p->staging, (total ? total : 1) * 8));
  uint64_t *stg = (uint64_t *)p->staging.p;
  launch_t(ctx, "pma_merge", k_pma_merge, dim3(grid_for(ctx, p->NL * 32, 32 * kMergeWarps, 6)),
           dim3(32 * kMergeWarps), 0, p->src, p->dst, p->cnt, p->NL, keys, bstart, (const uint32_t *)nullptr, rpre,
           stg, insert, 1);
  BYO_TRY(check_launch(ctx, "pma_rebuild merge"));
  p->rebuilds++;
  return pma_layout(g, stg, total, leaves_for(total));
}

int pma_compact(byo_graph *g, uint32_t *out) {
  byo_ctx *ctx = g->ctx;
  Pma *p = g->pma;
  BYO_TRY(ensure(ctx, p->epre, (p->NL + 1) * 8));
  uint64_t *epre = (uint64_t *)p->epre.p;
  BYO_TRY(scan_u32_to_u64(ctx, p->cnt, p->NL, epre));
  launch(ctx, k_pma_compact, dim3(grid_for(ctx, p->NL * 32, 256, 16)), dim3(256), 0, (const uint32_t *)p->dst,
         (const uint32_t *)p->cnt, (const uint64_t *)epre, p->NL, out);
  return check_launch(ctx, "pma_compact");
}

int traversal_view(byo_graph *g, byo_graph **out) {
  *out = g;
  if (!(g->container == BYO_CONTAINER_PMA && g->pma) && !(g->container == BYO_CONTAINER_VOS && g->vos) &&
      !(g->container == BYO_CONTAINER_PCSR && g->pcsr))
    return BYO_OK;
  byo_ctx *ctx = g->ctx;
  byo_graph *s = g->snap;
  if (!s) {
    s = new byo_graph();
    s->ctx = ctx;
    s->container = BYO_CONTAINER_CSR;
    g->snap = s;
  }
  s->tune = g->tune;
  if (s->d_off && s->n == g->n && g->snap_version == g->version) {
    *out = s;
    return BYO_OK;
  }
  if (!s->d_off || s->n != g->n) {
    if (s->d_off) cudaFree(s->d_off);
    s->d_off = nullptr;
    BYO_CU(ctx, cudaMalloc(&s->d_off, (g->n + 1) * 8));
  }
  if (!s->d_slots || s->slots_cap < g->m + 16) {
    if (s->d_slots) cudaFree(s->d_slots);
    s->d_slots = nullptr;
    s->slots_cap = 0;
    const uint64_t cap = g->m + g->m / 16 + 16;  // room for a few batches of growth
    BYO_CU(ctx, cudaMalloc(&s->d_slots, cap * 4));
    s->slots_cap = cap;
  }
  s->n = g->n;
  s->m = g->m;
  s->nslots = g->m;
  s->d_deg = g->d_deg;
  BYO_TRY(scan_u32_to_u64(ctx, g->d_deg, g->n, s->d_off));
  if (g->pma) BYO_TRY(pma_compact(g, s->d_slots));
  else if (g->pcsr) BYO_TRY(pcsr_compact(g, s->d_slots));
  else BYO_TRY(vos_compact(g, s->d_off, s->d_slots));
  g->snap_version = g->version;
  *out = s;
  return BYO_OK;
}

// After a merge that left overflowing leaves (or a remove that shrinks the
// array): rcount from the merge (for a segment-list merge, cnt with the merged
// leaves' counts from seg), then the windows over the counts are gathered and
// spread, or the whole array is rebuilt; the view is rebuilt either way.
static int pma_finish_windowed(byo_graph *g, bool list, const uint64_t *bstart, const unsigned long long *d_nseg,
                               uint64_t b, uint64_t total, bool shrink) {
  byo_ctx *ctx = g->ctx;
  Pma *p = g->pma;
  const uint64_t NL = p->NL;
  const double cap = (double)NL * kLeaf;
  BYO_TRY(ensure(ctx, p->rcount, NL * 4));
  BYO_TRY(ensure(ctx, p->rpre, (NL + 1) * 8));
  uint32_t *rcount = (uint32_t *)p->rcount.p;
  uint64_t *rpre = (uint64_t *)p->rpre.p;
  unsigned int *flags = (unsigned int *)((unsigned long long *)p->misc.p + 2);
  uint64_t *h = nullptr;
  BYO_TRY(pinned(ctx, 4096, (void **)&h));
  if (list) {
    BYO_CU(ctx, cudaMemcpyAsync(rcount, p->cnt, NL * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    launch(ctx, k_pma_seg_counts, dim3(grid_for(ctx, b, 256)), dim3(256), 0, (const uint64_t *)bstart,
           d_nseg, rcount);
  }
  BYO_TRY(scan_u32_to_u64(ctx, rcount, NL, rpre));
  BYO_TRY(ensure(ctx, p->win, NL * 4));
  uint32_t *win = (uint32_t *)p->win.p;
  bool rebuild = shrink || (double)total > kRootMax * cap;
  if (!rebuild) {
    BYO_TRY(ensure(ctx, p->marks, (uint64_t)(p->H + 1) * NL));
    uint8_t *marks = (uint8_t *)p->marks.p;
    BYO_CU(ctx, cudaMemsetAsync(marks, 0, (uint64_t)(p->H + 1) * NL, ctx->stream));
    BYO_CU(ctx, cudaMemsetAsync(flags + 1, 0, 8, ctx->stream));
    launch(ctx, k_pma_windows, dim3(grid_for(ctx, NL, 256)), dim3(256), 0, (const uint32_t *)rcount,
           (const uint64_t *)rpre, NL, p->H, marks, flags + 1, flags + 2);
    BYO_CU(ctx, cudaMemcpyAsync(h, flags, 16, cudaMemcpyDeviceToHost, ctx->stream));
    BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
    rebuild = ((const unsigned int *)h)[1] != 0;
    if (!rebuild) launch(ctx, k_pma_cover, dim3(grid_for(ctx, NL, 256)), dim3(256), 0, (const uint8_t *)marks, NL,
                         p->H, win);
  }
  BYO_TRY(ensure(ctx, p->staging, (total ? total : 1) * 8));
  uint64_t *stg = (uint64_t *)p->staging.p;
  launch(ctx, k_pma_gather, dim3(grid_for(ctx, NL * 32, 256, 16)), dim3(256), 0, (const uint32_t *)p->src,
         (const uint32_t *)p->dst, (const uint32_t *)rcount, (const uint32_t *)p->cnt, NL, (const uint32_t *)win,
         rebuild ? 1 : 0, (const uint64_t *)rpre, (const uint64_t *)p->ovf.p, (const uint64_t *)p->ovf_off.p, stg);
  BYO_TRY(check_launch(ctx, "pma_gather"));
  if (rebuild) {
    ctx->last_update_strategy = 1;
    p->rebuilds++;
    return pma_layout(g, stg, total, leaves_for(total));
  }
  p->windows++;
  launch_t(ctx, "pma_redistribute", k_pma_spread, dim3(grid_for(ctx, NL, 1, 16)), dim3(kPmaBlock), 0,
           (const uint64_t *)stg, (const uint64_t *)rpre, (const uint32_t *)win, NL, p->src, p->dst, p->cnt, p->sep,
           NL, 0, (const uint64_t *)p->sep);
  BYO_TRY(check_launch(ctx, "pma_update"));
  return pma_view(g, total);
}

uint64_t pma_leaf_slots() { return kLeaf; }

int pma_update(byo_graph *g, const uint64_t *d_keys_in, uint64_t count, int sorted, int insert,
               uint64_t *changed) {
  byo_ctx *ctx = g->ctx;
  Pma *p = g->pma;
  if (!p) return set_error(ctx, BYO_ENOTSUP, "not a PMA container");
  g->version++;  // any snapshot of the contents is stale from here on
  const uint64_t m_before = g->m;
  // 1. bounds and order checks, sort (duplicates kept: the merges skip them)
  BYO_TRY(ensure(ctx, p->keys_a, count * 8));
  BYO_TRY(ensure(ctx, p->keys_b, count * 8));
  BYO_TRY(ensure(ctx, p->misc, 128));
  uint64_t *ka = (uint64_t *)p->keys_a.p, *kb = (uint64_t *)p->keys_b.p;
  unsigned long long *bounds = (unsigned long long *)p->misc.p;
  unsigned int *flags = (unsigned int *)(bounds + 2);  // [0] unsorted, [1] grow, [2] any overflow, [4..] counters
  BYO_CU(ctx, cudaMemsetAsync(p->misc.p, 0, 128, ctx->stream));
  // the largest src and dst come from the one-block sort for a batch that
  // fits it, else from k_key_bounds; no sort indexes out of bounds by key, so
  // the checks can be read after the sort (or after the merge)
  const bool small_sort = !sorted && count <= kSmallSort;
  if (small_sort) {
    if (count <= 1024)
      launch(ctx, k_sort_small<1>, dim3(1), dim3(1024), 0, d_keys_in, (uint32_t)count, ka, bounds);
    else if (count <= 2048)
      launch(ctx, k_sort_small<2>, dim3(1), dim3(1024), 0, d_keys_in, (uint32_t)count, ka, bounds);
    else
      launch(ctx, k_sort_small<4>, dim3(1), dim3(1024), 0, d_keys_in, (uint32_t)count, ka, bounds);
  } else {
    launch(ctx, k_key_bounds, dim3(grid_for(ctx, count, 256)), dim3(256), 0, d_keys_in, count, bounds);
    if (sorted)
      launch(ctx, k_check_sorted, dim3(grid_for(ctx, count, 256)), dim3(256), 0, d_keys_in, count, flags);
  }
  uint64_t *h = nullptr;
  BYO_TRY(pinned(ctx, 4096, (void **)&h));
  // 2. strategy: in-place merge (default), rebuild when asked for or chosen by
  // the learned policy from the host-side features (batch size, m, slots,
  // sortedness, direction); capacity may still force a rebuild below.
  int strategy = 0;
  if (ctx->update_policy == BYO_UPDATE_REBUILD) strategy = 1;
  else if (ctx->update_policy == BYO_UPDATE_LEARNED)
    strategy = update_strategy(ctx, count, m_before, p->NL * kLeaf, sorted, insert);
  ctx->last_update_strategy = strategy;
  // A batch of at most one key per leaf takes the segment-list merge, which
  // visits only its own leaves and keeps the view current around them.  An
  // in-place merge (either kind) validates the batch on the device -- the
  // segment kernel, or the routing for the rank merge, drops an invalid batch,
  // and no sort indexes out of bounds by key -- and the result is checked
  // after the merge's synchronisation; the rebuild strategy checks it first.
  const bool list = count <= p->NL && count < (1ull << 32);
  const bool defer = strategy == 0;
  if (!defer) {
    BYO_CU(ctx, cudaMemcpyAsync(h, p->misc.p, 32, cudaMemcpyDeviceToHost, ctx->stream));
    BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
    if (h[0] >= g->n || h[1] >= g->n) return set_error(ctx, BYO_EINVAL, "update key with src or dst >= n");
    if (sorted && (((unsigned int *)(h + 2))[0])) return set_error(ctx, BYO_EINVAL, "sorted batch not increasing");
  }
  uint64_t *batch = nullptr;
  uint64_t b = count;
  if (sorted) {
    batch = const_cast<uint64_t *>(d_keys_in);
  } else if (small_sort) {
    batch = ka;
  } else {
    // sorted, duplicates kept: the optimistic merge drops them itself
    BYO_TRY(sort_bucketed(ctx, d_keys_in, count, g->n, ka, kb));
    batch = ka;
  }
  // bstart doubles as the segment list (two words per touched leaf) and rpre
  // as the merged leaves' view ranges (two words each)
  const uint64_t NL = p->NL;
  const uint64_t list_words = list ? 2 * std::min<uint64_t>(count, NL) + 2 : 0;
  BYO_TRY(ensure(ctx, p->bstart, std::max<uint64_t>(NL + 1, list_words) * 8));
  BYO_TRY(ensure(ctx, p->rcount, NL * 4));
  BYO_TRY(ensure(ctx, p->rpre, std::max<uint64_t>(NL + 1, list_words) * 8));
  uint64_t *bstart = (uint64_t *)p->bstart.p, *rpre = (uint64_t *)p->rpre.p;
  uint32_t *rcount = (uint32_t *)p->rcount.p;
  if (strategy == 1) {
    launch(ctx, k_pma_route, dim3(grid_for(ctx, NL + 1, 256)), dim3(256), 0, (const uint64_t *)p->sep, NL,
           (const uint64_t *)batch, b, bstart, (const unsigned long long *)nullptr, (uint64_t)0,
           (const unsigned int *)nullptr);
    if (!sorted) {  // the counting merge wants unique keys
      BYO_TRY(unique_u64(ctx, ka, count, 0, kb, &b));
      batch = kb;
      launch(ctx, k_pma_route, dim3(grid_for(ctx, NL + 1, 256)), dim3(256), 0, (const uint64_t *)p->sep, NL,
             (const uint64_t *)batch, b, bstart, (const unsigned long long *)nullptr, (uint64_t)0,
             (const unsigned int *)nullptr);
    }
    launch(ctx, k_pma_count, dim3(grid_for(ctx, NL * 32, 32 * kPmaWarps, 4)), dim3(32 * kPmaWarps), 0,
           (const uint32_t *)p->src, (const uint32_t *)p->dst, (const uint32_t *)p->cnt, NL,
           (const uint64_t *)batch, (const uint64_t *)bstart, insert, rcount);
    BYO_TRY(scan_u32_to_u64(ctx, rcount, NL, rpre));
    BYO_CU(ctx, cudaMemcpyAsync(h, rpre + NL, 8, cudaMemcpyDeviceToHost, ctx->stream));
    BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
    const uint64_t total = h[0];
    if (changed) *changed = insert ? total - m_before : m_before - total;
    g->upd = UpdateStats{b, insert ? total - m_before : m_before - total, NL, m_before, 1u};
    if (total == m_before) return BYO_OK;
    return pma_rebuild(g, batch, bstart, rpre, total, insert);
  }
  // 3. optimistic merge: leaves that fit are done in place.  A batch much
  // smaller than the leaf count visits only its own leaves (segment list),
  // keeps the degrees up to date in the merge, and refreshes the view only
  // around those leaves.
  BYO_TRY(ensure(ctx, p->ovf, (NL * kLeaf + b + 1) * 8));
  BYO_TRY(ensure(ctx, p->ovf_off, NL * 8));
  // counters, cleared with the rest of misc: [0] cursor, [1] overflowing
  // leaves, [2] delta, [3] segments, [4] view chunks, [5] leaves merged,
  // [6] keys those leaves held before the merge
  unsigned long long *ctr = (unsigned long long *)(flags + 4);
  const double cap = (double)NL * kLeaf;
  const double shrink_below = !insert && NL > 1 ? kRootMin * cap : -1.0;
  if (list) {
    uint64_t *seg = bstart;  // 2 * min(b, NL) + 2 words
    launch(ctx, k_pma_segments, dim3(grid_for(ctx, b, 256)), dim3(256), 0, (const uint64_t *)p->sep, NL,
           (const uint64_t *)batch, b, seg, ctr + 3, defer ? (const unsigned long long *)bounds : nullptr, g->n,
           (const unsigned int *)flags);
    // the merge refreshes the offsets around the leaves it merged in place:
    // ranges in rpre, chunks of long ranges in win (both free here)
    BYO_TRY(ensure(ctx, p->win, ((g->n + 1) / kViewChunk + b + 64) * 8));
    ViewOut view{(const uint64_t *)p->sep, g->n, g->d_off, rpre, (uint64_t *)p->win.p, ctr + 4};
    launch_t(ctx, "pma_merge", k_pma_merge_opt, dim3(grid_for(ctx, b * 32, 32 * kOptWarps, 6)),
             dim3(32 * kOptWarps), 0, p->src, p->dst, p->cnt, NL, (const uint64_t *)batch, seg,
             (const unsigned long long *)(ctr + 3), insert, (uint64_t *)p->ovf.p, (uint64_t *)p->ovf_off.p, ctr,
             (long long *)(ctr + 2), g->d_deg, view);
  } else {
    launch(ctx, k_pma_route, dim3(grid_for(ctx, NL + 1, 256)), dim3(256), 0, (const uint64_t *)p->sep, NL,
           (const uint64_t *)batch, b, bstart, defer ? (const unsigned long long *)bounds : nullptr, g->n,
           (const unsigned int *)flags);
    launch_t(ctx, "pma_merge", k_pma_merge_rank, dim3(grid_for(ctx, NL * 32, 32 * kRankWarps, 8)),
             dim3(32 * kRankWarps), 0, p->src, p->dst, p->cnt, NL, (const uint64_t *)batch,
             (const uint64_t *)bstart, insert, rcount, (uint64_t *)p->ovf.p, (uint64_t *)p->ovf_off.p, ctr,
             (long long *)(ctr + 2));
  }
  BYO_CU(ctx, cudaMemcpyAsync(h, p->misc.p, 88, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  if (defer) {
    if (h[0] >= g->n || h[1] >= g->n) return set_error(ctx, BYO_EINVAL, "update key with src or dst >= n");
    if (sorted && (((unsigned int *)(h + 2))[0])) return set_error(ctx, BYO_EINVAL, "sorted batch not increasing");
  }
  const uint64_t *hc = h + 4;  // the counters
  const uint64_t novf = hc[1];
  const long long delta = (long long)hc[2];
  const uint64_t total = (uint64_t)((long long)m_before + delta);
  if (changed) *changed = insert ? total - m_before : m_before - total;
  const bool shrink = (double)total < shrink_below;
  g->upd = UpdateStats{b, insert ? total - m_before : m_before - total, hc[5], hc[6],
                       (novf || shrink) ? 2u : 0u};
  if (novf == 0 && !shrink) {
    if (list) {
      // long ranges left by the merge (rare: keys far past a leaf's last key)
      const uint64_t nch = hc[4];
      if (nch)
        launch(ctx, k_pma_view_chunks, dim3(grid_for(ctx, nch, 1, 8)), dim3(kViewThreads), 0,
               (const uint32_t *)p->src, (const uint32_t *)p->cnt, (const uint64_t *)bstart,
               (const uint64_t *)rpre, (const uint64_t *)p->win.p, (const unsigned long long *)(ctr + 4), g->d_off,
               (const unsigned long long *)ctr, m_before, shrink_below, (const uint64_t *)nullptr,
               (uint64_t *)nullptr);
      g->m = total;
      return check_launch(ctx, "pma_update");
    }
    BYO_TRY(check_launch(ctx, "pma_update"));
    return pma_view(g, total);
  }
  // 4. overflow (or shrink): windows over the counts after the merge
  return pma_finish_windowed(g, list, bstart, (const unsigned long long *)(ctr + 3), b, total, shrink);
}

// ---------------------------------------------------------------- update stream
// A run of small batches (each <= kSmallSort keys and at most NL/2 of them, so
// that the segment-list merge applies) drained by one persistent cooperative
// kernel: per batch, CTA 0 sorts the keys in registers; the grid finds the
// segments, merges the leaves (refreshing the offsets around them), and fills
// long offset ranges, with a bounded grid barrier between the phases.  A batch
// whose merge overflows a leaf or shrinks the array stops the kernel after its
// merge; the host finishes that batch with the windowed path and relaunches
// from the next one.  A batch with a key >= n stops it before its merge.
// Query ops (the mixed stream) run a 64-source bit-lane BFS over the
// container's own slots between the batches, inside the same kernel and under
// the same barrier: the query state is cleared, the traversal runs
// (ms_bfs_body), the levels are written to the query's output, and CTA 0
// sorts the next batch.
constexpr int kStreamThreads = 1024, kStreamWarps = kStreamThreads / 32;
constexpr size_t kStreamSmem = (size_t)kStreamWarps * (kLeaf + kOptSeg) * 8;

struct StreamCtl {
  GridBar bar;
  unsigned long long bounds[2][2];
  unsigned long long ctr[2][6];  // per buffer: [0] overflow cursor [1] overflowing leaves [2] delta [3] segments
                                 // [4] view chunks
  long long m;                   // keys in the container
  unsigned int stop, reason;     // batch index + 1 where the kernel stopped; 1 overflow or shrink, 2 invalid keys,
                                 // 3 a query's hub chunk list overflowed
  unsigned long long t_prev;     // globaltimer at the end of the previous op (or the kernel's start)
};

constexpr unsigned char kOpQuery = 2;  // ops[b]: 0 remove, 1 insert, 2 query

// Batch b uses buffer b & 1 of the sorted keys, segment list, offset ranges
// and chunk list, so that the next batch can be sorted and its segments found
// while this one is merged and its long ranges filled.
struct StreamArgs {
  uint32_t *src, *dst, *cnt;
  const uint64_t *sep;
  uint64_t NL, n;
  uint64_t *off;
  uint32_t *deg;
  const uint64_t *keys, *boff;
  const unsigned char *ops;
  uint64_t first, nbatch;
  uint64_t *sorted, *seg, *vrange, *chunks, *ovf, *ovf_off;
  uint64_t chunk_words;  // per buffer
  double shrink_below;   // a remove that leaves fewer keys rebuilds the array
  long long *changed;
  StreamCtl *ctl;
  // queries (ops[b] == kOpQuery): op b runs the query described by
  // qargs[qnum[b]] (device memory: its sources, its levels output and the
  // shared work arrays and control block); op_ns[2b], op_ns[2b + 1]: op b's
  // start and end (globaltimer)
  const MsArgs *qargs;
  const uint32_t *qnum;
  unsigned long long *op_ns;
};

// One chunk of a long offset range, by the whole CTA (Y: the leaf's src list).
__device__ __forceinline__ void view_chunk_block(const uint32_t *__restrict__ src, const uint32_t *__restrict__ cnt,
                                                 const uint64_t *__restrict__ seg, const uint64_t *__restrict__ range,
                                                 uint64_t ch, uint64_t *off, uint32_t *Y) {
  const uint64_t q = ch >> 32, t = ch & 0xFFFFFFFFull;
  const uint64_t j = seg[2 * q] & 0xFFFFFFFFull;
  const uint64_t a = range[2 * q] + t * kViewChunk, e0 = range[2 * q + 1];
  const uint64_t e = a + kViewChunk < e0 ? a + kViewChunk : e0;
  const uint32_t c = cnt[j];
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < c; k += blockDim.x) Y[k] = src[j * kLeaf + k];
  __syncthreads();
  for (uint64_t v = a + threadIdx.x; v < e; v += blockDim.x) {
    uint32_t lo = 0, hi = c;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (Y[mid] < v) lo = mid + 1; else hi = mid;
    }
    off[v] = lo < c ? j * kLeaf + lo : (j + 1) * kLeaf;
  }
}

__device__ __forceinline__ void stream_sort(const StreamArgs &a, uint64_t bi, uint64_t *As) {
  StreamCtl *c = a.ctl;
  const int buf = (int)(bi & 1);
  if (threadIdx.x < 6) c->ctr[buf][threadIdx.x] = 0;
  const uint64_t k0 = a.boff[bi], count = a.boff[bi + 1] - k0;
  uint64_t *out = a.sorted + (size_t)buf * kSmallSort;
  uint64_t(*red)[32] = reinterpret_cast<uint64_t(*)[32]>(As + kSmallSort);
  if (count <= 1024) sort_small_block<1>(a.keys + k0, (uint32_t)count, out, c->bounds[buf], As, red);
  else if (count <= 2048) sort_small_block<2>(a.keys + k0, (uint32_t)count, out, c->bounds[buf], As, red);
  else sort_small_block<4>(a.keys + k0, (uint32_t)count, out, c->bounds[buf], As, red);
}

// Per batch bi, two phases between grid barriers:
//   1. the long offset ranges of batch bi-1 (its merge is done), and the
//      segments of batch bi (its keys were sorted during phase 2 of bi-1);
//   2. the merge of batch bi by CTAs 1.., while CTA 0 sorts batch bi+1.
__global__ void __launch_bounds__(kStreamThreads) k_pma_stream(StreamArgs a) {
  extern __shared__ unsigned long long stream_smem[];
  uint64_t *As = reinterpret_cast<uint64_t *>(stream_smem);  // [kStreamWarps][kLeaf]
  uint64_t *Bs = As + (size_t)kStreamWarps * kLeaf;           // [kStreamWarps][kOptSeg]
  StreamCtl *c = a.ctl;
  const unsigned nb = gridDim.x, w = threadIdx.x >> 5;
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, nthr = (uint64_t)gridDim.x * blockDim.x;
  // warps that merge: those of CTAs 1.. (all of them on a one-CTA grid)
  const bool solo = nb == 1;
  const uint64_t mw0 = solo ? 0 : 32, nmw = (nthr >> 5) - mw0, gw = (tid >> 5) - (solo ? 0 : 32);
  if (tid == 0) c->t_prev = globaltimer_ns();
  if (blockIdx.x == 0 && a.ops[a.first] != kOpQuery) stream_sort(a, a.first, As);
  if (!grid_sync(&c->bar, nb)) return;
  for (uint64_t bi = a.first;; bi++) {
    const int cur = (int)(bi & 1), prv = cur ^ 1;
    const bool has = bi < a.nbatch;
    const bool query = has && a.ops[bi] == kOpQuery;
    const bool valid = has && (query || (c->bounds[cur][0] < a.n && c->bounds[cur][1] < a.n));
    // phase 1
    if (bi > a.first) {
      const uint64_t nch = *(volatile unsigned long long *)&c->ctr[prv][4];
      const uint64_t *chk = a.chunks + (size_t)prv * a.chunk_words;
      for (uint64_t t = blockIdx.x; t < nch; t += gridDim.x)
        view_chunk_block(a.src, a.cnt, a.seg + (size_t)prv * 2 * kSmallSort,
                         a.vrange + (size_t)prv * 2 * kSmallSort, chk[t], a.off, reinterpret_cast<uint32_t *>(As));
      if (tid == 0) {
        const long long d = (long long)c->ctr[prv][2];
        a.changed[bi - 1] = d;
        c->m += d;
      }
    }
    const uint64_t count = has ? a.boff[bi + 1] - a.boff[bi] : 0;
    if (valid && !query)
      segments_range(a.sep, a.NL, a.sorted + (size_t)cur * kSmallSort, count,
                     a.seg + (size_t)cur * 2 * kSmallSort, &c->ctr[cur][3], tid, nthr);
    if (!grid_sync(&c->bar, nb)) return;
    if (!has) return;
    if (!valid) {
      if (tid == 0) {
        c->stop = (unsigned int)bi + 1;
        c->reason = 2;
      }
      return;
    }
    const bool next_update = bi + 1 < a.nbatch && a.ops[bi + 1] != kOpQuery;
    if (query) {
      // a 64-source BFS over the current contents
      const MsArgs &qa = a.qargs[a.qnum[bi]];
      MsCtl *qc = qa.ctl;
      if (blockIdx.x == 0)
        for (uint32_t i = threadIdx.x; i < sizeof(MsCtl) / 8; i += blockDim.x)
          reinterpret_cast<unsigned long long *>(qc)[i] = 0;
      if (!grid_sync(&c->bar, nb)) return;
      ms_bfs_body(qa, &c->bar);
      if (!grid_sync(&c->bar, nb)) return;  // the round count is visible to all
      ms_levels_body(qa, tid, nthr);
      if (blockIdx.x == 0 && next_update) stream_sort(a, bi + 1, As);
      if (tid == 0) {
        c->ctr[cur][2] = 0;  // a query changes nothing and leaves no ranges to fill
        c->ctr[cur][4] = 0;
        if (qc->bar.err & 2u) {
          c->stop = (unsigned int)bi + 1;
          c->reason = 3;
        }
      }
      if (!grid_sync(&c->bar, nb)) return;
      if (tid == 0 && a.op_ns) {
        const unsigned long long t = globaltimer_ns();
        a.op_ns[2 * bi] = c->t_prev;
        a.op_ns[2 * bi + 1] = t;
        c->t_prev = t;
      }
      if (*(volatile unsigned int *)&c->stop) return;
      continue;
    }
    // phase 2
    const int insert = a.ops[bi];
    if (!solo && blockIdx.x == 0) {
      if (next_update) stream_sort(a, bi + 1, As);
    } else {
      const ViewOut view{a.sep, a.n, a.off, a.vrange + (size_t)cur * 2 * kSmallSort,
                         a.chunks + (size_t)cur * a.chunk_words, &c->ctr[cur][4]};
      const uint64_t ns = *(volatile unsigned long long *)&c->ctr[cur][3];
      long long dsum = 0;
      uint64_t tleaves = 0, tentries = 0;  // not reported by the stream
      for (uint64_t q = gw; q < ns; q += nmw)
        dsum += merge_leaf(q, a.src, a.dst, a.cnt, a.NL, a.sorted + (size_t)cur * kSmallSort,
                           a.seg + (size_t)cur * 2 * kSmallSort, insert, a.ovf, a.ovf_off, c->ctr[cur], a.deg, view,
                           As + (size_t)w * kLeaf, Bs + (size_t)w * kOptSeg, tleaves, tentries);
      if (lane_id() == 0 && dsum) atomicAdd(&c->ctr[cur][2], (unsigned long long)dsum);
      if (solo) {
        __syncthreads();
        if (next_update) stream_sort(a, bi + 1, As);
      }
    }
    if (!grid_sync(&c->bar, nb)) return;
    if (tid == 0 && a.op_ns) {
      const unsigned long long t = globaltimer_ns();
      a.op_ns[2 * bi] = c->t_prev;
      a.op_ns[2 * bi + 1] = t;
      c->t_prev = t;
    }
    const long long total = c->m + (long long)*(volatile unsigned long long *)&c->ctr[cur][2];
    if (*(volatile unsigned long long *)&c->ctr[cur][1] || (!insert && (double)total < a.shrink_below)) {
      if (tid == 0) {
        c->stop = (unsigned int)bi + 1;
        c->reason = 1;
      }
      return;
    }
  }
}

int pma_update_stream(byo_graph *g, const uint64_t *d_keys, const uint64_t *d_boff, const uint64_t *h_boff,
                      const unsigned char *d_ops, const unsigned char *h_ops, uint64_t nbatch, long long *h_changed,
                      const StreamQueries *qs) {
  byo_ctx *ctx = g->ctx;
  Pma *p = g->pma;
  if (!p) return set_error(ctx, BYO_ENOTSUP, "not a PMA container");
  for (uint64_t bi = 0; bi < nbatch; bi++) h_changed[bi] = 0;
  if (!nbatch) return BYO_OK;
  g->version++;
  // queries: their numbering, sources, descriptors, shared control block and
  // per-op times, in one workspace
  std::vector<uint32_t> qnum(nbatch, 0);
  uint64_t nq = 0;
  for (uint64_t b = 0; b < nbatch; b++)
    if (h_ops[b] == kOpQuery) qnum[b] = (uint32_t)nq++;
  if (nq && !qs) return set_error(ctx, BYO_EINVAL, "update stream: query ops need sources");
  uint32_t *d_qnum = nullptr, *d_qsrcs = nullptr;
  MsArgs *d_qargs = nullptr;
  MsCtl *d_qctl = nullptr;
  unsigned long long *d_op_ns = nullptr;
  if (qs) {
    const size_t b_qnum = nbatch * 4, b_srcs = nq * qs->k * 4, b_args = nq * sizeof(MsArgs);
    const size_t o_srcs = (b_qnum + 15) & ~15ull, o_args = (o_srcs + b_srcs + 15) & ~15ull;
    const size_t o_ctl = (o_args + b_args + 15) & ~15ull, o_ns = (o_ctl + sizeof(MsCtl) + 15) & ~15ull;
    unsigned char *wsp = nullptr;
    BYO_TRY(ws(g, WS_STREAM_Q, o_ns + 16 * nbatch + 16, &wsp));
    d_qnum = reinterpret_cast<uint32_t *>(wsp);
    d_qsrcs = reinterpret_cast<uint32_t *>(wsp + o_srcs);
    d_qargs = reinterpret_cast<MsArgs *>(wsp + o_args);
    d_qctl = reinterpret_cast<MsCtl *>(wsp + o_ctl);
    d_op_ns = reinterpret_cast<unsigned long long *>(wsp + o_ns);
    BYO_CU(ctx, cudaMemcpyAsync(d_qnum, qnum.data(), b_qnum, cudaMemcpyHostToDevice, ctx->stream));
    if (nq) BYO_CU(ctx, cudaMemcpyAsync(d_qsrcs, qs->h_srcs, b_srcs, cudaMemcpyHostToDevice, ctx->stream));
    BYO_CU(ctx, cudaMemsetAsync(d_op_ns, 0, 16 * nbatch, ctx->stream));
    BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));  // qnum is read from host memory above
  }
  std::vector<MsArgs> qargs(nq);
  StreamCtl *c = nullptr;
  long long *d_changed = nullptr;
  BYO_TRY(ensure(ctx, p->misc, 128 + sizeof(StreamCtl) + 8 * nbatch));
  c = reinterpret_cast<StreamCtl *>((char *)p->misc.p + 128);
  d_changed = reinterpret_cast<long long *>(c + 1);
  BYO_CU(ctx, cudaFuncSetAttribute(k_pma_stream, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStreamSmem));
  int per_sm = 0;
  BYO_CU(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pma_stream, kStreamThreads, kStreamSmem));
  if (per_sm < 1) return set_error(ctx, BYO_EDEVICE, "update stream: persistent kernel cannot be resident");
  StreamCtl *hc = nullptr;
  BYO_TRY(pinned(ctx, std::max<size_t>(sizeof(StreamCtl), 4096), (void **)&hc));
  uint64_t bi = 0;
  while (bi < nbatch) {
    const uint64_t NL = p->NL;
    const uint64_t cnt_b = h_boff[bi + 1] - h_boff[bi];
    const bool query = h_ops[bi] == kOpQuery;
    if (cnt_b == 0 && !query) {
      bi++;
      continue;
    }
    if (!query && (cnt_b > kSmallSort || 2 * cnt_b > NL)) {  // not a small batch: the ordinary update
      uint64_t ch = 0;
      BYO_TRY(pma_update(g, d_keys + h_boff[bi], cnt_b, 0, h_ops[bi], &ch));
      h_changed[bi] = (long long)ch;
      bi++;
      continue;
    }
    // the run of small batches (and queries) from bi
    uint64_t be = bi;
    while (be < nbatch && (h_ops[be] == kOpQuery || (h_boff[be + 1] - h_boff[be] <= kSmallSort &&
                                                     2 * (h_boff[be + 1] - h_boff[be]) <= NL)))
      be++;
    if (nq) {  // the queries read the container's current slots
      MsArgs base = {};
      BYO_TRY(ms_args_setup(g, qs->k, &base));
      base.ctl = d_qctl;
      for (uint64_t q = 0; q < nq; q++) {
        qargs[q] = base;
        qargs[q].srcs = d_qsrcs + q * qs->k;
        qargs[q].levels = qs->d_levels + q * qs->k * g->n;
      }
      BYO_CU(ctx, cudaMemcpyAsync(d_qargs, qargs.data(), nq * sizeof(MsArgs), cudaMemcpyHostToDevice, ctx->stream));
    }
    const uint64_t chunk_words = (g->n + 1) / kViewChunk + kSmallSort + 64;
    BYO_TRY(ensure(ctx, p->keys_a, 2 * kSmallSort * 8));
    BYO_TRY(ensure(ctx, p->bstart, std::max<uint64_t>(NL + 1, 4 * kSmallSort) * 8));
    BYO_TRY(ensure(ctx, p->rpre, std::max<uint64_t>(NL + 1, 4 * kSmallSort) * 8));
    BYO_TRY(ensure(ctx, p->win, 2 * chunk_words * 8));
    BYO_TRY(ensure(ctx, p->ovf, (NL * kLeaf + kSmallSort + 1) * 8));
    BYO_TRY(ensure(ctx, p->ovf_off, NL * 8));
    std::memset(hc, 0, sizeof(StreamCtl));
    hc->m = (long long)g->m;
    hc->bar.limit_ms = ctx->bar_limit_ms;
    hc->bar.extra = ctx->bar_extra;
    BYO_CU(ctx, cudaMemcpyAsync(c, hc, sizeof(StreamCtl), cudaMemcpyHostToDevice, ctx->stream));
    StreamArgs a;
    a.src = p->src;
    a.dst = p->dst;
    a.cnt = p->cnt;
    a.sep = p->sep;
    a.NL = NL;
    a.n = g->n;
    a.off = g->d_off;
    a.deg = g->d_deg;
    a.keys = d_keys;
    a.boff = d_boff;
    a.ops = d_ops;
    a.first = bi;
    a.nbatch = be;
    a.sorted = (uint64_t *)p->keys_a.p;
    a.seg = (uint64_t *)p->bstart.p;
    a.vrange = (uint64_t *)p->rpre.p;
    a.chunks = (uint64_t *)p->win.p;
    a.ovf = (uint64_t *)p->ovf.p;
    a.ovf_off = (uint64_t *)p->ovf_off.p;
    a.chunk_words = chunk_words;
    a.shrink_below = NL > 1 ? kRootMin * (double)NL * kLeaf : -1.0;
    a.changed = d_changed;
    a.ctl = c;
    a.qargs = d_qargs;
    a.qnum = d_qnum;
    a.op_ns = d_op_ns;
    void *args[] = {(void *)&a};
    BYO_CU(ctx, cudaLaunchCooperativeKernel((const void *)k_pma_stream, dim3(ctx->num_sms * per_sm),
                                            dim3(kStreamThreads), args, kStreamSmem, ctx->stream));
    ctx->launches++;
    BYO_CU(ctx, cudaMemcpyAsync(hc, c, sizeof(StreamCtl), cudaMemcpyDeviceToHost, ctx->stream));
    BYO_CU(ctx, cudaMemcpyAsync(h_changed + bi, d_changed + bi, 8 * (be - bi), cudaMemcpyDeviceToHost,
                                ctx->stream));
    BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
    if (hc->bar.err) return set_error(ctx, BYO_ETIMEDOUT, "update stream: grid barrier timed out");
    BYO_TRY(check_launch(ctx, "pma_stream"));
    const uint64_t done_to = hc->stop ? hc->stop - 1 : be;  // batches [bi, done_to) are complete
    for (uint64_t k = bi; k < done_to; k++) h_changed[k] = h_changed[k] < 0 ? -h_changed[k] : h_changed[k];
    g->m = (uint64_t)hc->m;
    if (!hc->stop) {
      bi = be;
      continue;
    }
    if (hc->reason == 2) {
      for (uint64_t k = done_to; k < nbatch; k++) h_changed[k] = 0;
      return set_error(ctx, BYO_EINVAL, "update key with src or dst >= n");
    }
    if (hc->reason == 3) return set_error(ctx, BYO_EDEVICE, "mixed stream: a query's hub chunk list overflowed");
    // batch done_to merged with overflowing leaves (or shrinking): finish it
    const int buf = (int)(done_to & 1);
    const long long delta = (long long)hc->ctr[buf][2];
    const uint64_t total = (uint64_t)((long long)g->m + delta);
    const bool shrink = !h_ops[done_to] && (double)total < a.shrink_below;
    h_changed[done_to] = delta < 0 ? -delta : delta;
    const unsigned long long *d_nseg = &c->ctr[buf][3];
    BYO_TRY(pma_finish_windowed(g, true, a.seg + (size_t)buf * 2 * kSmallSort, d_nseg,
                                h_boff[done_to + 1] - h_boff[done_to], total, shrink));
    bi = done_to + 1;
  }
  if (qs && qs->h_op_ns) {
    BYO_CU(ctx, cudaMemcpyAsync(qs->h_op_ns, d_op_ns, 16 * nbatch, cudaMemcpyDeviceToHost, ctx->stream));
    BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return BYO_OK;
}

}  // namespace byo

// vos.cu -- a vector of per-vertex sorted neighbour runs with slack: the GPU
// counterpart of BYO's vector-of-sets containers (run_vector_pma.cc,
// run_vector_vector.cc: gbbs::symmetric_set_graph over one set per vertex,
// gbbs/graph.h:788-1465), behind the same C ABI as the CSR and the PMA.
//
// Layout: one slot array; vertex v owns slots [base[v], base[v+1]), holds its
// deg[v] neighbours sorted at the start of its region and kSentinel in the
// rest.  Region sizes are powers of two >= 5/4 deg + 2 (none for an isolated
// vertex).  base doubles as the traversal view's offsets (gaps are
// kSentinel, as in the PMA's view), deg as its degrees.
//
// A batch (sorted, duplicates kept) is grouped by source; every batch key
// finds its rank in its vertex's run (binary search); a scan over the kept
// keys places them; the run's old keys shift by the number of keys inserted
// before them (or removed before them), found by a binary search over the
// batch keys' ranks.  All of this is flattened over the touched vertices'
// keys, so a hub and a leaf vertex cost the same per key.  The merged runs go
// to a staging area and back into their regions; a run that outgrows its
// region makes every region be laid out again (the runs copied to a new slot
// array, overflowing ones from the staging area).
#include <algorithm>
#include <vector>

#include "device.cuh"
#include "internal.h"
#include "scan.cuh"

namespace byo {

struct Vos {
  DevBuf keys_a, keys_b, misc;
  DevBuf rk, kflag, kscan, segid, segs, tbase, abase, rnew, temp, ovt, chunks;
};

__host__ __device__ __forceinline__ uint64_t vos_cap(uint64_t d) {
  if (!d) return 0;
  const uint64_t want = d + (d >> 2) + 2;
  uint64_t c = 4;
  while (c < want) c <<= 1;
  return c;
}

struct InCap {
  const uint32_t *deg;
  __device__ uint64_t operator()(uint64_t v) const { return vos_cap(deg[v]); }
};

__global__ void k_vos_place(const uint64_t *__restrict__ keys, uint64_t m, const uint64_t *__restrict__ offc,
                            const uint64_t *__restrict__ base, uint32_t *slots) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[i], v = k >> 32;
    slots[base[v] + (i - offc[v])] = (uint32_t)k;
  }
}

// Regions of the current degrees; g->d_off becomes the region starts.
static int vos_regions(byo_graph *g, uint64_t **base_out, uint64_t *total) {
  byo_ctx *ctx = g->ctx;
  uint64_t *base = nullptr;
  BYO_CU(ctx, cudaMalloc(&base, (g->n + 1) * 8));
  const uint64_t *tot = nullptr;
  int rc = scan_apply(ctx, g->n, InCap{g->d_deg}, OutPrefix{base}, &tot);
  uint64_t *h = nullptr;
  if (rc == BYO_OK) rc = pinned(ctx, 4096, (void **)&h);
  if (rc == BYO_OK) {
    cudaMemcpyAsync(base + g->n, tot, 8, cudaMemcpyDeviceToDevice, ctx->stream);
    cudaMemcpyAsync(h, tot, 8, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = set_error(ctx, BYO_EDEVICE, "vos regions", e);
  }
  if (rc != BYO_OK) {
    cudaFree(base);
    return rc;
  }
  *base_out = base;
  *total = h[0];
  return BYO_OK;
}

// g->d_off / d_deg allocated (n+1, n), keys sorted and unique.
int vos_build(byo_graph *g, const uint64_t *d_keys, uint64_t m) {
  byo_ctx *ctx = g->ctx;
  g->vos = new Vos();
  uint64_t *offc = g->d_off;  // the compact offsets first
  BYO_TRY(offsets_from_keys(ctx, d_keys, m, g->n, offc));
  BYO_TRY(degrees_from_offsets(ctx, offc, g->n, g->d_deg));
  uint64_t *base = nullptr, total = 0;
  BYO_TRY(vos_regions(g, &base, &total));
  uint32_t *slots = nullptr;
  cudaError_t e = cudaMalloc(&slots, (total + 16) * 4);
  if (e != cudaSuccess) {
    cudaFree(base);
    return set_error(ctx, BYO_ENOMEM, "cudaMalloc vos slots", e);
  }
  BYO_CU(ctx, cudaMemsetAsync(slots, 0xFF, (total + 16) * 4, ctx->stream));
  launch(ctx, k_vos_place, dim3(grid_for(ctx, m, 256)), dim3(256), 0, d_keys, m, (const uint64_t *)offc,
         (const uint64_t *)base, slots);
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  cudaFree(g->d_off);
  g->d_off = base;
  g->d_slots = slots;
  g->nslots = total;
  g->m = m;
  return check_launch(ctx, "vos_build");
}

void vos_destroy(Vos *v) {
  if (!v) return;
  for (DevBuf *b : {&v->keys_a, &v->keys_b, &v->misc, &v->rk, &v->kflag, &v->kscan, &v->segid, &v->segs, &v->tbase,
                    &v->abase, &v->rnew, &v->temp, &v->ovt, &v->chunks})
    free_buf(*b);
  delete v;
}

// The compact CSR of the runs (for the read-only algorithms' snapshot):
// out[offc[v] ..] = the first deg[v] slots of v's region.
// The element ranges of units (vertices, touched runs) are walked in chunks
// of kChunk consecutive positions, a warp per chunk, so a hub's run is spread
// over many warps and no warp's work depends on the degrees.  For each chunk
// the warp loads the starts and metadata of up to 32 consecutive units (from
// first[c], the unit holding the chunk's first position) into shared memory,
// lane j unit j, handles the chunk's positions inside them -- each lane finds
// its first position's unit by a binary search over the 32 starts and then
// steps forward with its positions -- and moves on to the next 32 units until
// the chunk ends.
constexpr int kVosBlock = 256;
constexpr int kVosWarps = kVosBlock / 32;
constexpr uint64_t kChunk = 2048;

// first[c] = the unit whose range [ust[u], ust[u+1]) holds position c * kChunk
__global__ void k_chunk_first(const uint64_t *__restrict__ ust, uint64_t nunits, uint32_t *first) {
  for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < nunits;
       u += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t a = ust[u], b = ust[u + 1];
    for (uint64_t c = (a + kChunk - 1) / kChunk; c * kChunk < b; c++) first[c] = (uint32_t)u;
  }
}

static int chunk_first(byo_ctx *ctx, DevBuf &buf, const uint64_t *ust, uint64_t nunits, uint64_t total,
                       uint32_t **first, uint64_t *nchunks) {
  *nchunks = (total + kChunk - 1) / kChunk;
  BYO_TRY(ensure(ctx, buf, (*nchunks + 1) * 4));
  *first = (uint32_t *)buf.p;
  if (nunits)
    launch(ctx, k_chunk_first, dim3(grid_for(ctx, nunits, 256)), dim3(256), 0, ust, nunits, *first);
  return BYO_OK;
}

// last j in [0, nu) with st[j] <= p (st[nu] is the window's end)
__device__ __forceinline__ int unit_of(const uint64_t *st, int nu, uint64_t p) {
  int lo = 0, hi = nu;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (st[mid] <= p) lo = mid; else hi = mid;
  }
  return lo;
}
// From the unit j of an earlier position to the unit of p: a lane's positions
// rise by 32 per step and runs hold ~30 keys, so this is about one compare.
__device__ __forceinline__ int unit_next(const uint64_t *st, int nu, int j, uint64_t p) {
  while (j + 1 < nu && st[j + 1] <= p) j++;
  return j;
}

__global__ void __launch_bounds__(kVosBlock) k_vos_compact(const uint64_t *__restrict__ base,
                                                           const uint32_t *__restrict__ slots,
                                                           const uint64_t *__restrict__ offc, uint64_t n,
                                                           const uint32_t *__restrict__ first, uint64_t nchunks,
                                                           uint32_t *out) {
  __shared__ uint64_t st[kVosWarps][33], sb[kVosWarps][32];
  const unsigned lane = lane_id(), w = threadIdx.x >> 5;
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t total = offc[n];
  for (uint64_t c = gw; c < nchunks; c += nw) {
    const uint64_t c0 = c * kChunk, c1 = min(c0 + kChunk, total);
    uint64_t u = first[c];
    for (;;) {
      const int nu = (int)min((uint64_t)32, n - u);
      if ((int)lane < nu) {
        st[w][lane] = offc[u + lane];
        sb[w][lane] = base[u + lane];
      }
      if (lane == 0) st[w][nu] = offc[u + nu];
      __syncwarp();
      const uint64_t lo = max(c0, st[w][0]), hi = min(c1, st[w][nu]);
      int j = lo + lane < hi ? unit_of(st[w], nu, lo + lane) : 0;
      for (uint64_t p = lo + lane; p < hi; p += 128) {
        uint32_t x[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const uint64_t pp = p + 32 * q;
          if (pp < hi) {
            j = unit_next(st[w], nu, j, pp);
            x[q] = slots[sb[w][j] + (pp - st[w][j])];
          }
        }
#pragma unroll
        for (int q = 0; q < 4; q++)
          if (p + 32 * q < hi) out[p + 32 * q] = x[q];
      }
      const bool more = st[w][nu] < c1;
      __syncwarp();
      if (!more) break;
      u += nu;
    }
  }
}

int vos_compact(byo_graph *g, const uint64_t *offc, uint32_t *out) {
  uint32_t *first = nullptr;
  uint64_t nchunks = 0;
  BYO_TRY(chunk_first(g->ctx, g->vos->chunks, offc, g->n, g->m, &first, &nchunks));
  if (nchunks)
    launch(g->ctx, k_vos_compact, dim3(grid_for(g->ctx, nchunks * 32, kVosBlock, 8)), dim3(kVosBlock), 0,
           (const uint64_t *)g->d_off, (const uint32_t *)g->d_slots, offc, g->n, (const uint32_t *)first, nchunks,
           out);
  return check_launch(g->ctx, "vos_compact");
}

// ---------------------------------------------------------------- update

// out[0], out[1]: the largest src and dst; out[4] set when `sorted` and the
// batch is not strictly increasing.
__global__ void k_vos_bounds(const uint64_t *__restrict__ keys, uint64_t cnt, int sorted, unsigned long long *out) {
  unsigned long long ms = 0, md = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[i];
    ms = ms > (k >> 32) ? ms : (k >> 32);
    md = md > (k & 0xFFFFFFFFull) ? md : (k & 0xFFFFFFFFull);
    if (sorted && i > 0 && keys[i - 1] >= k) out[4] = 1;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long a = __shfl_xor_sync(kFull, ms, o), b = __shfl_xor_sync(kFull, md, o);
    ms = ms > a ? ms : a;
    md = md > b ? md : b;
  }
  if (lane_id() == 0) {
    atomicMax(out, ms);
    atomicMax(out + 1, md);
  }
}

// segment starts: a key whose source differs from the previous key's
struct InSegStart {
  const uint64_t *keys;
  __device__ uint64_t operator()(uint64_t q) const { return q == 0 || (keys[q] >> 32) != (keys[q - 1] >> 32); }
};
struct OutSeg {
  const uint64_t *keys;
  uint32_t *segid;
  uint64_t *segs;  // segs[s] = first key of segment s
  __device__ void operator()(uint64_t q, uint64_t pre, uint64_t f) const {
    segid[q] = (uint32_t)(pre + f - 1);
    if (f) segs[pre] = q;
  }
};

// rank of every batch key in its vertex's run; kept: inserted (absent, first
// of its duplicates) or removed (present, first of its duplicates)
__global__ void k_vos_rank(const uint64_t *__restrict__ keys, uint64_t cnt, const uint64_t *__restrict__ base,
                           const uint32_t *__restrict__ deg, const uint32_t *__restrict__ slots, int insert,
                           uint32_t *rk, uint32_t *kflag) {
  for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < cnt; q += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[q], v = k >> 32;
    const uint32_t x = (uint32_t)k, d = deg[v];
    const uint32_t *A = slots + base[v];
    uint32_t lo = 0, hi = d;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (A[mid] < x) lo = mid + 1; else hi = mid;
    }
    const bool found = lo < d && A[lo] == x;
    const bool dup = q > 0 && keys[q - 1] == k;
    rk[q] = lo;
    kflag[q] = insert ? (!found && !dup) : (found && !dup);
  }
}

struct InU32Flag {
  const uint32_t *f;
  __device__ uint64_t operator()(uint64_t i) const { return f[i]; }
};
// per segment: its run's size after the update (rnew) and before (A keys)
struct InSegNew {
  const uint64_t *keys, *segs, *kscan;
  const uint32_t *deg;
  uint64_t nseg, cnt;
  int insert;
  __device__ uint64_t operator()(uint64_t s) const {
    const uint64_t b0 = segs[s], b1 = s + 1 < nseg ? segs[s + 1] : cnt;
    const uint64_t kept = kscan[b1] - kscan[b0], d = deg[keys[b0] >> 32];
    return insert ? d + kept : d - kept;
  }
};
struct InSegOld {
  const uint64_t *keys, *segs;
  const uint32_t *deg;
  __device__ uint64_t operator()(uint64_t s) const { return deg[keys[segs[s]] >> 32]; }
};

// The old keys of the touched runs, in chunks over their concatenation
// (abase): each key moves to its place in the staging copy of its run,
// shifted by the kept batch keys of its run that go before it (insert:
// rank <= i; remove: rank < i, and a kept batch key among those of rank i
// removes it).
// The ranks and kept-key prefix of a window's batch keys are staged in shared
// memory when they fit; each lane walks a pointer forward through its run's
// batch keys as its keys rise.
constexpr int kShiftStage = 256;
__global__ void __launch_bounds__(kVosBlock)
    k_vos_shift(const uint64_t *__restrict__ keys, uint64_t cnt, const uint64_t *__restrict__ segs, uint64_t nseg,
                const uint64_t *__restrict__ abase, const uint64_t *__restrict__ tbase,
                const uint32_t *__restrict__ rk, const uint32_t *__restrict__ kflag,
                const uint64_t *__restrict__ kscan, const uint64_t *__restrict__ base,
                const uint32_t *__restrict__ slots, int insert, const uint32_t *__restrict__ first,
                uint64_t nchunks, uint32_t *temp) {
  __shared__ uint64_t st[kVosWarps][33], stb[kVosWarps][32], sbs[kVosWarps][32];
  __shared__ uint32_t kb[kVosWarps][33];  // batch key range of each run, relative to the window's first
  __shared__ uint32_t srk[kVosWarps][kShiftStage];
  __shared__ uint32_t sks[kVosWarps][kShiftStage + 1];  // kept prefix relative to the window's first key
  const unsigned lane = lane_id(), w = threadIdx.x >> 5;
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t total = abase[nseg];
  for (uint64_t c = gw; c < nchunks; c += nw) {
    const uint64_t c0 = c * kChunk, c1 = min(c0 + kChunk, total);
    uint64_t s0 = first[c];
    for (;;) {
      const int nu = (int)min((uint64_t)32, nseg - s0);
      const uint64_t sg = s0 + lane;
      const uint64_t g0 = segs[s0], g1 = s0 + nu < nseg ? segs[s0 + nu] : cnt;
      if ((int)lane < nu) {
        const uint64_t b0 = segs[sg];
        st[w][lane] = abase[sg];
        stb[w][lane] = tbase[sg];
        sbs[w][lane] = base[keys[b0] >> 32];
        kb[w][lane] = (uint32_t)(b0 - g0);
      }
      if (lane == 0) {
        st[w][nu] = abase[s0 + nu];
        kb[w][nu] = (uint32_t)(g1 - g0);
      }
      const uint32_t K = (uint32_t)(g1 - g0);
      const bool staged = K <= kShiftStage;
      if (staged) {
        const uint64_t ks0 = kscan[g0];
        for (uint32_t k = lane; k < K; k += 32) srk[w][k] = rk[g0 + k];
        for (uint32_t k = lane; k <= K; k += 32) sks[w][k] = (uint32_t)(kscan[g0 + k] - ks0);
      }
      __syncwarp();
      const uint64_t lo = max(c0, st[w][0]), hi = min(c1, st[w][nu]);
      int jc = lo + lane < hi ? unit_of(st[w], nu, lo + lane) : 0;
      int bj = -1;      // run of the lane's batch-key pointer
      uint32_t bl = 0;  // first batch key of run bj not yet before the lane's key
      for (uint64_t p0 = lo + lane; p0 < hi; p0 += 128) {
        int jq[4];
        uint32_t xq[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const uint64_t p = p0 + 32 * q;
          jq[q] = -1;
          if (p < hi) {
            jc = unit_next(st[w], nu, jc, p);
            jq[q] = jc;
            xq[q] = slots[sbs[w][jc] + (p - st[w][jc])];
          }
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
          if (jq[q] < 0) continue;
          const int j = jq[q];
          const uint32_t i = (uint32_t)(p0 + 32 * q - st[w][j]);
          const uint32_t lb = kb[w][j], e = kb[w][j + 1];
          // the lane's keys rise within a run, so its pointer into the run's
          // batch keys (sorted by rank) only moves forward
          if (j != bj) {
            bj = j;
            bl = lb;
          }
          if (insert)  // batch keys with rank <= i go before A[i]
            while (bl < e && (staged ? srk[w][bl] : rk[g0 + bl]) <= i) bl++;
          else  // the first batch key with rank >= i removes A[i] when it is kept
            while (bl < e && (staged ? srk[w][bl] : rk[g0 + bl]) < i) bl++;
          const uint32_t l = bl;
          const uint32_t before = staged ? sks[w][l] - sks[w][lb] : (uint32_t)(kscan[g0 + l] - kscan[g0 + lb]);
          if (insert) {
            temp[stb[w][j] + i + before] = xq[q];
          } else {
            // the batch keys of rank i: absent ones (below A[i]) first, then
            // A[i] itself and its duplicates; A[i] goes if any is kept
            bool gone = false;
            for (uint32_t t = l; t < e && !gone && (staged ? srk[w][t] : rk[g0 + t]) == i; t++)
              gone = kflag[g0 + t] != 0;
            if (!gone) temp[stb[w][j] + i - before] = xq[q];
          }
        }
      }
      const bool more = st[w][nu] < c1;
      __syncwarp();
      if (!more) break;
      s0 += nu;
    }
  }
}

__global__ void k_vos_insert_new(const uint64_t *__restrict__ keys, uint64_t cnt, const uint32_t *__restrict__ segid,
                                 const uint64_t *__restrict__ segs, const uint64_t *__restrict__ tbase,
                                 const uint32_t *__restrict__ rk, const uint32_t *__restrict__ kflag,
                                 const uint64_t *__restrict__ kscan, uint32_t *temp) {
  for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < cnt; q += (uint64_t)gridDim.x * blockDim.x) {
    if (!kflag[q]) continue;
    const uint32_t s = segid[q];
    temp[tbase[s] + rk[q] + (kscan[q] - kscan[segs[s]])] = (uint32_t)keys[q];
  }
}

// Runs that still fit go back into their regions: chunks over the staging
// area (tbase), a run that outgrew its region skipped.
__global__ void __launch_bounds__(kVosBlock) k_vos_back(const uint64_t *__restrict__ keys,
                                                        const uint64_t *__restrict__ segs, uint64_t nseg,
                                                        const uint64_t *__restrict__ tbase,
                                                        const uint64_t *__restrict__ base,
                                                        const uint32_t *__restrict__ temp,
                                                        const uint32_t *__restrict__ first, uint64_t nchunks,
                                                        uint32_t *slots) {
  __shared__ uint64_t st[kVosWarps][33], sbs[kVosWarps][32];
  const unsigned lane = lane_id(), w = threadIdx.x >> 5;
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t total = tbase[nseg];
  for (uint64_t c = gw; c < nchunks; c += nw) {
    const uint64_t c0 = c * kChunk, c1 = min(c0 + kChunk, total);
    uint64_t s0 = first[c];
    for (;;) {
      const int nu = (int)min((uint64_t)32, nseg - s0);
      const uint64_t sg = s0 + lane;
      if ((int)lane < nu) {
        const uint64_t v = keys[segs[sg]] >> 32;
        const uint64_t t = tbase[sg], b = base[v];
        st[w][lane] = t;
        sbs[w][lane] = tbase[sg + 1] - t <= base[v + 1] - b ? b : ~0ull;
      }
      if (lane == 0) st[w][nu] = tbase[s0 + nu];
      __syncwarp();
      const uint64_t lo = max(c0, st[w][0]), hi = min(c1, st[w][nu]);
      int jc = lo + lane < hi ? unit_of(st[w], nu, lo + lane) : 0;
      for (uint64_t p = lo + lane; p < hi; p += 128) {
        uint32_t x[4];
        int jj[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const uint64_t pp = p + 32 * q;
          jj[q] = -1;
          if (pp < hi) {
            jc = unit_next(st[w], nu, jc, pp);
            jj[q] = jc;
            x[q] = temp[pp];
          }
        }
#pragma unroll
        for (int q = 0; q < 4; q++)
          if (jj[q] >= 0 && sbs[w][jj[q]] != ~0ull) slots[sbs[w][jj[q]] + (p + 32 * q - st[w][jj[q]])] = x[q];
      }
      const bool more = st[w][nu] < c1;
      __syncwarp();
      if (!more) break;
      s0 += nu;
    }
  }
}

// Per touched run, a lane each: its degree; outgrown runs counted and
// remembered (ovt[v] = staging start); a run that shrank gets sentinels after
// its new end (the warp fills each such tail).  Counts reduced per block.
__global__ void __launch_bounds__(kVosBlock) k_vos_runs(const uint64_t *__restrict__ keys,
                                                        const uint64_t *__restrict__ segs, uint64_t nseg,
                                                        const uint64_t *__restrict__ tbase,
                                                        const uint64_t *__restrict__ base, uint32_t *slots,
                                                        uint32_t *deg, uint64_t *ovt,
                                                        unsigned long long *ctr /* [0] outgrown runs, [1] delta */) {
  __shared__ long long red[2][kVosWarps];
  const unsigned lane = lane_id(), w = threadIdx.x >> 5;
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  long long delta = 0, outgrown = 0;
  for (uint64_t s0 = gw * 32; s0 < nseg; s0 += nw * 32) {
    const uint64_t sg = s0 + lane;
    uint64_t b = 0, r = 0, d = 0;
    bool fits = false;
    if (sg < nseg) {
      const uint64_t v = keys[segs[sg]] >> 32;
      const uint64_t t = tbase[sg];
      b = base[v];
      r = tbase[sg + 1] - t;
      d = deg[v];
      fits = r <= base[v + 1] - b;
      if (!fits) {
        ovt[v] = t;
        outgrown++;
      }
      deg[v] = (uint32_t)r;
      delta += (long long)r - (long long)d;
    }
    unsigned m = __ballot_sync(kFull, fits && d > r);
    while (m) {
      const int j = __ffs(m) - 1;
      m &= m - 1;
      const uint64_t bj = __shfl_sync(kFull, b, j), rj = __shfl_sync(kFull, r, j), dj = __shfl_sync(kFull, d, j);
      for (uint64_t i = rj + lane; i < dj; i += 32) slots[bj + i] = kSentinel;
    }
  }
  delta = warp_sum(delta);
  outgrown = warp_sum(outgrown);
  if (lane == 0) {
    red[0][w] = delta;
    red[1][w] = outgrown;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    long long a = 0, o = 0;
    for (int i = 0; i < kVosWarps; i++) {
      a += red[0][i];
      o += red[1][i];
    }
    if (o) atomicAdd(&ctr[0], (unsigned long long)o);
    if (a) atomicAdd(&ctr[1], (unsigned long long)a);
  }
}

// every run into a new slot array (outgrown ones from the staging area)
__global__ void k_vos_relayout(const uint64_t *__restrict__ old_base, const uint32_t *__restrict__ old_slots,
                               const uint64_t *__restrict__ new_base, const uint32_t *__restrict__ deg,
                               const uint64_t *__restrict__ ovt, const uint32_t *__restrict__ temp, uint64_t n,
                               uint32_t *slots) {
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t v = gw; v < n; v += nw) {
    const uint32_t d = deg[v];
    const uint32_t *src = ovt[v] != ~0ull ? temp + ovt[v] : old_slots + old_base[v];
    for (uint32_t i = lane_id(); i < d; i += 32) slots[new_base[v] + i] = src[i];
  }
}

int vos_update(byo_graph *g, const uint64_t *d_keys_in, uint64_t count, int sorted, int insert, uint64_t *changed) {
  byo_ctx *ctx = g->ctx;
  Vos *V = g->vos;
  if (!V) return set_error(ctx, BYO_ENOTSUP, "not a vector-of-runs container");
  g->version++;
  uint64_t *h = nullptr;
  BYO_TRY(pinned(ctx, 4096, (void **)&h));
  // 1. validate, sort (duplicates kept)
  BYO_TRY(ensure(ctx, V->misc, 64));
  // [0,1] bounds, [2] outgrown, [3] delta, [4] a "sorted" batch out of order
  unsigned long long *ctr = (unsigned long long *)V->misc.p;
  BYO_CU(ctx, cudaMemsetAsync(ctr, 0, 64, ctx->stream));
  launch(ctx, k_vos_bounds, dim3(grid_for(ctx, count, 256)), dim3(256), 0, d_keys_in, count, sorted, ctr);
  BYO_CU(ctx, cudaMemcpyAsync(h, ctr, 40, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  if (h[0] >= g->n || h[1] >= g->n) return set_error(ctx, BYO_EINVAL, "update key with src or dst >= n");
  if (h[4]) return set_error(ctx, BYO_EINVAL, "sorted batch not increasing");
  BYO_TRY(ensure(ctx, V->keys_a, count * 8));
  BYO_TRY(ensure(ctx, V->keys_b, count * 8));
  const uint64_t *keys = d_keys_in;
  if (!sorted) {
    BYO_TRY(sort_bucketed(ctx, d_keys_in, count, g->n, (uint64_t *)V->keys_a.p, (uint64_t *)V->keys_b.p));
    keys = (const uint64_t *)V->keys_a.p;
  }
  // 2. segments (one per source), ranks, kept keys
  BYO_TRY(ensure(ctx, V->segid, count * 4));
  BYO_TRY(ensure(ctx, V->segs, (count + 1) * 8));
  BYO_TRY(ensure(ctx, V->rk, count * 4));
  BYO_TRY(ensure(ctx, V->kflag, count * 4));
  BYO_TRY(ensure(ctx, V->kscan, (count + 1) * 8));
  uint32_t *segid = (uint32_t *)V->segid.p, *rk = (uint32_t *)V->rk.p, *kflag = (uint32_t *)V->kflag.p;
  uint64_t *segs = (uint64_t *)V->segs.p, *kscan = (uint64_t *)V->kscan.p;
  const uint64_t *tot = nullptr;
  BYO_TRY(scan_apply(ctx, count, InSegStart{keys}, OutSeg{keys, segid, segs}, &tot));
  BYO_CU(ctx, cudaMemcpyAsync(h, tot, 8, cudaMemcpyDeviceToHost, ctx->stream));
  launch(ctx, k_vos_rank, dim3(grid_for(ctx, count, 256)), dim3(256), 0, keys, count, (const uint64_t *)g->d_off,
         (const uint32_t *)g->d_deg, (const uint32_t *)g->d_slots, insert, rk, kflag);
  BYO_TRY(scan_apply(ctx, count, InU32Flag{kflag}, OutPrefix{kscan}, &tot));
  BYO_CU(ctx, cudaMemcpyAsync(kscan + count, tot, 8, cudaMemcpyDeviceToDevice, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  const uint64_t nseg = h[0];
  // 3. staging layout: new run sizes (tbase) and old ones (abase)
  BYO_TRY(ensure(ctx, V->tbase, (nseg + 1) * 8));
  BYO_TRY(ensure(ctx, V->abase, (nseg + 1) * 8));
  uint64_t *tbase = (uint64_t *)V->tbase.p, *abase = (uint64_t *)V->abase.p;
  BYO_TRY(scan_apply(ctx, nseg, InSegNew{keys, segs, kscan, g->d_deg, nseg, count, insert}, OutPrefix{tbase}, &tot));
  BYO_CU(ctx, cudaMemcpyAsync(tbase + nseg, tot, 8, cudaMemcpyDeviceToDevice, ctx->stream));
  BYO_CU(ctx, cudaMemcpyAsync(h, tot, 8, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_TRY(scan_apply(ctx, nseg, InSegOld{keys, segs, g->d_deg}, OutPrefix{abase}, &tot));
  BYO_CU(ctx, cudaMemcpyAsync(abase + nseg, tot, 8, cudaMemcpyDeviceToDevice, ctx->stream));
  BYO_CU(ctx, cudaMemcpyAsync(h + 1, tot, 8, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  const uint64_t total_t = h[0], total_a = h[1];
  BYO_TRY(ensure(ctx, V->temp, (total_t + 1) * 4));
  uint32_t *temp = (uint32_t *)V->temp.p;
  // 4. merged runs into the staging area, back into their regions
  // chunk tables for the shift (over the old keys) and the copy back (over
  // the staging area), sized once: the buffer must not move between the two
  BYO_TRY(ensure(ctx, V->chunks, ((total_a > total_t ? total_a : total_t) / kChunk + 2) * 4));
  uint32_t *first = nullptr;
  uint64_t nchunks = 0;
  BYO_TRY(chunk_first(ctx, V->chunks, abase, nseg, total_a, &first, &nchunks));
  if (nchunks)
    launch(ctx, k_vos_shift, dim3(grid_for(ctx, nchunks * 32, kVosBlock, 8)), dim3(kVosBlock), 0, keys, count,
           (const uint64_t *)segs, nseg, (const uint64_t *)abase, (const uint64_t *)tbase, (const uint32_t *)rk,
           (const uint32_t *)kflag, (const uint64_t *)kscan, (const uint64_t *)g->d_off,
           (const uint32_t *)g->d_slots, insert, (const uint32_t *)first, nchunks, temp);
  if (insert)
    launch(ctx, k_vos_insert_new, dim3(grid_for(ctx, count, 256)), dim3(256), 0, keys, count,
           (const uint32_t *)segid, (const uint64_t *)segs, (const uint64_t *)tbase, (const uint32_t *)rk,
           (const uint32_t *)kflag, (const uint64_t *)kscan, temp);
  BYO_TRY(ensure(ctx, V->ovt, g->n * 8));
  uint64_t *ovt = (uint64_t *)V->ovt.p;
  BYO_CU(ctx, cudaMemsetAsync(ovt, 0xFF, g->n * 8, ctx->stream));
  BYO_TRY(chunk_first(ctx, V->chunks, tbase, nseg, total_t, &first, &nchunks));
  if (nchunks)
    launch_t(ctx, "vos_merge", k_vos_back, dim3(grid_for(ctx, nchunks * 32, kVosBlock, 8)), dim3(kVosBlock), 0,
             keys, (const uint64_t *)segs, nseg, (const uint64_t *)tbase, (const uint64_t *)g->d_off,
             (const uint32_t *)temp, (const uint32_t *)first, nchunks, g->d_slots);
  launch(ctx, k_vos_runs, dim3(grid_for(ctx, (nseg + 31) / 32 * 32, kVosBlock, 8)), dim3(kVosBlock), 0, keys,
         (const uint64_t *)segs, nseg, (const uint64_t *)tbase, (const uint64_t *)g->d_off, g->d_slots, g->d_deg,
         ovt, ctr + 2);
  BYO_CU(ctx, cudaMemcpyAsync(h, ctr + 2, 16, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  const uint64_t outgrown = h[0];
  const long long delta = (long long)h[1];
  g->m = (uint64_t)((long long)g->m + delta);
  if (changed) *changed = (uint64_t)(delta < 0 ? -delta : delta);
  if (!outgrown) return check_launch(ctx, "vos_update");
  // 5. a run outgrew its region: lay every region out again
  uint64_t *nbase = nullptr, ntotal = 0;
  BYO_TRY(vos_regions(g, &nbase, &ntotal));
  uint32_t *nslots = nullptr;
  cudaError_t e = cudaMalloc(&nslots, (ntotal + 16) * 4);
  if (e != cudaSuccess) {
    cudaFree(nbase);
    return set_error(ctx, BYO_ENOMEM, "cudaMalloc vos slots", e);
  }
  BYO_CU(ctx, cudaMemsetAsync(nslots, 0xFF, (ntotal + 16) * 4, ctx->stream));
  launch(ctx, k_vos_relayout, dim3(grid_for(ctx, g->n * 32, 256, 8)), dim3(256), 0, (const uint64_t *)g->d_off,
         (const uint32_t *)g->d_slots, (const uint64_t *)nbase, (const uint32_t *)g->d_deg, (const uint64_t *)ovt,
         (const uint32_t *)temp, g->n, nslots);
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  cudaFree(g->d_off);
  cudaFree(g->d_slots);
  g->d_off = nbase;
  g->d_slots = nslots;
  g->nslots = ntotal;
  return check_launch(ctx, "vos_relayout");
}

}  // namespace byo

// primitives.cu -- device replacements for the parlaylib primitives on the
// path (gbbs/bridge.h:208-313): scan, radix sort, unique, CSR offsets.
//
// Radix sort: LSD, 8-bit digits, only over the key bytes that can differ
// (sig_mask), three launches per pass:
//   histogram  per SORT_TILE-key tile, 256 bins in shared memory;
//   scan       digit-major tile histograms -> global output offsets;
//   scatter    stable ranking inside the tile with __match_any_sync, one
//              256-key sub-round at a time, then one store per key.
// Algorithmic bytes per pass: 8 (histogram read) + 8 + 8 (scatter read/write)
// per key.
#include <vector>

#include "device.cuh"
#include "internal.h"
#include "scan.cuh"

namespace byo {

// ---------------------------------------------------------------- host utilities

int set_error(byo_ctx *ctx, int code, const char *what, cudaError_t e) {
  if (ctx) {
    ctx->err = what ? what : "";
    if (e != cudaSuccess) {
      ctx->err += ": ";
      ctx->err += cudaGetErrorString(e);
    }
  }
  return code;
}

bool ktimer_begin(byo_ctx *ctx, const char *tag) {
  if (ctx->ktag != "*" && ctx->ktag != tag) return false;
  while (ctx->kev.size() < ctx->kev_used + 2) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return false;
    ctx->kev.push_back(e);
  }
  cudaEventRecord(ctx->kev[ctx->kev_used], ctx->stream);
  ctx->ktags.push_back(tag);
  return true;
}

void ktimer_end(byo_ctx *ctx) {
  cudaEventRecord(ctx->kev[ctx->kev_used + 1], ctx->stream);
  ctx->kev_used += 2;
}

int check_launch(byo_ctx *ctx, const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(ctx, BYO_EDEVICE, what, e);
  return BYO_OK;
}

void free_buf(DevBuf &b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
}

int ensure(byo_ctx *ctx, DevBuf &b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (b.bytes >= bytes) return BYO_OK;
  // The old contents are not preserved; buffers grow only between uses.
  if (b.p) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return set_error(ctx, BYO_EDEVICE, "sync before realloc", e);
    cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
  }
  size_t want = bytes + bytes / 8;  // headroom against repeated small growth
  cudaError_t e = cudaMalloc(&b.p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    b.p = nullptr;
    return set_error(ctx, BYO_ENOMEM, "cudaMalloc", e);
  }
  b.bytes = want;
  return BYO_OK;
}

int pinned(byo_ctx *ctx, size_t bytes, void **out) {
  if (ctx->pinned_bytes < bytes) {
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    ctx->pinned = nullptr;
    ctx->pinned_bytes = 0;
    cudaError_t e = cudaMallocHost(&ctx->pinned, bytes);
    if (e != cudaSuccess) return set_error(ctx, BYO_ENOMEM, "cudaMallocHost", e);
    ctx->pinned_bytes = bytes;
  }
  *out = ctx->pinned;
  return BYO_OK;
}

int grid_for(byo_ctx *ctx, uint64_t work, int block, int per_sm) {
  uint64_t want = (work + block - 1) / block;
  uint64_t cap = (uint64_t)ctx->num_sms * per_sm;
  if (want > cap) want = cap;
  if (want < 1) want = 1;
  return (int)want;
}

int memset_async(byo_ctx *ctx, void *p, int v, size_t bytes) {
  if (bytes == 0) return BYO_OK;
  BYO_CU(ctx, cudaMemsetAsync(p, v, bytes, ctx->stream));
  return BYO_OK;
}

uint64_t sig_mask_for(uint64_t n) {
  // keys are src<<32 | dst with src, dst < n
  uint64_t lo = 0;
  if (n > 1) {
    uint64_t top = n - 1;
    lo = 1;
    while (lo <= top && lo != 0) lo <<= 1;
    lo = lo - 1;
    if (lo > 0xFFFFFFFFull) lo = 0xFFFFFFFFull;
  }
  return lo | (lo << 32);
}

// ---------------------------------------------------------------- scans

int scan_u32_to_u64(byo_ctx *ctx, const uint32_t *in, uint64_t count, uint64_t *out) {
  const uint64_t *tot = nullptr;
  BYO_TRY(scan_apply(ctx, count, InU32{in}, OutPrefix{out}, &tot));
  BYO_CU(ctx, cudaMemcpyAsync(out + count, tot, sizeof(uint64_t), cudaMemcpyDeviceToDevice, ctx->stream));
  return BYO_OK;
}

int scan_u64(byo_ctx *ctx, const uint64_t *in, uint64_t count, uint64_t *out) {
  const uint64_t *tot = nullptr;
  BYO_TRY(scan_apply(ctx, count, InU64{in}, OutPrefix{out}, &tot));
  BYO_CU(ctx, cudaMemcpyAsync(out + count, tot, sizeof(uint64_t), cudaMemcpyDeviceToDevice, ctx->stream));
  return BYO_OK;
}

int scan_gather_deg(byo_ctx *ctx, const uint32_t *deg, const uint32_t *list, uint64_t count,
                    uint64_t *out) {
  const uint64_t *tot = nullptr;
  BYO_TRY(scan_apply(ctx, count, InDegOfList{deg, list}, OutPrefix{out}, &tot));
  BYO_CU(ctx, cudaMemcpyAsync(out + count, tot, sizeof(uint64_t), cudaMemcpyDeviceToDevice, ctx->stream));
  return BYO_OK;
}

int scan_gather_range(byo_ctx *ctx, const uint64_t *off, const uint32_t *list, uint64_t count,
                      uint64_t *out) {
  const uint64_t *tot = nullptr;
  BYO_TRY(scan_apply(ctx, count, InRangeOfList{off, list}, OutPrefix{out}, &tot));
  BYO_CU(ctx, cudaMemcpyAsync(out + count, tot, sizeof(uint64_t), cudaMemcpyDeviceToDevice, ctx->stream));
  return BYO_OK;
}

// ---------------------------------------------------------------- radix sort

constexpr int SORT_BLOCK = 256;
constexpr int SORT_SUB = 16;  // sub-rounds of SORT_BLOCK keys per tile
constexpr int SORT_TILE = SORT_BLOCK * SORT_SUB;
constexpr int SORT_WARPS = SORT_BLOCK / 32;

__global__ void __launch_bounds__(SORT_BLOCK) k_radix_hist(const uint64_t *__restrict__ keys,
                                                           uint64_t count, int shift,
                                                           uint32_t *__restrict__ hist,
                                                           uint32_t ntiles) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t base = (uint64_t)blockIdx.x * SORT_TILE;
#pragma unroll 4
  for (int k = 0; k < SORT_SUB; k++) {
    uint64_t i = base + (uint64_t)k * SORT_BLOCK + threadIdx.x;
    if (i < count) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(uint64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one tile: keys are ranked inside the tile (match_any per
// 256-key sub-round), placed in shared memory in digit order, then written
// out in that order so each digit's run goes to consecutive global addresses.
__global__ void __launch_bounds__(SORT_BLOCK) k_radix_scatter(const uint64_t *__restrict__ in,
                                                              uint64_t *__restrict__ out,
                                                              uint64_t count, int shift,
                                                              const uint64_t *__restrict__ offs,
                                                              const uint32_t *__restrict__ hist,
                                                              uint32_t ntiles) {
  __shared__ uint64_t tile[SORT_TILE];
  __shared__ uint32_t run[256];     // next local slot per digit
  __shared__ uint32_t lbase[256];   // local start of each digit
  __shared__ uint64_t gbase[256];   // global start of each digit for this tile
  __shared__ uint32_t wh[SORT_WARPS][256];
  __shared__ uint32_t scan_tmp[SORT_BLOCK / 32 + 1];
  const unsigned t = threadIdx.x, w = t >> 5;
  {
    const uint32_t c = hist[(uint64_t)t * ntiles + blockIdx.x];
    uint32_t tot;
    const uint32_t pre = block_exclusive_scan(c, scan_tmp, &tot);
    lbase[t] = pre;
    run[t] = pre;
    gbase[t] = offs[(uint64_t)t * ntiles + blockIdx.x];
  }
#pragma unroll
  for (int q = 0; q < SORT_WARPS; q++) wh[q][t] = 0;
  __syncthreads();
  const uint64_t base = (uint64_t)blockIdx.x * SORT_TILE;
  const uint32_t nt = (uint32_t)(count - base < SORT_TILE ? count - base : SORT_TILE);
  for (int k = 0; k < SORT_SUB; k++) {
    const uint32_t li = k * SORT_BLOCK + t;
    const bool valid = li < nt;
    const uint64_t key = valid ? in[base + li] : 0;
    const unsigned d = valid ? (unsigned)((key >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(kFull, d);
    const unsigned rank = __popc(peers & lanemask_lt());
    if (valid && rank == 0) wh[w][d] = __popc(peers);
    __syncthreads();
    {
      uint32_t r = run[t];
#pragma unroll
      for (int q = 0; q < SORT_WARPS; q++) {
        const uint32_t c = wh[q][t];
        wh[q][t] = r;
        r += c;
      }
      run[t] = r;
    }
    __syncthreads();
    if (valid) tile[wh[w][d] + rank] = key;
    __syncthreads();
#pragma unroll
    for (int q = 0; q < SORT_WARPS; q++) wh[q][t] = 0;
    __syncthreads();
  }
  // tile[] is in digit order: consecutive threads write consecutive addresses
  for (uint32_t p = t; p < nt; p += SORT_BLOCK) {
    const uint64_t key = tile[p];
    const unsigned d = (unsigned)((key >> shift) & 255u);
    out[gbase[d] + (p - lbase[d])] = key;
  }
}

int sort_u64(byo_ctx *ctx, uint64_t *keys, uint64_t *tmp, uint64_t count, uint64_t sig_mask,
             uint64_t **sorted) {
  uint64_t *a = keys, *b = tmp;
  if (count > 1) {
    const uint64_t ntiles = (count + SORT_TILE - 1) / SORT_TILE;
    uint32_t *hist = nullptr;
    uint64_t *offs = nullptr;
    BYO_TRY(scratch(ctx, 4, 256 * ntiles, &hist));
    BYO_TRY(scratch(ctx, 5, 256 * ntiles + 1, &offs));
    for (int shift = 0; shift < 64; shift += 8) {
      if (((sig_mask >> shift) & 0xFF) == 0) continue;
      launch(ctx, k_radix_hist, dim3((unsigned)ntiles), dim3(SORT_BLOCK), 0, (const uint64_t *)a,
             count, shift, hist, (uint32_t)ntiles);
      BYO_TRY(scan_u32_to_u64(ctx, hist, 256 * ntiles, offs));
      launch_t(ctx, "sort_scatter", k_radix_scatter, dim3((unsigned)ntiles), dim3(SORT_BLOCK), 0, (const uint64_t *)a,
               b, count, shift, (const uint64_t *)offs, (const uint32_t *)hist, (uint32_t)ntiles);
      uint64_t *s = a;
      a = b;
      b = s;
    }
  }
  *sorted = a;
  return check_launch(ctx, "sort_u64");
}

// ---------------------------------------------------------------- bucketed batch sort
// For update batches: keys (src << 32 | dst) with src, dst < n.  One counting
// pass partitions the keys into buckets by the top bits of src (about 24 keys
// per bucket for a uniform batch),
// then one warp per bucket sorts it by rank in shared memory.  Buckets larger
// than kWarpBucket fall back to the LSD sort on their range.
// Traffic: read, read + write, read + write = 40 bytes per key (LSD over 44
// significant bits needs 6 passes of 24 bytes).

// The bucket of a key; a src >= n (a batch that validation will reject after
// the sort) goes to the last bucket, so no key indexes out of bounds.
__device__ __forceinline__ uint64_t key_bucket(uint64_t k, int shift, uint64_t nb) {
  const uint64_t b = (k >> 32) >> shift;
  return b < nb ? b : nb - 1;
}

__global__ void k_bucket_count(const uint64_t *__restrict__ keys, uint64_t count, int shift, uint64_t nb,
                               unsigned int *cnt) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x)
    atomicAdd(cnt + key_bucket(keys[i], shift, nb), 1u);
}

__global__ void k_bucket_scatter(const uint64_t *__restrict__ keys, uint64_t count, int shift, uint64_t nb,
                                 const uint64_t *__restrict__ boff, unsigned int *cursor, uint64_t *out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[i];
    const uint64_t b = key_bucket(k, shift, nb);
    out[boff[b] + atomicAdd(cursor + b, 1u)] = k;
  }
}

// One warp per bucket: warp_bitonic (device.cuh).  Buckets are padded with
// ~0 to R*32 keys; buckets above kWarpBucket keys are listed for the LSD
// fallback.
constexpr uint32_t kWarpBucket = 512;
constexpr uint64_t kTwoLevelMin = 1ull << 21;  // batches from this size take the two-level sort


template <int R>
__device__ __forceinline__ void bucket_sort_regs(const uint64_t *__restrict__ in, uint64_t *out, uint64_t lo,
                                                 uint32_t s) {
  uint64_t v[R];
#pragma unroll
  for (int r = 0; r < R; r++) {
    const uint32_t i = r * 32 + lane_id();
    v[r] = i < s ? in[lo + i] : ~0ull;
  }
  warp_bitonic<R>(v);
#pragma unroll
  for (int r = 0; r < R; r++) {
    const uint32_t i = r * 32 + lane_id();
    if (i < s) out[lo + i] = v[r];
  }
}

__global__ void __launch_bounds__(256) k_bucket_sort(const uint64_t *__restrict__ in, uint64_t *out,
                                                    const uint64_t *__restrict__ boff, uint64_t nb,
                                                    unsigned int *large, unsigned int *nlarge) {
  const unsigned lane = lane_id();
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t b = gw; b < nb; b += nw) {
    const uint64_t lo = boff[b], s = boff[b + 1] - lo;
    if (s == 0) continue;
    if (s > kWarpBucket) {
      if (lane == 0) large[atomicAdd(nlarge, 1u)] = (unsigned int)b;
      continue;
    }
    if (s <= 32) bucket_sort_regs<1>(in, out, lo, (uint32_t)s);
    else if (s <= 64) bucket_sort_regs<2>(in, out, lo, (uint32_t)s);
    else if (s <= 128) bucket_sort_regs<4>(in, out, lo, (uint32_t)s);
    else if (s <= 256) bucket_sort_regs<8>(in, out, lo, (uint32_t)s);
    else bucket_sort_regs<16>(in, out, lo, (uint32_t)s);
  }
}

// ---------------------------------------------------------------- two-level batch sort
// For batches of millions of keys the bucketed sort's scatter (one returning
// atomic and one random 8-byte write per key) dominates.  Two levels instead:
//   1. coarse bins by the top C bits of src (2^C <= kBins, ~10K keys each):
//      a global histogram (block-aggregated), then each CTA partitions a
//      tile of kBinTile keys by bin in shared memory, reserves one run per
//      bin with a single returning atomic, and writes the runs with
//      consecutive stores;
//   2. one CTA per bin: a counting sort in shared memory by the next 10 key
//      bits (fine buckets of ~10 keys), then a warp per fine bucket sorts it
//      in registers (warp_bitonic) and writes it out.
// Bins above kBinCap keys and fine buckets above kWarpBucket keys (skewed
// batches) are listed and sorted afterwards by the LSD sort on their range.
constexpr int kBinThreads = 1024;
constexpr uint32_t kBins = 2048;
constexpr uint32_t kBinTile = 8192;
constexpr uint32_t kBinPer = 12;                      // keys per thread in the per-bin sort
constexpr uint32_t kBinCap = kBinPer * 1024;          // keys of one coarse bin sorted in shared memory
constexpr uint32_t kFine = 4096;  // fine buckets per bin (12 bits)
constexpr uint32_t kRankMax = 64;  // fine buckets sorted by counting ranks

__device__ __forceinline__ uint32_t coarse_bin(uint64_t key, int shift, uint32_t nbins) {
  const uint64_t b = key >> shift;
  return b < nbins ? (uint32_t)b : nbins - 1;
}

__global__ void __launch_bounds__(kBinThreads) k_bin_hist(const uint64_t *__restrict__ keys, uint64_t count,
                                                          int shift, uint32_t nbins, unsigned int *gcnt) {
  __shared__ unsigned int h[kBins];
  for (uint32_t i = threadIdx.x; i < nbins; i += kBinThreads) h[i] = 0;
  __syncthreads();
  for (uint64_t i = blockIdx.x * (uint64_t)kBinThreads + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * kBinThreads)
    atomicAdd(&h[coarse_bin(__ldg(keys + i), shift, nbins)], 1u);
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < nbins; i += kBinThreads)
    if (h[i]) atomicAdd(&gcnt[i], h[i]);
}

__global__ void __launch_bounds__(kBinThreads) k_bin_scatter(const uint64_t *__restrict__ keys, uint64_t count,
                                                             int shift, uint32_t nbins,
                                                             const uint64_t *__restrict__ gstart,
                                                             unsigned int *gcursor, uint64_t *out) {
  extern __shared__ unsigned long long bin_smem[];
  uint64_t *S = reinterpret_cast<uint64_t *>(bin_smem);  // kBinTile keys grouped by bin
  uint64_t *base = S + kBinTile;                          // [nbins] where the tile's run of a bin starts in out
  unsigned int *cnt = reinterpret_cast<unsigned int *>(base + kBins);  // [nbins]
  unsigned int *off = cnt + kBins;                                      // [nbins + 1] exclusive prefix
  __shared__ unsigned int wsum[kBinThreads / 32];
  constexpr uint32_t kPer = kBinTile / kBinThreads;
  const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
  for (uint64_t t0 = (uint64_t)blockIdx.x * kBinTile; t0 < count; t0 += (uint64_t)gridDim.x * kBinTile) {
    const uint32_t tn = (uint32_t)(count - t0 < kBinTile ? count - t0 : kBinTile);
    for (uint32_t i = threadIdx.x; i < nbins; i += kBinThreads) cnt[i] = 0;
    __syncthreads();
    uint64_t k[kPer];
    uint32_t rank[kPer];
#pragma unroll
    for (uint32_t q = 0; q < kPer; q++) {
      const uint32_t i = q * kBinThreads + threadIdx.x;
      k[q] = i < tn ? __ldcs(keys + t0 + i) : 0;
      rank[q] = i < tn ? atomicAdd(&cnt[coarse_bin(k[q], shift, nbins)], 1u) : 0;
    }
    __syncthreads();
    // exclusive prefix over the bins: two bins per thread, then a block scan
    {
      const uint32_t b0 = 2 * threadIdx.x;
      const uint32_t c0 = b0 < nbins ? cnt[b0] : 0, c1 = b0 + 1 < nbins ? cnt[b0 + 1] : 0;
      const uint32_t v = c0 + c1;
      uint32_t inc = warp_inclusive_scan(v);
      if (lane == 31) wsum[warp] = inc;
      __syncthreads();
      if (warp == 0) {
        const uint32_t w = wsum[lane];
        const uint32_t wi = warp_inclusive_scan(w);
        wsum[lane] = wi - w;
      }
      __syncthreads();
      const uint32_t ex = wsum[warp] + inc - v;
      if (b0 < nbins) off[b0] = ex;
      if (b0 + 1 < nbins) off[b0 + 1] = ex + c0;
      if (threadIdx.x == 0) off[nbins] = tn;
    }
    // one run per bin in the output
    for (uint32_t b = threadIdx.x; b < nbins; b += kBinThreads)
      if (cnt[b]) base[b] = gstart[b] + atomicAdd(&gcursor[b], cnt[b]);
    __syncthreads();
#pragma unroll
    for (uint32_t q = 0; q < kPer; q++) {
      const uint32_t i = q * kBinThreads + threadIdx.x;
      if (i < tn) S[off[coarse_bin(k[q], shift, nbins)] + rank[q]] = k[q];
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < tn; i += kBinThreads) {
      const uint64_t x = S[i];
      const uint32_t b = coarse_bin(x, shift, nbins);
      out[base[b] + (i - off[b])] = x;
    }
    __syncthreads();
  }
}

// One CTA per coarse bin.  Fine buckets by the next kFineBits bits of the
// significant key sig = src << lg | dst (2 lg bits; coarse bins are its top C
// bits), shifted down by fsh.
__device__ __forceinline__ uint32_t fine_digit(uint64_t x, int lg, int fsh) {
  const uint64_t sig = ((x >> 32) << lg) | (x & 0xFFFFFFFFull);
  return (uint32_t)(sig >> fsh) & (kFine - 1);
}

__global__ void __launch_bounds__(kBinThreads) k_bin_sort(const uint64_t *__restrict__ in, uint64_t *out,
                                                          const uint64_t *__restrict__ gstart, uint32_t nbins,
                                                          int lg, int fsh, unsigned long long *large,
                                                          unsigned int *nlarge) {
  extern __shared__ unsigned long long bin_smem[];
  uint64_t *S = reinterpret_cast<uint64_t *>(bin_smem);               // [kBinCap]
  unsigned int *fcnt = reinterpret_cast<unsigned int *>(S + kBinCap);  // [kFine]
  unsigned int *foff = fcnt + kFine;                                   // [kFine + 1]
  __shared__ unsigned int wsum[kBinThreads / 32];
  __shared__ unsigned int big[kBinCap / (kRankMax + 1) + 1], nbig;
  constexpr uint32_t kPerT = kFine / kBinThreads;  // fine counters per thread in the scan
  const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
  for (uint32_t bin = blockIdx.x; bin < nbins; bin += gridDim.x) {
    const uint64_t s0 = gstart[bin], sz = gstart[bin + 1] - s0;
    if (sz == 0) continue;
    if (sz > kBinCap) {  // copied unsorted, sorted afterwards on its range
      for (uint64_t i = threadIdx.x; i < sz; i += kBinThreads) out[s0 + i] = in[s0 + i];
      if (threadIdx.x == 0) {
        const unsigned int at = atomicAdd(nlarge, 1u);
        large[2 * at] = s0;
        large[2 * at + 1] = sz;
      }
      continue;
    }
    const uint32_t n32 = (uint32_t)sz;
    // the bin's keys in registers, all loads in flight at once
    uint64_t kx[kBinPer];
#pragma unroll
    for (uint32_t q = 0; q < kBinPer; q++) {
      const uint32_t i = q * kBinThreads + threadIdx.x;
      kx[q] = i < n32 ? __ldcs(in + s0 + i) : 0;
    }
#pragma unroll
    for (uint32_t t = 0; t < kPerT; t++) fcnt[t * kBinThreads + threadIdx.x] = 0;
    if (threadIdx.x == 0) nbig = 0;
    __syncthreads();
#pragma unroll
    for (uint32_t q = 0; q < kBinPer; q++)
      if (q * kBinThreads + threadIdx.x < n32) atomicAdd(&fcnt[fine_digit(kx[q], lg, fsh)], 1u);
    __syncthreads();
    {  // exclusive prefix: kPerT consecutive counters per thread, then a block scan
      uint32_t c[kPerT], v = 0;
#pragma unroll
      for (uint32_t t = 0; t < kPerT; t++) {
        c[t] = fcnt[threadIdx.x * kPerT + t];
        v += c[t];
      }
      const uint32_t inc = warp_inclusive_scan(v);
      if (lane == 31) wsum[warp] = inc;
      __syncthreads();
      if (warp == 0) {
        const uint32_t w = wsum[lane];
        wsum[lane] = warp_inclusive_scan(w) - w;
      }
      __syncthreads();
      uint32_t ex = wsum[warp] + inc - v;
#pragma unroll
      for (uint32_t t = 0; t < kPerT; t++) {
        const uint32_t f = threadIdx.x * kPerT + t;
        foff[f] = ex;
        fcnt[f] = 0;  // reused as the fill cursor
        if (c[t] > kRankMax) big[atomicAdd(&nbig, 1u)] = f;
        ex += c[t];
      }
      if (threadIdx.x == 0) foff[kFine] = n32;
    }
    __syncthreads();
#pragma unroll
    for (uint32_t q = 0; q < kBinPer; q++) {
      if (q * kBinThreads + threadIdx.x >= n32) continue;
      const uint64_t x = kx[q];
      const uint32_t f = fine_digit(x, lg, fsh);
      S[foff[f] + atomicAdd(&fcnt[f], 1u)] = x;
    }
    __syncthreads();
    // fine buckets of up to kRankMax keys (nearly all): every key counts the
    // keys of its bucket that go before it (ties by position) and writes
    // itself at that rank
    for (uint32_t i = threadIdx.x; i < n32; i += kBinThreads) {
      const uint64_t x = S[i];
      const uint32_t f = fine_digit(x, lg, fsh);
      const uint32_t lo = foff[f], hi = foff[f + 1];
      if (hi - lo > kRankMax) continue;
      uint32_t r = 0;
      for (uint32_t q = lo; q < hi; q++) {
        const uint64_t y = S[q];
        r += (y < x) | ((y == x) & (q < i));
      }
      out[s0 + lo + r] = x;
    }
    // larger ones: a warp each
    for (uint32_t t = warp; t < nbig; t += kBinThreads / 32) {
      const uint32_t f = big[t];
      const uint32_t lo = foff[f], fs = foff[f + 1] - lo;
      if (fs > kWarpBucket) {  // copied unsorted, sorted afterwards on its range
        for (uint32_t i = lane; i < fs; i += 32) out[s0 + lo + i] = S[lo + i];
        if (lane == 0) {
          const unsigned int at = atomicAdd(nlarge, 1u);
          large[2 * at] = s0 + lo;
          large[2 * at + 1] = fs;
        }
        continue;
      }
      const uint64_t *src = S + lo;
      uint64_t *dst = out + s0 + lo;
      if (fs <= 128) {
        uint64_t v[4];
#pragma unroll
        for (int r = 0; r < 4; r++) v[r] = r * 32 + lane < fs ? src[r * 32 + lane] : ~0ull;
        warp_bitonic<4>(v);
#pragma unroll
        for (int r = 0; r < 4; r++)
          if (r * 32 + lane < fs) dst[r * 32 + lane] = v[r];
      } else {
        uint64_t v[16];
#pragma unroll
        for (int r = 0; r < 16; r++) v[r] = r * 32 + lane < fs ? src[r * 32 + lane] : ~0ull;
        warp_bitonic<16>(v);
#pragma unroll
        for (int r = 0; r < 16; r++)
          if (r * 32 + lane < fs) dst[r * 32 + lane] = v[r];
      }
    }
    __syncthreads();
  }
}

int sort_two_level(byo_ctx *ctx, const uint64_t *in, uint64_t count, uint64_t n, uint64_t *out, uint64_t *tmp) {
  int lg = 0;
  while ((1ull << lg) < n) lg++;
  // about 8K keys per coarse bin (at most kBins bins)
  int C = 1;
  while (C < 11 && C < lg && (count >> C) > 8192) C++;
  const uint32_t nbins = 1u << C;
  const int shift = 32 + lg - C;
  const int fsh = 2 * lg - C - 12 > 0 ? 2 * lg - C - 12 : 0;  // fine digit: the next 12 bits of src << lg | dst
  // one scratch buffer (slot 6; the scan below uses slot 7): bin starts
  // [nbins + 1], the list of ranges left for the LSD sort, then 32-bit bin
  // counts, cursors and the list length
  uint64_t *gstart = nullptr;
  const uint64_t nlist = 2 * (count / kWarpBucket + nbins + 1);
  BYO_TRY(scratch(ctx, 6, (uint64_t)nbins + 1 + nlist + nbins + 4, &gstart));
  unsigned long long *large = reinterpret_cast<unsigned long long *>(gstart + nbins + 1);
  unsigned int *gcnt = reinterpret_cast<unsigned int *>(gstart + nbins + 1 + nlist);
  unsigned int *gcursor = gcnt + nbins, *nlarge = gcnt + 2 * nbins;
  BYO_CU(ctx, cudaMemsetAsync(gcnt, 0, (2 * (uint64_t)nbins + 8) * 4, ctx->stream));
  launch(ctx, k_bin_hist, dim3(grid_for(ctx, count, kBinThreads, 2)), dim3(kBinThreads), 0, in, count, shift, nbins,
         gcnt);
  BYO_TRY(scan_u32_to_u64(ctx, gcnt, nbins, gstart));
  const size_t smem1 = (kBinTile + kBins) * 8 + (2 * kBins + 1) * 4;
  const size_t smem2 = kBinCap * 8 + (2 * kFine + 1) * 4;
  BYO_CU(ctx, cudaFuncSetAttribute(k_bin_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1));
  BYO_CU(ctx, cudaFuncSetAttribute(k_bin_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2));
  const uint64_t tiles = (count + kBinTile - 1) / kBinTile;
  launch_t(ctx, "sort_scatter", k_bin_scatter, dim3((unsigned)std::min<uint64_t>(tiles, 2ull * ctx->num_sms)),
           dim3(kBinThreads), smem1, in, count, shift, nbins, (const uint64_t *)gstart, gcursor, tmp);
  launch_t(ctx, "sort_bins", k_bin_sort, dim3(std::min<uint32_t>(nbins, 2u * ctx->num_sms)), dim3(kBinThreads),
           smem2, (const uint64_t *)tmp, out, (const uint64_t *)gstart, nbins, lg, fsh, large, nlarge);
  BYO_TRY(check_launch(ctx, "sort_two_level"));
  unsigned int *h = nullptr;
  BYO_TRY(pinned(ctx, 4096, (void **)&h));
  BYO_CU(ctx, cudaMemcpyAsync(h, nlarge, 4, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  const unsigned int nl = h[0];
  if (nl) {
    // skewed ranges, already in place in out: the LSD sort (it reuses
    // scratch 4 and 5) on each, tmp's range as its second buffer
    std::vector<unsigned long long> ranges(2 * (size_t)nl);
    BYO_CU(ctx, cudaMemcpy(ranges.data(), large, 16ull * nl, cudaMemcpyDeviceToHost));
    for (unsigned int q = 0; q < nl; q++) {
      const uint64_t lo = ranges[2 * q], sz = ranges[2 * q + 1];
      uint64_t *res = nullptr;
      BYO_TRY(sort_u64(ctx, out + lo, tmp + lo, sz, sig_mask_for(n), &res));
      if (res != out + lo) BYO_CU(ctx, cudaMemcpyAsync(out + lo, res, sz * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    }
  }
  return check_launch(ctx, "sort_two_level");
}

int sort_bucketed(byo_ctx *ctx, const uint64_t *in, uint64_t count, uint64_t n, uint64_t *out, uint64_t *tmp) {
  if (count == 0) return BYO_OK;
  if (count >= kTwoLevelMin) return sort_two_level(ctx, in, count, n, out, tmp);
  int lg = 0;
  while ((1ull << lg) < n) lg++;
  // about 24 keys per bucket: most buckets sort in one or two registers a lane
  int D = 8;
  while (D < 24 && (1ull << D) * 24 < count) D++;
  if (D > lg) D = lg;
  const int shift = lg - D;
  const uint64_t nb = ((n - 1) >> shift) + 1;
  if (count > nb * (kWarpBucket / 2)) {
    // buckets would mostly overflow the register sort: global LSD instead
    uint64_t *res = nullptr;
    BYO_CU(ctx, cudaMemcpyAsync(out, in, count * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    BYO_TRY(sort_u64(ctx, out, tmp, count, sig_mask_for(n), &res));
    if (res != out) BYO_CU(ctx, cudaMemcpyAsync(out, res, count * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    return check_launch(ctx, "sort_bucketed");
  }
  unsigned int *cnt = nullptr;
  uint64_t *boff = nullptr;
  BYO_TRY(scratch(ctx, 4, 2 * nb + 8, &cnt));  // counts, cursors, large-bucket count
  BYO_TRY(scratch(ctx, 5, nb + 1, &boff));
  unsigned int *cursor = cnt + nb, *nlarge = cnt + 2 * nb;
  BYO_CU(ctx, cudaMemsetAsync(cnt, 0, (2 * nb + 8) * 4, ctx->stream));
  launch(ctx, k_bucket_count, dim3(grid_for(ctx, count, 256, 16)), dim3(256), 0, in, count, shift, nb, cnt);
  BYO_TRY(scan_u32_to_u64(ctx, cnt, nb, boff));
  launch(ctx, k_bucket_scatter, dim3(grid_for(ctx, count, 256, 16)), dim3(256), 0, in, count, shift, nb,
         (const uint64_t *)boff, cursor, tmp);
  // the large-bucket list reuses the count array (the counts live in boff now)
  launch_t(ctx, "sort_scatter", k_bucket_sort, dim3(grid_for(ctx, nb * 32, 256, 8)), dim3(256), 0,
           (const uint64_t *)tmp, out, (const uint64_t *)boff, nb, cnt, nlarge);
  BYO_TRY(check_launch(ctx, "sort_bucketed"));
  unsigned int *h = nullptr;
  BYO_TRY(pinned(ctx, 4096, (void **)&h));
  BYO_CU(ctx, cudaMemcpyAsync(h, nlarge, 4, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  const unsigned int nl = h[0];
  if (nl) {
    // the LSD sort below reuses scratch slots 4 and 5 (counts, offsets):
    // take every large bucket's range first
    std::vector<unsigned int> big(nl);
    std::vector<uint64_t> ranges(2 * (size_t)nl);
    BYO_CU(ctx, cudaMemcpy(big.data(), cnt, nl * 4, cudaMemcpyDeviceToHost));
    for (unsigned int q = 0; q < nl; q++)
      BYO_CU(ctx, cudaMemcpy(&ranges[2 * q], boff + big[q], 16, cudaMemcpyDeviceToHost));
    const uint64_t low_src = ((1ull << shift) - 1) << 32;
    const uint64_t dst_mask = (lg >= 32) ? 0xFFFFFFFFull : ((1ull << lg) - 1);
    for (unsigned int q = 0; q < nl; q++) {
      const uint64_t lo = ranges[2 * q], sz = ranges[2 * q + 1] - ranges[2 * q];
      uint64_t *res = nullptr;
      BYO_CU(ctx, cudaMemcpyAsync(out + lo, tmp + lo, sz * 8, cudaMemcpyDeviceToDevice, ctx->stream));
      BYO_TRY(sort_u64(ctx, out + lo, tmp + lo, sz, low_src | dst_mask, &res));
      if (res != out + lo)
        BYO_CU(ctx, cudaMemcpyAsync(out + lo, res, sz * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    }
  }
  return check_launch(ctx, "sort_bucketed");
}

// ---------------------------------------------------------------- unique / compaction

struct InKeep {
  const uint64_t *k;
  int drop_loops;
  __device__ uint64_t operator()(uint64_t i) const {
    uint64_t x = k[i];
    bool keep = (i == 0) || (x != k[i - 1]);
    if (drop_loops && (uint32_t)(x >> 32) == (uint32_t)x) keep = false;
    return keep ? 1 : 0;
  }
};
struct OutCompact {
  const uint64_t *k;
  uint64_t *out;
  __device__ void operator()(uint64_t i, uint64_t pre, uint64_t v) const {
    if (v) out[pre] = k[i];
  }
};

int unique_u64(byo_ctx *ctx, const uint64_t *in, uint64_t count, int drop_loops, uint64_t *out,
               uint64_t *out_count) {
  const uint64_t *tot = nullptr;
  BYO_TRY(scan_apply(ctx, count, InKeep{in, drop_loops}, OutCompact{in, out}, &tot));
  uint64_t *h = nullptr;
  BYO_TRY(pinned(ctx, 4096, (void **)&h));
  BYO_CU(ctx, cudaMemcpyAsync(h, tot, sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  *out_count = h[0];
  return BYO_OK;
}

// ---------------------------------------------------------------- CSR helpers

__global__ void k_offsets_from_keys(const uint64_t *__restrict__ keys, uint64_t count, uint64_t n,
                                    uint64_t *__restrict__ off) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t s = keys[i] >> 32;
    uint64_t sp1 = (i == 0) ? 0 : (keys[i - 1] >> 32) + 1;
    for (uint64_t v = sp1; v <= s && v <= n; v++) off[v] = i;
    if (i == count - 1)
      for (uint64_t v = s + 1; v <= n; v++) off[v] = count;
  }
}

__global__ void k_fill_u64(uint64_t *p, uint64_t count, uint64_t val) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x)
    p[i] = val;
}

int offsets_from_keys(byo_ctx *ctx, const uint64_t *keys, uint64_t count, uint64_t n,
                      uint64_t *offsets) {
  if (count == 0) {
    launch(ctx, k_fill_u64, dim3(grid_for(ctx, n + 1, 256)), dim3(256), 0, offsets, n + 1, (uint64_t)0);
  } else {
    launch(ctx, k_offsets_from_keys, dim3(grid_for(ctx, count, 256)), dim3(256), 0, keys, count, n,
           offsets);
  }
  return check_launch(ctx, "offsets_from_keys");
}

__global__ void k_dst_from_keys(const uint64_t *__restrict__ keys, uint64_t count,
                                uint32_t *__restrict__ dst) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x)
    dst[i] = (uint32_t)keys[i];
}

int dst_from_keys(byo_ctx *ctx, const uint64_t *keys, uint64_t count, uint32_t *dst) {
  if (count == 0) return BYO_OK;
  launch(ctx, k_dst_from_keys, dim3(grid_for(ctx, count, 256)), dim3(256), 0, keys, count, dst);
  return check_launch(ctx, "dst_from_keys");
}

__global__ void k_degrees_from_offsets(const uint64_t *__restrict__ off, uint64_t n,
                                       uint32_t *__restrict__ deg) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    deg[v] = (uint32_t)(off[v + 1] - off[v]);
}

int degrees_from_offsets(byo_ctx *ctx, const uint64_t *off, uint64_t n, uint32_t *deg) {
  if (n == 0) return BYO_OK;
  launch(ctx, k_degrees_from_offsets, dim3(grid_for(ctx, n, 256)), dim3(256), 0, off, n, deg);
  return check_launch(ctx, "degrees_from_offsets");
}

__global__ void k_reduce_max_u64(const uint64_t *__restrict__ in, uint64_t count,
                                 unsigned long long *out) {
  uint64_t m = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x)
    m = in[i] > m ? in[i] : m;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    uint64_t t = __shfl_xor_sync(kFull, m, o);
    m = t > m ? t : m;
  }
  if (lane_id() == 0) atomicMax(out, (unsigned long long)m);
}

int reduce_max_u64(byo_ctx *ctx, const uint64_t *in, uint64_t count, uint64_t *out_host) {
  unsigned long long *d = nullptr;
  BYO_TRY(scratch(ctx, 3, 1, &d));
  BYO_CU(ctx, cudaMemsetAsync(d, 0, sizeof(uint64_t), ctx->stream));
  if (count) launch(ctx, k_reduce_max_u64, dim3(grid_for(ctx, count, 256)), dim3(256), 0, in, count, d);
  uint64_t *h = nullptr;
  BYO_TRY(pinned(ctx, 4096, (void **)&h));
  BYO_CU(ctx, cudaMemcpyAsync(h, d, sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  *out_host = h[0];
  return check_launch(ctx, "reduce_max");
}

}  // namespace byo

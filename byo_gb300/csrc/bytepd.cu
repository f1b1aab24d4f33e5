// bytepd.cu -- byte-PD compressed neighbour lists, encoded and decoded on the
// GPU.
//
// The format is the reference's bytepd_amortized encoding
// (gbbs/encodings/byte_pd_amortized.h:1100-1155 writes a vertex,
// byte_pd_amortized.cc:7-55 its integers, the reader's iter at
// byte_pd_amortized.h:180-260) in the compressed graph file of
// gbbs/graph_io.h:351-390 (int64 n, m, total bytes; uint64 byte offsets
// [n+1]; uint32 degrees [n]; the bytes).  A vertex of degree d > 0 holds
// uint32 d, uint32 byte offsets (from the vertex start) of blocks 1 .. nb-1
// (nb = 1 + (d-1)/P), and per block uint32 i*P followed by up to P
// neighbours: the first as a signed difference from the source (first byte:
// bit 7 "more bytes", bit 6 sign, six value bits; then 7 bits per byte), the
// rest as differences to the previous neighbour (7 bits per byte, bit 7
// "more").  The reader's P is PARALLEL_DEGREE = 1000 (gbbs/macros.h:83).
//
// GB300 holds a 2^32-edge CSR in 16 GB, so the graph is decoded once into the
// library's CSR / PMA at load time rather than traversed compressed.
//
// Decode: one warp per block.  The warp reads 32 bytes at a time, a ballot of
// the bytes with bit 7 clear marks where integers end, each ending lane
// assembles its integer from up to 5 bytes by shuffles, and a warp scan of the
// differences gives the neighbour ids, written with consecutive stores; the
// next window starts after the last complete integer.  Encode: every edge's
// byte length is independent (its difference to the source or the previous
// neighbour), so a scan over the lengths places every edge's bytes and every
// block header, and a thread per edge writes them.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "device.cuh"
#include "internal.h"
#include "scan.cuh"

namespace byo {

constexpr uint32_t kBpdDefaultBlock = 1000;

__device__ __forceinline__ uint32_t bpd_u32(const unsigned char *p) {
  return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24;
}
__device__ __forceinline__ void bpd_put_u32(unsigned char *p, uint32_t x) {
  p[0] = (unsigned char)x;
  p[1] = (unsigned char)(x >> 8);
  p[2] = (unsigned char)(x >> 16);
  p[3] = (unsigned char)(x >> 24);
}
__host__ __device__ __forceinline__ uint32_t bpd_blocks(uint64_t d, uint32_t P) {
  return d ? (uint32_t)(1 + (d - 1) / P) : 0;
}
__device__ __forceinline__ uint32_t varint_bytes(uint64_t a) {  // 7 bits a byte; 0 takes none
  uint32_t k = 0;
  while (a) {
    k++;
    a >>= 7;
  }
  return k;
}

// ---------------------------------------------------------------- decode

struct InBlocks {
  const uint32_t *deg;
  uint32_t P;
  __device__ uint64_t operator()(uint64_t v) const { return bpd_blocks(deg[v], P); }
};

// blk_vertex[first block of v + i] = v
__global__ void k_bpd_block_owner(const uint32_t *__restrict__ deg, uint64_t n, uint32_t P,
                                  const uint64_t *__restrict__ bfirst, uint32_t *blk_vertex) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b0 = bfirst[v], nb = bfirst[v + 1] - b0;
    for (uint64_t i = 0; i < nb; i++) blk_vertex[b0 + i] = (uint32_t)v;
  }
}

// bad: 1 malformed run
__global__ void __launch_bounds__(256) k_bpd_decode(const unsigned char *__restrict__ bytes,
                                                    const uint64_t *__restrict__ bo,
                                                    const uint32_t *__restrict__ deg,
                                                    const uint64_t *__restrict__ off,
                                                    const uint64_t *__restrict__ bfirst,
                                                    const uint32_t *__restrict__ blk_vertex, uint64_t nblocks,
                                                    uint32_t P, uint32_t *nbrs, unsigned int *bad) {
  const unsigned lane = lane_id();
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t g = gw; g < nblocks; g += nw) {
    const uint32_t v = blk_vertex[g];
    const uint64_t i = g - bfirst[v];
    const uint64_t d = deg[v], vb = bo[v], vlen = bo[v + 1] - vb;
    const uint32_t nbk = bpd_blocks(d, P);
    const unsigned char *base = bytes + vb;
    const uint64_t hdr = 4 + 4ull * (nbk - 1);
    if (vlen < hdr + 4 || bpd_u32(base) != d) {
      if (lane == 0) atomicOr(bad, 1u);
      continue;
    }
    const uint64_t pb = i == 0 ? hdr : bpd_u32(base + 4 + 4 * (i - 1));
    const uint64_t pe = i + 1 == nbk ? vlen : bpd_u32(base + 4 + 4 * i);
    if (pb + 4 > pe || pe > vlen) {
      if (lane == 0) atomicOr(bad, 1u);
      continue;
    }
    if (i + 1 < nbk && pe + 4 > vlen) {
      if (lane == 0) atomicOr(bad, 1u);
      continue;
    }
    const uint64_t e0 = bpd_u32(base + pb), e1 = i + 1 == nbk ? d : bpd_u32(base + pe);
    if (e0 > e1 || e1 > d) {
      if (lane == 0) atomicOr(bad, 1u);
      continue;
    }
    const uint32_t k = (uint32_t)(e1 - e0);
    uint32_t *out = nbrs + off[v] + e0;
    uint64_t p = vb + pb + 4;
    const uint64_t pend = vb + pe;
    uint32_t done = 0;
    int64_t run = 0;  // the last neighbour written
    while (done < k) {
      const bool in = p + lane < pend;
      const uint32_t b = in ? bytes[p + lane] : 0x80u;
      unsigned T = __ballot_sync(kFull, in && !(b & 0x80u));
      // only the integers this block still needs
      const uint32_t need = k - done;
      while ((uint32_t)__popc(T) > need) T &= ~(1u << (31 - __clz(T)));
      if (!T) {  // an integer running past the block, or longer than 32 bytes
        if (lane == 0) atomicOr(bad, 1u);
        break;
      }
      const bool mine = (T >> lane) & 1u;
      const unsigned below = T & lanemask_lt();
      const uint32_t start = below ? 32 - __clz(below) : 0;
      const bool first = done == 0 && start == 0;  // the block's first neighbour
      uint64_t val = 0;
      bool neg = false, over = false;
#pragma unroll
      for (int j = 0; j < 5; j++) {
        const uint32_t src_lane = start + j < 32 ? start + j : 31;
        const uint32_t bj = __shfl_sync(kFull, b, src_lane);
        if (mine && start + j <= lane) {
          if (first) {
            if (j == 0) {
              val = bj & 0x3fu;
              neg = (bj & 0x40u) != 0;
            } else {
              val |= (uint64_t)(bj & 0x7fu) << (6 + 7 * (j - 1));
            }
          } else {
            val |= (uint64_t)(bj & 0x7fu) << (7 * j);
          }
        }
      }
      if (mine && lane - start >= 5) over = true;
      // differences to the previous neighbour; the first is taken from the source
      int64_t delta = 0;
      if (mine) delta = first ? (neg ? (int64_t)v - (int64_t)val : (int64_t)v + (int64_t)val) - run : (int64_t)val;
      int64_t inc = delta;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(kFull, inc, o);
        if (lane >= (unsigned)o) inc += y;
      }
      const int64_t id = run + inc;
      if (mine) {
        if (over || id < 0 || id > 0xFFFFFFFEll || (!first && val == 0)) atomicOr(bad, 1u);
        out[done + __popc(below)] = (uint32_t)id;
      }
      if (__any_sync(kFull, mine && over)) break;
      run += __shfl_sync(kFull, inc, 31);
      done += __popc(T);
      p += 32 - __clz(T);
    }
  }
}

// The blocks of P edges of every vertex: bfirst[v] (its first block, n+1
// entries) and owner[block] = v (both cudaMalloc'd, the caller frees them).
static int block_list(byo_ctx *ctx, uint64_t n, const uint32_t *d_deg, uint32_t P, uint64_t **bfirst_out,
                      uint32_t **owner_out, uint64_t *nblocks) {
  const uint64_t *tot = nullptr;
  uint64_t *bfirst = nullptr;
  uint32_t *owner = nullptr;
  BYO_CU(ctx, cudaMalloc(&bfirst, (n + 1) * 8));
  int rc = scan_apply(ctx, n, InBlocks{d_deg, P}, OutPrefix{bfirst}, &tot);
  uint64_t *h = nullptr;
  if (rc == BYO_OK) rc = pinned(ctx, 4096, (void **)&h);
  if (rc == BYO_OK) {
    cudaMemcpyAsync(bfirst + n, tot, 8, cudaMemcpyDeviceToDevice, ctx->stream);
    cudaMemcpyAsync(h, tot, 8, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = set_error(ctx, BYO_EDEVICE, "byte-PD blocks", e);
  }
  const uint64_t nb = rc == BYO_OK ? h[0] : 0;
  if (rc == BYO_OK) {
    cudaError_t e = cudaMalloc(&owner, (nb ? nb : 1) * 4);
    if (e != cudaSuccess) rc = set_error(ctx, BYO_ENOMEM, "cudaMalloc", e);
  }
  if (rc == BYO_OK)
    launch(ctx, k_bpd_block_owner, dim3(grid_for(ctx, n, 256)), dim3(256), 0, d_deg, n, P, (const uint64_t *)bfirst,
           owner);
  if (rc != BYO_OK) {
    cudaFree(bfirst);
    if (owner) cudaFree(owner);
    return rc;
  }
  *bfirst_out = bfirst;
  *owner_out = owner;
  *nblocks = nb;
  return BYO_OK;
}

int bytepd_decode(byo_ctx *ctx, uint64_t n, const uint64_t *d_bo, const uint32_t *d_deg, const unsigned char *d_bytes,
                  uint32_t P, uint64_t *d_off, uint32_t *d_nbrs) {
  BYO_TRY(scan_u32_to_u64(ctx, d_deg, n, d_off));
  uint64_t *bfirst = nullptr;
  uint32_t *owner = nullptr;
  uint64_t nblocks = 0;
  BYO_TRY(block_list(ctx, n, d_deg, P, &bfirst, &owner, &nblocks));
  unsigned int *bad = nullptr;
  int rc = BYO_OK;
  cudaError_t e0 = cudaMalloc(&bad, 4);
  if (e0 != cudaSuccess) rc = set_error(ctx, BYO_ENOMEM, "cudaMalloc", e0);
  if (rc == BYO_OK) {
    cudaMemsetAsync(bad, 0, 4, ctx->stream);
    launch_t(ctx, "bytepd_decode", k_bpd_decode, dim3(grid_for(ctx, nblocks * 32, 256, 8)), dim3(256), 0, d_bytes,
             d_bo, d_deg, (const uint64_t *)d_off, (const uint64_t *)bfirst, (const uint32_t *)owner, nblocks, P,
             d_nbrs, bad);
    unsigned int hb = 0;
    cudaMemcpyAsync(&hb, bad, 4, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = set_error(ctx, BYO_EDEVICE, "byte-PD decode", e);
    else if (hb) rc = set_error(ctx, BYO_EINVAL, "malformed byte-PD data");
  }
  if (owner) cudaFree(owner);
  if (bad) cudaFree(bad);
  cudaFree(bfirst);
  return rc;
}

// ---------------------------------------------------------------- encode

// bytes of each edge's integer, a warp per block of P edges (hubs spread over
// many warps); bad |= 1 for a list that is not strictly increasing
__global__ void k_bpd_len(const uint64_t *__restrict__ off, const uint32_t *__restrict__ nbrs, uint32_t P,
                          const uint64_t *__restrict__ bfirst, const uint32_t *__restrict__ blk_vertex,
                          uint64_t nblocks, unsigned char *len, unsigned int *bad) {
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t g = gw; g < nblocks; g += nw) {
    const uint32_t v = blk_vertex[g];
    const uint64_t b = off[v], e = off[v + 1];
    const uint64_t x0 = b + (g - bfirst[v]) * P, x1 = x0 + P < e ? x0 + P : e;
    for (uint64_t x = x0 + lane_id(); x < x1; x += 32) {
      if (x > b && nbrs[x] <= nbrs[x - 1]) atomicOr(bad, 1u);
      uint32_t l;
      if (x == x0) {
        const int64_t diff = (int64_t)nbrs[x] - (int64_t)v;
        l = 1 + varint_bytes((uint64_t)(diff < 0 ? -diff : diff) >> 6);
      } else {
        l = varint_bytes(nbrs[x] - nbrs[x - 1]);
      }
      len[x] = (unsigned char)l;
    }
  }
}

struct InLen {
  const unsigned char *len;
  __device__ uint64_t operator()(uint64_t i) const { return len[i]; }
};
// bytes of vertex v: headers plus its edges' bytes (epos is their prefix)
struct InVertexBytes {
  const uint64_t *off, *epos;
  uint32_t P;
  __device__ uint64_t operator()(uint64_t v) const {
    const uint64_t d = off[v + 1] - off[v];
    if (!d) return 0;
    const uint32_t nb = bpd_blocks(d, P);
    return 4 + 4ull * (nb - 1) + 4ull * nb + (epos[off[v + 1]] - epos[off[v]]);
  }
};

// A warp per block of P edges writes its header (and, for block 0, the
// vertex's degree) and its edges' bytes.
__global__ void k_bpd_write(const uint64_t *__restrict__ off, const uint32_t *__restrict__ nbrs, uint32_t P,
                            const uint64_t *__restrict__ bfirst, const uint32_t *__restrict__ blk_vertex,
                            uint64_t nblocks, const uint64_t *__restrict__ epos, const uint64_t *__restrict__ bo,
                            unsigned char *bytes) {
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t g = gw; g < nblocks; g += nw) {
    const uint32_t v = blk_vertex[g];
    const uint64_t b = off[v], e = off[v + 1], d = e - b, blk = g - bfirst[v];
    const uint32_t nb = bpd_blocks(d, P);
    unsigned char *base = bytes + bo[v];
    const uint64_t hdr = 4 + 4ull * (nb - 1);
    const uint64_t x0 = b + blk * P, x1 = x0 + P < e ? x0 + P : e;
    const uint64_t q0 = hdr + 4 * (blk + 1) + (epos[x0] - epos[b]);  // the block's first edge byte
    if (lane_id() == 0) {
      if (blk == 0) bpd_put_u32(base, (uint32_t)d);
      else bpd_put_u32(base + 4 + 4 * (blk - 1), (uint32_t)(q0 - 4));
      bpd_put_u32(base + q0 - 4, (uint32_t)(blk * P));
    }
    for (uint64_t x = x0 + lane_id(); x < x1; x += 32) {
      unsigned char *w = base + q0 + (epos[x] - epos[x0]);
      uint64_t a;
      if (x == x0) {
        const int64_t diff = (int64_t)nbrs[x] - (int64_t)v;
        a = (uint64_t)(diff < 0 ? -diff : diff);
        unsigned char c = (unsigned char)(a & 0x3f);
        if (diff < 0) c |= 0x40;
        a >>= 6;
        if (a) c |= 0x80;
        *w++ = c;
      } else {
        a = nbrs[x] - nbrs[x - 1];
      }
      while (a) {
        unsigned char y = (unsigned char)(a & 0x7f);
        a >>= 7;
        if (a) y |= 0x80;
        *w++ = y;
      }
    }
  }
}

// Encodes the device CSR of g (its snapshot for a PMA); the device byte
// offsets bo[n+1] and bytes are returned in *d_bo / *d_bytes (cudaMalloc'd,
// the caller frees them).
int bytepd_encode(byo_graph *g, uint32_t P, uint64_t **d_bo_out, unsigned char **d_bytes_out, uint64_t *nbytes) {
  byo_ctx *ctx = g->ctx;
  byo_graph *t = nullptr;
  BYO_TRY(traversal_view(g, &t));
  const uint64_t n = t->n, m = t->nslots;
  *d_bo_out = nullptr;
  *d_bytes_out = nullptr;
  unsigned char *len = nullptr;
  uint64_t *epos = nullptr, *bo = nullptr;
  unsigned char *bytes = nullptr;
  unsigned int *bad = nullptr;
  int rc = BYO_OK;
  cudaError_t e = cudaMalloc(&len, m ? m : 1);
  if (e == cudaSuccess) e = cudaMalloc(&epos, (m + 1) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&bo, (n + 1) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&bad, 4);
  if (e != cudaSuccess) rc = set_error(ctx, BYO_ENOMEM, "cudaMalloc", e);
  uint64_t *h = nullptr;
  if (rc == BYO_OK) rc = pinned(ctx, 4096, (void **)&h);
  uint64_t *bfirst = nullptr;
  uint32_t *owner = nullptr;
  uint64_t nblocks = 0;
  if (rc == BYO_OK) rc = block_list(ctx, n, t->d_deg, P, &bfirst, &owner, &nblocks);
  if (rc == BYO_OK) {
    cudaMemsetAsync(bad, 0, 4, ctx->stream);
    launch(ctx, k_bpd_len, dim3(grid_for(ctx, nblocks * 32, 256, 8)), dim3(256), 0, (const uint64_t *)t->d_off,
           (const uint32_t *)t->d_slots, P, (const uint64_t *)bfirst, (const uint32_t *)owner, nblocks, len, bad);
    const uint64_t *tot = nullptr;
    rc = scan_apply(ctx, m, InLen{len}, OutPrefix{epos}, &tot);
    if (rc == BYO_OK) {
      cudaMemcpyAsync(epos + m, tot, 8, cudaMemcpyDeviceToDevice, ctx->stream);
      rc = scan_apply(ctx, n, InVertexBytes{t->d_off, epos, P}, OutPrefix{bo}, &tot);
    }
    if (rc == BYO_OK) {
      cudaMemcpyAsync(bo + n, tot, 8, cudaMemcpyDeviceToDevice, ctx->stream);
      cudaMemcpyAsync(h, tot, 8, cudaMemcpyDeviceToHost, ctx->stream);
      cudaMemcpyAsync(h + 1, bad, 4, cudaMemcpyDeviceToHost, ctx->stream);
      e = cudaStreamSynchronize(ctx->stream);
      if (e != cudaSuccess) rc = set_error(ctx, BYO_EDEVICE, "byte-PD sizes", e);
      else if ((uint32_t)h[1]) rc = set_error(ctx, BYO_EINVAL, "byte-PD: adjacency not strictly increasing");
    }
  }
  const uint64_t total = rc == BYO_OK ? h[0] : 0;
  if (rc == BYO_OK && (e = cudaMalloc(&bytes, total ? total : 1)) != cudaSuccess)
    rc = set_error(ctx, BYO_ENOMEM, "cudaMalloc", e);
  if (rc == BYO_OK) {
    launch_t(ctx, "bytepd_encode", k_bpd_write, dim3(grid_for(ctx, nblocks * 32, 256, 8)), dim3(256), 0,
             (const uint64_t *)t->d_off, (const uint32_t *)t->d_slots, P, (const uint64_t *)bfirst,
             (const uint32_t *)owner, nblocks, (const uint64_t *)epos, (const uint64_t *)bo, bytes);
    rc = check_launch(ctx, "bytepd_encode");
  }
  if (bfirst) cudaFree(bfirst);
  if (owner) cudaFree(owner);
  if (len) cudaFree(len);
  if (epos) cudaFree(epos);
  if (bad) cudaFree(bad);
  if (rc != BYO_OK) {
    if (bo) cudaFree(bo);
    if (bytes) cudaFree(bytes);
    return rc;
  }
  *d_bo_out = bo;
  *d_bytes_out = bytes;
  *nbytes = total;
  return BYO_OK;
}

// ---------------------------------------------------------------- host side

int graph_from_bytepd_host(byo_ctx *ctx, uint64_t n, const uint64_t *h_bo, const uint32_t *h_deg,
                           const unsigned char *h_bytes, uint64_t nbytes, uint32_t P, int container,
                           byo_graph **out) {
  if (n >= 0xFFFFFFFFull) return set_error(ctx, BYO_EINVAL, "n must be < 2^32 - 1");
  if (!h_bo || (n && !h_deg) || (nbytes && !h_bytes)) return set_error(ctx, BYO_EINVAL, "null byte-PD array");
  if (h_bo[0] != 0 || h_bo[n] > nbytes) return set_error(ctx, BYO_EINVAL, "byte-PD offsets outside the bytes");
  uint64_t m = 0;
  for (uint64_t v = 0; v < n; v++) {
    if (h_bo[v + 1] < h_bo[v]) return set_error(ctx, BYO_EINVAL, "byte-PD offsets decrease");
    m += h_deg[v];
  }
  uint64_t *d_bo = nullptr, *d_off = nullptr;
  uint32_t *d_deg = nullptr, *d_nbrs = nullptr;
  unsigned char *d_bytes = nullptr;
  int rc = BYO_OK;
  cudaError_t e = cudaMalloc(&d_bo, (n + 1) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&d_deg, (n ? n : 1) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&d_bytes, nbytes ? nbytes : 1);
  if (e == cudaSuccess) e = cudaMalloc(&d_off, (n + 1) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&d_nbrs, (m ? m : 1) * 4);
  if (e != cudaSuccess) rc = set_error(ctx, BYO_ENOMEM, "cudaMalloc", e);
  if (rc == BYO_OK) {
    cudaMemcpyAsync(d_bo, h_bo, (n + 1) * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (n) cudaMemcpyAsync(d_deg, h_deg, n * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (nbytes) cudaMemcpyAsync(d_bytes, h_bytes, nbytes, cudaMemcpyHostToDevice, ctx->stream);
    rc = bytepd_decode(ctx, n, d_bo, d_deg, d_bytes, P, d_off, d_nbrs);
  }
  if (rc == BYO_OK) rc = graph_from_device_csr(ctx, container, n, m, d_off, d_nbrs, out);
  for (void *p : {(void *)d_bo, (void *)d_deg, (void *)d_bytes, (void *)d_off, (void *)d_nbrs})
    if (p) cudaFree(p);
  return rc;
}

int bytepd_read_file(byo_ctx *ctx, const char *path, uint32_t P, int container, byo_graph **out) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return set_error(ctx, BYO_EINVAL, "byte-PD file: cannot open");
  int64_t hdr[3];
  int rc = BYO_OK;
  std::vector<uint64_t> bo;
  std::vector<uint32_t> deg;
  std::vector<unsigned char> bytes;
  if (std::fread(hdr, 8, 3, f) != 3 || hdr[0] < 0 || hdr[1] < 0 || hdr[2] < 0) {
    rc = set_error(ctx, BYO_EINVAL, "byte-PD file: short header");
  } else if ((uint64_t)hdr[0] >= 0xFFFFFFFFull) {
    rc = set_error(ctx, BYO_EINVAL, "byte-PD file: n does not fit 32-bit ids");
  } else {
    const uint64_t n = (uint64_t)hdr[0], nbytes = (uint64_t)hdr[2];
    bo.resize(n + 1);
    deg.resize(n ? n : 1);
    bytes.resize(nbytes ? nbytes : 1);
    if (std::fread(bo.data(), 8, n + 1, f) != n + 1 || (n && std::fread(deg.data(), 4, n, f) != n) ||
        (nbytes && std::fread(bytes.data(), 1, nbytes, f) != nbytes))
      rc = set_error(ctx, BYO_EINVAL, "byte-PD file: body shorter than the header says");
  }
  std::fclose(f);
  BYO_TRY(rc);
  const uint64_t n = (uint64_t)hdr[0];
  uint64_t m = 0;
  for (uint64_t v = 0; v < n; v++) m += deg[v];
  if (m != (uint64_t)hdr[1]) return set_error(ctx, BYO_EINVAL, "byte-PD file: degrees do not sum to m");
  return graph_from_bytepd_host(ctx, n, bo.data(), deg.data(), bytes.data(), (uint64_t)hdr[2], P, container, out);
}

int bytepd_write_file(byo_graph *g, const char *path, uint32_t P) {
  byo_ctx *ctx = g->ctx;
  uint64_t *d_bo = nullptr;
  unsigned char *d_bytes = nullptr;
  uint64_t nbytes = 0;
  BYO_TRY(bytepd_encode(g, P, &d_bo, &d_bytes, &nbytes));
  const uint64_t n = g->n;
  std::vector<uint64_t> bo(n + 1);
  std::vector<uint32_t> deg(n ? n : 1);
  std::vector<unsigned char> bytes(nbytes ? nbytes : 1);
  byo_graph *t = nullptr;
  int rc = traversal_view(g, &t);
  if (rc == BYO_OK) {
    cudaMemcpyAsync(bo.data(), d_bo, (n + 1) * 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (n) cudaMemcpyAsync(deg.data(), t->d_deg, n * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (nbytes) cudaMemcpyAsync(bytes.data(), d_bytes, nbytes, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = set_error(ctx, BYO_EDEVICE, "byte-PD download", e);
  }
  cudaFree(d_bo);
  cudaFree(d_bytes);
  BYO_TRY(rc);
  FILE *f = std::fopen(path, "wb");
  if (!f) return set_error(ctx, BYO_EINVAL, "byte-PD file: cannot create");
  const int64_t hdr[3] = {(int64_t)n, (int64_t)g->m, (int64_t)nbytes};
  bool ok = std::fwrite(hdr, 8, 3, f) == 3 && std::fwrite(bo.data(), 8, n + 1, f) == n + 1 &&
            (n == 0 || std::fwrite(deg.data(), 4, n, f) == n) &&
            (nbytes == 0 || std::fwrite(bytes.data(), 1, nbytes, f) == nbytes);
  ok = (std::fclose(f) == 0) && ok;
  return ok ? BYO_OK : set_error(ctx, BYO_EINVAL, "byte-PD file: write failed");
}

int bytepd_encode_host(byo_graph *g, uint32_t P, uint64_t *h_bo, uint32_t *h_deg, unsigned char *h_bytes,
                       uint64_t *nbytes) {
  byo_ctx *ctx = g->ctx;
  uint64_t *d_bo = nullptr;
  unsigned char *d_bytes = nullptr;
  uint64_t total = 0;
  BYO_TRY(bytepd_encode(g, P, &d_bo, &d_bytes, &total));
  int rc = BYO_OK;
  const uint64_t cap = *nbytes;
  *nbytes = total;
  if (h_bytes && cap < total) rc = set_error(ctx, BYO_EINVAL, "byte-PD: output buffer too small");
  byo_graph *t = nullptr;
  if (rc == BYO_OK) rc = traversal_view(g, &t);
  if (rc == BYO_OK) {
    if (h_bo) cudaMemcpyAsync(h_bo, d_bo, (g->n + 1) * 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (h_deg && g->n) cudaMemcpyAsync(h_deg, t->d_deg, g->n * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (h_bytes && total) cudaMemcpyAsync(h_bytes, d_bytes, total, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = set_error(ctx, BYO_EDEVICE, "byte-PD download", e);
  }
  cudaFree(d_bo);
  cudaFree(d_bytes);
  return rc;
}

}  // namespace byo

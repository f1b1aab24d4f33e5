// graph.cu -- container construction: from a host CSR (the loader's arrays,
// graph_io.h:117-123) or from a synthetic pair stream generated on the
// device, symmetrised, radix-sorted and deduplicated on the device.
//
// Generators are counter-based: pair i of a stream depends only on (seed, i),
// so the host oracle reproduces any slice bit for bit.
//   key(seed)      = mix64(seed)
//   draw(seed, c)  = mix64(key + c * 0x9E3779B97F4A7C15)
//   mix64          = the SplitMix64 output function (Steele, Lea & Flood,
//                    OOPSLA 2014)
// RMAT (Chakrabarti et al., SDM 2004) pair i takes 32-bit words of draws
// i*32 + l/2, level l most significant first, against integer thresholds.
#include <cmath>
#include <vector>

#include "device.cuh"
#include "internal.h"

namespace byo {

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t draw64(uint64_t key, uint64_t ctr) {
  return mix64(key + ctr * 0x9E3779B97F4A7C15ull);
}

static uint32_t prob_u32(double p) {
  if (p <= 0.0) return 0;
  double s = p * 4294967296.0;
  if (s >= 4294967295.0) return 0xFFFFFFFFu;
  return (uint32_t)s;
}

__device__ __forceinline__ void rmat_pair(uint64_t key, uint32_t lg_n, uint64_t i, uint32_t ta,
                                          uint32_t tab, uint32_t tabc, uint32_t &s, uint32_t &d) {
  s = 0;
  d = 0;
  uint64_t w = 0;
  for (uint32_t l = 0; l < lg_n; l++) {
    if ((l & 1) == 0) w = draw64(key, i * 32 + (l >> 1));
    uint32_t r = (l & 1) ? (uint32_t)(w >> 32) : (uint32_t)w;
    uint32_t bit = 1u << (lg_n - 1 - l);
    if (r < ta) {
    } else if (r < tab) {
      d |= bit;
    } else if (r < tabc) {
      s |= bit;
    } else {
      s |= bit;
      d |= bit;
    }
  }
}

__global__ void k_rmat_pairs(uint64_t key, uint32_t lg_n, uint64_t first, uint64_t count, uint32_t ta,
                             uint32_t tab, uint32_t tabc, uint32_t *src, uint32_t *dst) {
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < count;
       k += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t s, d;
    rmat_pair(key, lg_n, first + k, ta, tab, tabc, s, d);
    src[k] = s;
    dst[k] = d;
  }
}

__global__ void k_rmat_keys(uint64_t key, uint32_t lg_n, uint64_t count, uint32_t ta, uint32_t tab,
                            uint32_t tabc, uint64_t *keys) {
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < count;
       k += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t s, d;
    rmat_pair(key, lg_n, k, ta, tab, tabc, s, d);
    keys[k] = ((uint64_t)s << 32) | d;
    keys[count + k] = ((uint64_t)d << 32) | s;
  }
}

__device__ __forceinline__ void uniform_pair(uint64_t key, uint64_t n, uint64_t i, uint32_t &s, uint32_t &d) {
  uint64_t w = draw64(key, i);
  s = (uint32_t)(((w & 0xFFFFFFFFull) * n) >> 32);
  d = (uint32_t)(((w >> 32) * n) >> 32);
}

__global__ void k_uniform_pairs(uint64_t key, uint64_t n, uint64_t first, uint64_t count, uint32_t *src,
                                uint32_t *dst) {
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < count;
       k += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t s, d;
    uniform_pair(key, n, first + k, s, d);
    src[k] = s;
    dst[k] = d;
  }
}

__global__ void k_uniform_keys(uint64_t key, uint64_t n, uint64_t count, uint64_t *keys) {
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < count;
       k += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t s, d;
    uniform_pair(key, n, k, s, d);
    keys[k] = ((uint64_t)s << 32) | d;
    keys[count + k] = ((uint64_t)d << 32) | s;
  }
}

__global__ void k_grid_keys(uint32_t rows, uint32_t cols, uint64_t *keys, uint64_t per_dir) {
  // pair index k: vertex k/2, direction k&1 (right, down); absent pairs become
  // self loops of vertex 0 and are dropped with the others
  const uint64_t total = 2ull * rows * cols;
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < total;
       k += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t v = k >> 1;
    uint32_t r = (uint32_t)(v / cols), c = (uint32_t)(v % cols);
    uint64_t s = v, d = v;
    if ((k & 1) == 0) {
      if (c + 1 < cols) d = v + 1;
    } else {
      if (r + 1 < rows) d = v + cols;
    }
    if (d == s) s = d = 0;
    keys[k] = (s << 32) | d;
    keys[per_dir + k] = (d << 32) | s;
  }
}

__device__ __forceinline__ uint32_t cdf_pick(const uint64_t *__restrict__ cdf, uint64_t n, uint64_t x) {
  uint64_t lo = 0, hi = n - 1;
  while (lo < hi) {
    uint64_t mid = (lo + hi) >> 1;
    if (x < cdf[mid]) hi = mid; else lo = mid + 1;
  }
  return (uint32_t)lo;
}

__global__ void k_chung_lu_keys(uint64_t key, uint64_t n, const uint64_t *__restrict__ cdf, uint64_t count,
                                uint64_t *keys) {
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < count;
       k += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t s = cdf_pick(cdf, n, draw64(key, 2 * k) >> 1);
    uint64_t d = cdf_pick(cdf, n, draw64(key, 2 * k + 1) >> 1);
    keys[k] = (s << 32) | d;
    keys[count + k] = (d << 32) | s;
  }
}

// Chung-Lu endpoint table: cdf[i] = floor(2^63 * sum_{j<=i} w_j / W) with
// w_j = (j+1)^(-1/(exponent-1)), summed in index order; cdf[n-1] = 2^63.
static void chung_lu_cdf_host(uint64_t n, double exponent, std::vector<uint64_t> &cdf) {
  cdf.resize(n);
  double alpha = 1.0 / (exponent - 1.0), total = 0.0;
  for (uint64_t i = 0; i < n; i++) total += std::pow((double)(i + 1), -alpha);
  double run = 0.0;
  const double scale = 9223372036854775808.0;
  for (uint64_t i = 0; i < n; i++) {
    run += std::pow((double)(i + 1), -alpha);
    double f = run / total * scale;
    cdf[i] = f >= scale ? (1ull << 63) : (uint64_t)f;
  }
  cdf[n - 1] = 1ull << 63;
}

// ---------------------------------------------------------------- construction

__global__ void k_keys_from_csr(const uint64_t *__restrict__ off, const uint32_t *__restrict__ nbrs,
                                uint64_t n, uint64_t *keys) {
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t v = gw; v < n; v += nw)
    for (uint64_t j = off[v] + lane_id(); j < off[v + 1]; j += 32) keys[j] = (v << 32) | nbrs[j];
}

// strictly increasing per vertex and every id < n
__global__ void k_check_csr(const uint64_t *__restrict__ off, const uint32_t *__restrict__ nbrs, uint64_t n,
                            unsigned int *bad) {
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = off[v], e = off[v + 1];
    if (e < b) {
      atomicOr(bad, 1u);
      continue;
    }
    for (uint64_t j = b; j < e; j++) {
      if (nbrs[j] >= n || (j > b && nbrs[j] <= nbrs[j - 1])) {
        atomicOr(bad, 2u);
        break;
      }
    }
  }
}

int graph_alloc_view(byo_graph *g) {
  byo_ctx *ctx = g->ctx;
  if (g->d_off) cudaFree(g->d_off);
  if (g->d_deg) cudaFree(g->d_deg);
  g->d_off = nullptr;
  g->d_deg = nullptr;
  BYO_CU(ctx, cudaMalloc(&g->d_off, (g->n + 1) * sizeof(uint64_t)));
  BYO_CU(ctx, cudaMalloc(&g->d_deg, (g->n ? g->n : 1) * sizeof(uint32_t)));
  return BYO_OK;
}

int graph_from_sorted_keys(byo_ctx *ctx, int container, uint64_t n, const uint64_t *d_keys, uint64_t m,
                           byo_graph **out) {
  byo_graph *g = new byo_graph();
  g->ctx = ctx;
  g->container = container;
  g->n = n;
  g->m = m;
  int rc = graph_alloc_view(g);
  if (rc == BYO_OK) {
    if (container == BYO_CONTAINER_PMA) {
      rc = pma_build(g, d_keys, m);
    } else if (container == BYO_CONTAINER_VOS) {
      rc = vos_build(g, d_keys, m);
    } else if (container == BYO_CONTAINER_PCSR) {
      rc = pcsr_build(g, d_keys, m);
    } else {
      // 16 ids of padding: bulk copies of a slot run round its end up to 16 bytes
      cudaError_t e = cudaMalloc(&g->d_slots, (m + 16) * sizeof(uint32_t));
      if (e != cudaSuccess) rc = set_error(ctx, BYO_ENOMEM, "cudaMalloc slots", e);
      g->nslots = m;
      if (rc == BYO_OK) rc = offsets_from_keys(ctx, d_keys, m, n, g->d_off);
      if (rc == BYO_OK) rc = dst_from_keys(ctx, d_keys, m, g->d_slots);
      if (rc == BYO_OK) rc = degrees_from_offsets(ctx, g->d_off, n, g->d_deg);
    }
  }
  if (rc == BYO_OK) rc = check_launch(ctx, "graph_from_sorted_keys");
  if (rc == BYO_OK) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = set_error(ctx, BYO_EDEVICE, "graph build", e);
  }
  if (rc != BYO_OK) {
    byo_graph_destroy(g);
    return rc;
  }
  *out = g;
  return BYO_OK;
}

// A graph from a CSR already on the device (validated: sorted, duplicate-free,
// ids < n); the arrays stay the caller's.
int graph_from_device_csr(byo_ctx *ctx, int container, uint64_t n, uint64_t m, const uint64_t *d_off,
                          const uint32_t *d_nbrs, byo_graph **out) {
  uint64_t *keys = nullptr;
  unsigned int *d_bad = nullptr;
  int rc = BYO_OK;
  cudaError_t e = cudaMalloc(&keys, (m ? m : 1) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&d_bad, 4);
  if (e != cudaSuccess) rc = set_error(ctx, BYO_ENOMEM, "cudaMalloc", e);
  if (rc == BYO_OK) {
    cudaMemsetAsync(d_bad, 0, 4, ctx->stream);
    launch(ctx, k_check_csr, dim3(grid_for(ctx, n, 256)), dim3(256), 0, d_off, d_nbrs, n, d_bad);
    unsigned int bad = 0;
    cudaMemcpyAsync(&bad, d_bad, 4, cudaMemcpyDeviceToHost, ctx->stream);
    if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) rc = set_error(ctx, BYO_EDEVICE, "check CSR", e);
    else if (bad) rc = set_error(ctx, BYO_EINVAL, "adjacency must be sorted, duplicate-free and < n");
  }
  if (rc == BYO_OK) {
    launch(ctx, k_keys_from_csr, dim3(grid_for(ctx, n * 32, 256, 16)), dim3(256), 0, d_off, d_nbrs, n, keys);
    rc = graph_from_sorted_keys(ctx, container, n, keys, m, out);
  }
  if (keys) cudaFree(keys);
  if (d_bad) cudaFree(d_bad);
  return rc;
}

int graph_from_host_csr(byo_ctx *ctx, int container, uint64_t n, uint64_t m, const uint64_t *h_off,
                        const uint32_t *h_nbrs, byo_graph **out) {
  if (n >= 0xFFFFFFFFull) return set_error(ctx, BYO_EINVAL, "n must be < 2^32 - 1");
  if (!h_off || (m && !h_nbrs)) return set_error(ctx, BYO_EINVAL, "null CSR array");
  if (h_off[0] != 0 || h_off[n] != m) return set_error(ctx, BYO_EINVAL, "offsets[0] != 0 or offsets[n] != m");
  uint64_t *d_off = nullptr;
  uint32_t *d_nbrs = nullptr;
  int rc = BYO_OK;
  cudaError_t e = cudaMalloc(&d_off, (n + 1) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&d_nbrs, (m ? m : 1) * 4);
  if (e != cudaSuccess) rc = set_error(ctx, BYO_ENOMEM, "cudaMalloc", e);
  if (rc == BYO_OK) {
    cudaMemcpyAsync(d_off, h_off, (n + 1) * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (m) cudaMemcpyAsync(d_nbrs, h_nbrs, m * 4, cudaMemcpyHostToDevice, ctx->stream);
    rc = graph_from_device_csr(ctx, container, n, m, d_off, d_nbrs, out);
  }
  if (d_off) cudaFree(d_off);
  if (d_nbrs) cudaFree(d_nbrs);
  return rc;
}

int graph_generate(byo_ctx *ctx, int container, const byo_gen_spec *sp, byo_graph **out) {
  if (!sp) return set_error(ctx, BYO_EINVAL, "null spec");
  uint64_t n = 0, pairs = 0;
  switch (sp->kind) {
    case BYO_GEN_RMAT:
      if (sp->lg_n == 0 || sp->lg_n > 31) return set_error(ctx, BYO_EINVAL, "rmat: lg_n in [1,31]");
      n = 1ull << sp->lg_n;
      pairs = sp->draws;
      break;
    case BYO_GEN_ER:
    case BYO_GEN_CHUNG_LU:
      n = sp->n;
      pairs = sp->draws;
      if (n == 0 || n >= 0xFFFFFFFFull) return set_error(ctx, BYO_EINVAL, "n out of range");
      break;
    case BYO_GEN_GRID:
      n = sp->n * sp->draws;
      pairs = 2 * n;
      if (n == 0 || n >= 0xFFFFFFFFull) return set_error(ctx, BYO_EINVAL, "grid size out of range");
      break;
    default:
      return set_error(ctx, BYO_EINVAL, "unknown generator");
  }
  uint64_t *a = nullptr, *b = nullptr, *cdf = nullptr;
  const uint64_t total = 2 * pairs;
  cudaError_t e;
  if ((e = cudaMalloc(&a, (total ? total : 1) * 8)) != cudaSuccess) return set_error(ctx, BYO_ENOMEM, "cudaMalloc", e);
  if ((e = cudaMalloc(&b, (total ? total : 1) * 8)) != cudaSuccess) {
    cudaFree(a);
    return set_error(ctx, BYO_ENOMEM, "cudaMalloc", e);
  }
  const uint64_t key = mix64(sp->seed);
  const int grid = grid_for(ctx, pairs, 256, 16);
  int rc = BYO_OK;
  if (sp->kind == BYO_GEN_RMAT) {
    launch(ctx, k_rmat_keys, dim3(grid), dim3(256), 0, key, sp->lg_n, pairs, prob_u32(sp->a),
           prob_u32(sp->a + sp->b), prob_u32(sp->a + sp->b + sp->c), a);
  } else if (sp->kind == BYO_GEN_ER) {
    launch(ctx, k_uniform_keys, dim3(grid), dim3(256), 0, key, n, pairs, a);
  } else if (sp->kind == BYO_GEN_GRID) {
    launch(ctx, k_grid_keys, dim3(grid), dim3(256), 0, (uint32_t)sp->n, (uint32_t)sp->draws, a, pairs);
  } else {
    std::vector<uint64_t> h;
    chung_lu_cdf_host(n, sp->exponent, h);
    if ((e = cudaMalloc(&cdf, n * 8)) != cudaSuccess) rc = set_error(ctx, BYO_ENOMEM, "cudaMalloc", e);
    if (rc == BYO_OK) {
      cudaMemcpyAsync(cdf, h.data(), n * 8, cudaMemcpyHostToDevice, ctx->stream);
      launch(ctx, k_chung_lu_keys, dim3(grid), dim3(256), 0, key, n, (const uint64_t *)cdf, pairs, a);
      cudaStreamSynchronize(ctx->stream);  // h goes out of scope
    }
  }
  uint64_t *sorted = nullptr, m = 0;
  if (rc == BYO_OK) rc = sort_u64(ctx, a, b, total, sig_mask_for(n), &sorted);
  uint64_t *uniq = sorted == a ? b : a;
  if (rc == BYO_OK) rc = unique_u64(ctx, sorted, total, 1, uniq, &m);
  if (rc == BYO_OK) rc = graph_from_sorted_keys(ctx, container, n, uniq, m, out);
  cudaFree(a);
  cudaFree(b);
  if (cdf) cudaFree(cdf);
  return rc;
}

int gen_rmat_pairs(byo_ctx *ctx, uint64_t seed, uint32_t lg_n, double a, double b, double c, uint64_t first,
                   uint64_t count, uint32_t *src, uint32_t *dst) {
  if (lg_n == 0 || lg_n > 31 || !src || !dst) return set_error(ctx, BYO_EINVAL, "rmat pairs: bad argument");
  if (count)
    launch(ctx, k_rmat_pairs, dim3(grid_for(ctx, count, 256, 16)), dim3(256), 0, mix64(seed), lg_n, first,
           count, prob_u32(a), prob_u32(a + b), prob_u32(a + b + c), src, dst);
  return check_launch(ctx, "rmat pairs");
}

int gen_uniform_pairs(byo_ctx *ctx, uint64_t seed, uint64_t n, uint64_t first, uint64_t count, uint32_t *src,
                      uint32_t *dst) {
  if (!src || !dst || n == 0 || n > 0xFFFFFFFFull) return set_error(ctx, BYO_EINVAL, "uniform pairs: bad argument");
  if (count)
    launch(ctx, k_uniform_pairs, dim3(grid_for(ctx, count, 256, 16)), dim3(256), 0, mix64(seed), n, first,
           count, src, dst);
  return check_launch(ctx, "uniform pairs");
}

int gen_uniform_keys(byo_ctx *ctx, uint64_t seed, uint64_t n, uint64_t count, uint64_t *keys) {
  if (!keys || n == 0 || n > 0xFFFFFFFFull) return set_error(ctx, BYO_EINVAL, "uniform keys: bad argument");
  if (count)
    launch(ctx, k_uniform_keys, dim3(grid_for(ctx, count, 256, 16)), dim3(256), 0, mix64(seed), n, count, keys);
  return check_launch(ctx, "uniform keys");
}

}  // namespace byo

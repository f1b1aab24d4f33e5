// abi.cu -- the extern "C" boundary declared in include/byo_gpu.h.
// Argument checking, host<->device staging and object lifetime live here;
// the work is in engine.cu, algos.cu, graph.cu and pma.cu.
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "engine.h"
#include "internal.h"

using namespace byo;

#define BYO_VERSION_STR "byo_gpu 0.1 (sm_103a)"

namespace {

int need(byo_ctx *ctx, bool ok, const char *what) {
  return ok ? BYO_OK : set_error(ctx, BYO_EINVAL, what);
}

// Device scratch for host-memory wrappers: one buffer per graph slot.
template <typename T>
int host_out_buffer(byo_graph *g, uint64_t count, T **d) {
  return ws(g, WS_LABEL, count * sizeof(T) / sizeof(uint32_t) + 2, (uint32_t **)d);
}

int copy_to_host(byo_ctx *ctx, void *h, const void *d, size_t bytes) {
  if (!bytes) return BYO_OK;
  BYO_CU(ctx, cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  return BYO_OK;
}

__global__ void k_fill32(uint32_t *d, uint64_t count, uint32_t value) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x)
    d[i] = value;
}

}  // namespace

struct byo_functor {
  byo_graph *g = nullptr;
  int kind = BYO_F_BFS;
  TravState st;  // BFS_F
  DevBuf lp, visited;
  FunctorArgs fa;  // the other kinds
};

struct byo_vertex_subset {
  byo_graph *g = nullptr;
  Frontier f;
  DevBuf list, bits;
};

extern "C" {

const char *byo_version(void) { return BYO_VERSION_STR; }

int byo_gpu_init(int device, byo_ctx **out) {
  if (!out) return BYO_EINVAL;
  *out = nullptr;
  byo_ctx *ctx = new (std::nothrow) byo_ctx();
  if (!ctx) return BYO_ENOMEM;
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  for (int i = 0; e == cudaSuccess && i < 64; i++) e = cudaEventCreate(&ctx->ev[i]);
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return BYO_EDEVICE;
  }
  *out = ctx;
  return BYO_OK;
}

void byo_gpu_shutdown(byo_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (auto &b : ctx->scratch) free_buf(b);
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  for (int i = 0; i < 64; i++)
    if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
  for (cudaEvent_t e : ctx->kev) cudaEventDestroy(e);
  policy_destroy(ctx->policy);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char *byo_last_error(const byo_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }
void *byo_ctx_stream(byo_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }
uint64_t byo_ctx_launches(const byo_ctx *ctx) { return ctx ? ctx->launches : 0; }
int byo_buffer_alloc(byo_ctx *ctx, uint64_t bytes, void **d_out) {
  if (!ctx || !d_out) return BYO_EINVAL;
  *d_out = nullptr;
  if (cudaMalloc(d_out, bytes ? bytes : 1) != cudaSuccess) {
    cudaGetLastError();
    *d_out = nullptr;
    return set_error(ctx, BYO_ENOMEM, "buffer: device allocation");
  }
  return BYO_OK;
}

void byo_buffer_free(byo_ctx *ctx, void *d) {
  if (!ctx || !d) return;
  cudaStreamSynchronize(ctx->stream);
  cudaFree(d);
}

int byo_buffer_write(byo_ctx *ctx, void *d, uint64_t offset, const void *h, uint64_t bytes) {
  if (!ctx || !d || (bytes && !h)) return BYO_EINVAL;
  if (!bytes) return BYO_OK;
  BYO_CU(ctx, cudaMemcpyAsync(static_cast<char *>(d) + offset, h, bytes, cudaMemcpyHostToDevice, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  return BYO_OK;
}

int byo_buffer_read(byo_ctx *ctx, const void *d, uint64_t offset, void *h, uint64_t bytes) {
  if (!ctx || !d || (bytes && !h)) return BYO_EINVAL;
  return copy_to_host(ctx, h, static_cast<const char *>(d) + offset, bytes);
}

int byo_buffer_fill32(byo_ctx *ctx, void *d, uint64_t offset, uint64_t count, uint32_t value) {
  if (!ctx || !d || (offset & 3)) return BYO_EINVAL;
  if (!count) return BYO_OK;
  launch(ctx, k_fill32, dim3(grid_for(ctx, count, 256)), dim3(256), 0,
         reinterpret_cast<uint32_t *>(static_cast<char *>(d) + offset), count, value);
  return check_launch(ctx, "buffer fill");
}

int byo_ctx_synchronize(byo_ctx *ctx) {
  if (!ctx) return BYO_EINVAL;
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  return BYO_OK;
}

// ---------------------------------------------------------------- containers

int byo_graph_create_csr(byo_ctx *ctx, uint64_t n, uint64_t m, const uint64_t *h_offsets,
                         const uint32_t *h_nbrs, byo_graph **out) {
  if (!ctx || !out) return BYO_EINVAL;
  *out = nullptr;
  return graph_from_host_csr(ctx, BYO_CONTAINER_CSR, n, m, h_offsets, h_nbrs, out);
}

int byo_graph_create_pma(byo_ctx *ctx, uint64_t n, uint64_t m, const uint64_t *h_offsets,
                         const uint32_t *h_nbrs, byo_graph **out) {
  if (!ctx || !out) return BYO_EINVAL;
  *out = nullptr;
  return graph_from_host_csr(ctx, BYO_CONTAINER_PMA, n, m, h_offsets, h_nbrs, out);
}

static bool known_container(int c) {
  return c == BYO_CONTAINER_CSR || c == BYO_CONTAINER_PMA || c == BYO_CONTAINER_VOS || c == BYO_CONTAINER_PCSR;
}

int byo_graph_create(byo_ctx *ctx, int container, uint64_t n, uint64_t m, const uint64_t *h_offsets,
                     const uint32_t *h_nbrs, byo_graph **out) {
  if (!ctx || !out) return BYO_EINVAL;
  *out = nullptr;
  if (!known_container(container))
    return set_error(ctx, BYO_EINVAL, "unknown container");
  return graph_from_host_csr(ctx, container, n, m, h_offsets, h_nbrs, out);
}

int byo_adj_read(const char *path, int binary, uint64_t *n, uint64_t *m, uint64_t *offsets, uint32_t *nbrs) {
  if (!path || !n || !m || (offsets && !nbrs && *m)) return BYO_EINVAL;
  return adj_read_host(nullptr, path, binary, n, m, offsets, nbrs);
}

int byo_graph_read_adj(byo_ctx *ctx, const char *path, int binary, int container, byo_graph **out) {
  if (!ctx || !path || !out) return BYO_EINVAL;
  *out = nullptr;
  if (!known_container(container))
    return set_error(ctx, BYO_EINVAL, "unknown container");
  uint64_t n = 0, m = 0;
  BYO_TRY(adj_read_host(ctx, path, binary, &n, &m, nullptr, nullptr));
  std::vector<uint64_t> off(n + 1);
  std::vector<uint32_t> nb(m ? m : 1);
  BYO_TRY(adj_read_host(ctx, path, binary, &n, &m, off.data(), nb.data()));
  return graph_from_host_csr(ctx, container, n, m, off.data(), nb.data(), out);
}

int byo_graph_from_bytepd(byo_ctx *ctx, uint64_t n, const uint64_t *byte_offsets, const uint32_t *degrees,
                          const uint8_t *bytes, uint64_t nbytes, uint32_t block, int container, byo_graph **out) {
  if (!ctx || !out) return BYO_EINVAL;
  *out = nullptr;
  if (!known_container(container))
    return set_error(ctx, BYO_EINVAL, "unknown container");
  return graph_from_bytepd_host(ctx, n, byte_offsets, degrees, bytes, nbytes, block ? block : 1000, container, out);
}

int byo_graph_read_bytepd(byo_ctx *ctx, const char *path, uint32_t block, int container, byo_graph **out) {
  if (!ctx || !path || !out) return BYO_EINVAL;
  *out = nullptr;
  if (!known_container(container))
    return set_error(ctx, BYO_EINVAL, "unknown container");
  return bytepd_read_file(ctx, path, block ? block : 1000, container, out);
}

int byo_graph_write_bytepd(byo_graph *g, const char *path, uint32_t block) {
  if (!g || !path) return BYO_EINVAL;
  return bytepd_write_file(g, path, block ? block : 1000);
}

int byo_graph_encode_bytepd(byo_graph *g, uint32_t block, uint64_t *byte_offsets, uint32_t *degrees, uint8_t *bytes,
                            uint64_t *nbytes) {
  if (!g || !nbytes) return BYO_EINVAL;
  return bytepd_encode_host(g, block ? block : 1000, byte_offsets, degrees, bytes, nbytes);
}

int byo_graph_write_adj(byo_graph *g, const char *path, int binary) {
  if (!g || !path) return BYO_EINVAL;
  std::vector<uint64_t> off(g->n + 1);
  std::vector<uint32_t> nb(g->m ? g->m : 1);
  BYO_TRY(byo_graph_export_csr(g, off.data(), nb.data()));
  return adj_write_host(g->ctx, path, binary, g->n, g->m, off.data(), nb.data());
}

int byo_graph_generate(byo_ctx *ctx, int container, const byo_gen_spec *spec, byo_graph **out) {
  if (!ctx || !out) return BYO_EINVAL;
  *out = nullptr;
  if (!known_container(container))
    return set_error(ctx, BYO_EINVAL, "unknown container");
  return graph_generate(ctx, container, spec, out);
}

void byo_graph_destroy(byo_graph *g) {
  if (!g) return;
  if (g->ctx && g->ctx->stream) cudaStreamSynchronize(g->ctx->stream);
  if (g->snap) {
    g->snap->d_deg = nullptr;  // the container's, freed below
    byo_graph_destroy(g->snap);
    g->snap = nullptr;
  }
  for (auto &b : g->ws) free_buf(b);
  if (g->pma) pma_destroy(g->pma);
  else if (g->pcsr) pcsr_destroy(g->pcsr);  // owns d_slots
  else if (g->d_slots) cudaFree(g->d_slots);
  if (g->vos) vos_destroy(g->vos);
  if (g->d_off) cudaFree(g->d_off);
  if (g->d_deg) cudaFree(g->d_deg);
  delete g;
}

int byo_graph_container(const byo_graph *g) { return g ? g->container : BYO_EINVAL; }
uint64_t byo_graph_num_vertices(const byo_graph *g) { return g ? g->n : 0; }
uint64_t byo_graph_num_edges(const byo_graph *g) { return g ? g->m : 0; }
uint64_t byo_graph_num_slots(const byo_graph *g) { return g ? g->nslots : 0; }

int byo_graph_degrees(byo_graph *g, uint32_t *h_out) {
  if (!g || !h_out) return BYO_EINVAL;
  return copy_to_host(g->ctx, h_out, g->d_deg, g->n * 4);
}

__global__ void k_compact_slots(const uint64_t *__restrict__ off, const uint32_t *__restrict__ slots,
                                const uint64_t *__restrict__ out_off, uint64_t n, uint32_t *out) {
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const unsigned lane = threadIdx.x & 31;
  for (uint64_t v = gw; v < n; v += nw) {
    uint64_t w = out_off[v];
    for (uint64_t base = off[v]; base < off[v + 1]; base += 32) {
      uint64_t j = base + lane;
      uint32_t u = j < off[v + 1] ? slots[j] : kSentinel;
      bool keep = u != kSentinel;
      unsigned m = __ballot_sync(0xFFFFFFFFu, keep);
      if (keep) out[w + __popc(m & ((1u << lane) - 1))] = u;
      w += __popc(m);
    }
  }
}

int byo_graph_export_csr(byo_graph *g, uint64_t *h_offsets, uint32_t *h_nbrs) {
  if (!g || !h_offsets || (g->m && !h_nbrs)) return BYO_EINVAL;
  byo_ctx *ctx = g->ctx;
  uint64_t *d_off2 = nullptr;
  uint32_t *d_n2 = nullptr;
  BYO_TRY(ws(g, WS_SCAN, g->n + 1, &d_off2));
  BYO_TRY(ws(g, WS_TC_NBR, g->m + 1, &d_n2));
  BYO_TRY(scan_u32_to_u64(ctx, g->d_deg, g->n, d_off2));
  launch(ctx, k_compact_slots, dim3(grid_for(ctx, g->n * 32, 256, 16)), dim3(256), 0,
         (const uint64_t *)g->d_off, (const uint32_t *)g->d_slots, (const uint64_t *)d_off2, g->n, d_n2);
  BYO_TRY(check_launch(ctx, "export_csr"));
  BYO_TRY(copy_to_host(ctx, h_offsets, d_off2, (g->n + 1) * 8));
  if (h_offsets[g->n] != g->m) return set_error(ctx, BYO_EDEVICE, "export: degree sum != m");
  return copy_to_host(ctx, h_nbrs, d_n2, g->m * 4);
}

int byo_graph_neighbors(byo_graph *g, uint32_t v, uint32_t *h_out, uint64_t cap, uint64_t *deg) {
  if (!g || v >= g->n) return g ? set_error(g->ctx, BYO_EINVAL, "vertex out of range") : BYO_EINVAL;
  byo_ctx *ctx = g->ctx;
  uint64_t range[2];
  uint32_t d = 0;
  BYO_CU(ctx, cudaMemcpyAsync(range, g->d_off + v, 16, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaMemcpyAsync(&d, g->d_deg + v, 4, cudaMemcpyDeviceToHost, ctx->stream));
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  if (deg) *deg = d;
  if (!h_out || cap == 0) return BYO_OK;
  uint64_t len = range[1] - range[0];
  uint32_t *tmp = new (std::nothrow) uint32_t[len ? len : 1];
  if (!tmp) return set_error(ctx, BYO_ENOMEM, "host buffer");
  int rc = copy_to_host(ctx, tmp, g->d_slots + range[0], len * 4);
  uint64_t w = 0;
  for (uint64_t i = 0; rc == BYO_OK && i < len && w < cap; i++)
    if (tmp[i] != kSentinel) h_out[w++] = tmp[i];
  delete[] tmp;
  return rc;
}

static int update_common(byo_graph *g, const uint64_t *keys, uint64_t count, int sorted, int insert,
                         int host, uint64_t *changed) {
  if (!g) return BYO_EINVAL;
  byo_ctx *ctx = g->ctx;
  if (changed) *changed = 0;
  if (g->container != BYO_CONTAINER_PMA && g->container != BYO_CONTAINER_VOS && g->container != BYO_CONTAINER_PCSR)
    return set_error(ctx, BYO_ENOTSUP, "batch updates need the PMA, VOS or PCSR container");
  g->upd = UpdateStats{};
  if (count == 0) return BYO_OK;
  if (!keys) return set_error(ctx, BYO_EINVAL, "null keys");
  const uint64_t *d = keys;
  if (host) {
    uint64_t *buf = nullptr;
    BYO_TRY(ws(g, WS_TC_OFF, count, &buf));
    BYO_CU(ctx, cudaMemcpyAsync(buf, keys, count * 8, cudaMemcpyHostToDevice, ctx->stream));
    d = buf;
  }
  if (g->container == BYO_CONTAINER_VOS) return vos_update(g, d, count, sorted, insert, changed);
  if (g->container == BYO_CONTAINER_PCSR) return pcsr_update(g, d, count, sorted, insert, changed);
  return pma_update(g, d, count, sorted, insert, changed);
}

static int update_stream_common(byo_graph *g, const uint64_t *keys, int host, const uint64_t *h_offsets,
                                const uint8_t *h_ops, uint64_t nbatch, uint64_t *changed,
                                const StreamQueries *qs = nullptr) {
  if (!g || (nbatch && (!h_offsets || !h_ops))) return BYO_EINVAL;
  byo_ctx *ctx = g->ctx;
  if (g->container != BYO_CONTAINER_PMA && g->container != BYO_CONTAINER_VOS && g->container != BYO_CONTAINER_PCSR)
    return set_error(ctx, BYO_ENOTSUP, "batch updates need the PMA, VOS or PCSR container");
  if (!nbatch) return BYO_OK;
  if (h_offsets[0] != 0) return set_error(ctx, BYO_EINVAL, "update stream: offsets[0] != 0");
  for (uint64_t b = 0; b < nbatch; b++)
    if (h_offsets[b + 1] < h_offsets[b]) return set_error(ctx, BYO_EINVAL, "update stream: offsets decrease");
  // the update stream inserts on any nonzero op; the mixed stream reads
  // 0 remove, 1 insert, 2 query
  uint64_t nq = 0;
  for (uint64_t b = 0; qs && b < nbatch; b++) {
    if (h_ops[b] > BYO_OP_QUERY) return set_error(ctx, BYO_EINVAL, "mixed stream: unknown op");
    if (h_ops[b] == BYO_OP_QUERY) {
      if (h_offsets[b + 1] != h_offsets[b]) return set_error(ctx, BYO_EINVAL, "mixed stream: a query op holds keys");
      nq++;
    }
  }
  if (nq) {
    if (qs->k == 0 || qs->k > 64) return set_error(ctx, BYO_EINVAL, "mixed stream: 1 <= k <= 64 sources");
    if (!qs->h_srcs || !qs->d_levels) return set_error(ctx, BYO_EINVAL, "mixed stream: null sources or levels");
    if (g->n >= (1ull << 32) - 1) return set_error(ctx, BYO_EINVAL, "mixed stream: n too large");
    for (uint64_t i = 0; i < nq * qs->k; i++)
      if (qs->h_srcs[i] >= g->n) return set_error(ctx, BYO_EINVAL, "mixed stream: source >= n");
  }
  const uint64_t total = h_offsets[nbatch];
  if (total && !keys) return set_error(ctx, BYO_EINVAL, "update stream: null keys");
  const uint64_t *d = keys;
  if (host) {
    uint64_t *buf = nullptr;
    BYO_TRY(ws(g, WS_TC_OFF, total ? total : 1, &buf));
    if (total) BYO_CU(ctx, cudaMemcpyAsync(buf, keys, total * 8, cudaMemcpyHostToDevice, ctx->stream));
    d = buf;
  }
  uint64_t *sb = nullptr;
  BYO_TRY(ws(g, WS_STREAM, (nbatch + 1) + (nbatch + 7) / 8, &sb));
  BYO_CU(ctx, cudaMemcpyAsync(sb, h_offsets, (nbatch + 1) * 8, cudaMemcpyHostToDevice, ctx->stream));
  unsigned char *d_ops = reinterpret_cast<unsigned char *>(sb + nbatch + 1);
  std::vector<unsigned char> ops(nbatch);
  for (uint64_t b = 0; b < nbatch; b++) ops[b] = qs && h_ops[b] == BYO_OP_QUERY ? BYO_OP_QUERY : (h_ops[b] ? 1 : 0);
  BYO_CU(ctx, cudaMemcpyAsync(d_ops, ops.data(), nbatch, cudaMemcpyHostToDevice, ctx->stream));
  std::vector<long long> ch(nbatch);
  int rc = BYO_OK;
  if (g->container != BYO_CONTAINER_PMA) {  // VOS, PCSR: one op at a time
    uint64_t q = 0;
    for (uint64_t b = 0; b < nbatch && rc == BYO_OK; b++) {
      uint64_t c = 0;
      const uint64_t len = h_offsets[b + 1] - h_offsets[b];
      if (ops[b] == BYO_OP_QUERY) {
        byo_graph *t = nullptr;
        uint32_t rounds = 0;
        rc = traversal_view(g, &t);
        if (rc == BYO_OK)
          rc = bfs_multi_run(t, qs->h_srcs + q * qs->k, qs->k, qs->d_levels + q * qs->k * g->n, &rounds);
        q++;
      } else if (len && g->container == BYO_CONTAINER_VOS) {
        rc = vos_update(g, d + h_offsets[b], len, 0, ops[b], &c);
      } else if (len) {
        rc = pcsr_update(g, d + h_offsets[b], len, 0, ops[b], &c);
      }
      ch[b] = (long long)c;
    }
  } else {
    rc = pma_update_stream(g, d, sb, h_offsets, d_ops, ops.data(), nbatch, ch.data(), qs);
  }
  if (changed)
    for (uint64_t b = 0; b < nbatch; b++) changed[b] = (uint64_t)ch[b];
  return rc;
}

static int mixed_common(byo_graph *g, const uint64_t *keys, int host, const uint64_t *offsets, const uint8_t *ops,
                        uint64_t nops, const uint32_t *h_srcs, uint32_t k, uint32_t *d_levels, uint64_t *changed,
                        uint64_t *op_ns) {
  if (!g) return BYO_EINVAL;
  if (op_ns)
    for (uint64_t b = 0; b < 2 * nops; b++) op_ns[b] = 0;
  StreamQueries qs{h_srcs, k, d_levels, op_ns};
  return update_stream_common(g, keys, host, offsets, ops, nops, changed, &qs);
}

int byo_graph_mixed_stream(byo_graph *g, const uint64_t *h_keys, const uint64_t *offsets, const uint8_t *ops,
                           uint64_t nops, const uint32_t *h_srcs, uint32_t k, uint32_t *d_levels, uint64_t *changed,
                           uint64_t *op_ns) {
  return mixed_common(g, h_keys, 1, offsets, ops, nops, h_srcs, k, d_levels, changed, op_ns);
}

int byo_graph_mixed_stream_device(byo_graph *g, const uint64_t *d_keys, const uint64_t *offsets, const uint8_t *ops,
                                  uint64_t nops, const uint32_t *h_srcs, uint32_t k, uint32_t *d_levels,
                                  uint64_t *changed, uint64_t *op_ns) {
  return mixed_common(g, d_keys, 0, offsets, ops, nops, h_srcs, k, d_levels, changed, op_ns);
}

int byo_graph_update_stream(byo_graph *g, const uint64_t *h_keys, const uint64_t *offsets, const uint8_t *ops,
                            uint64_t nbatch, uint64_t *changed) {
  return update_stream_common(g, h_keys, 1, offsets, ops, nbatch, changed);
}
int byo_graph_update_stream_device(byo_graph *g, const uint64_t *d_keys, const uint64_t *offsets, const uint8_t *ops,
                                   uint64_t nbatch, uint64_t *changed) {
  return update_stream_common(g, d_keys, 0, offsets, ops, nbatch, changed);
}

int byo_graph_last_update_stats(const byo_graph *g, byo_update_stats *out) {
  if (!g || !out) return BYO_EINVAL;
  *out = byo_update_stats{};
  out->keys = g->upd.keys;
  out->changed = g->upd.changed;
  out->touched_leaves = g->upd.leaves;
  out->touched_entries = g->upd.entries;
  out->leaf_slots = g->container == BYO_CONTAINER_PMA    ? pma_leaf_slots()
                    : g->container == BYO_CONTAINER_PCSR ? pcsr_leaf_slots()
                                                         : 0;
  out->path = g->upd.path;
  return BYO_OK;
}

int byo_graph_insert_batch(byo_graph *g, const uint64_t *h_keys, uint64_t count, int sorted,
                           uint64_t *changed) {
  return update_common(g, h_keys, count, sorted, 1, 1, changed);
}
int byo_graph_remove_batch(byo_graph *g, const uint64_t *h_keys, uint64_t count, int sorted,
                           uint64_t *changed) {
  return update_common(g, h_keys, count, sorted, 0, 1, changed);
}
int byo_graph_insert_batch_device(byo_graph *g, const uint64_t *d_keys, uint64_t count, int sorted,
                                  uint64_t *changed) {
  return update_common(g, d_keys, count, sorted, 1, 0, changed);
}
int byo_graph_remove_batch_device(byo_graph *g, const uint64_t *d_keys, uint64_t count, int sorted,
                                  uint64_t *changed) {
  return update_common(g, d_keys, count, sorted, 0, 0, changed);
}

// ---------------------------------------------------------------- generators

int byo_gen_rmat_pairs_device(byo_ctx *ctx, uint64_t seed, uint32_t lg_n, double a, double b, double c,
                              uint64_t first, uint64_t count, uint32_t *d_src, uint32_t *d_dst) {
  if (!ctx) return BYO_EINVAL;
  return gen_rmat_pairs(ctx, seed, lg_n, a, b, c, first, count, d_src, d_dst);
}
int byo_gen_uniform_pairs_device(byo_ctx *ctx, uint64_t seed, uint64_t n, uint64_t first, uint64_t count,
                                 uint32_t *d_src, uint32_t *d_dst) {
  if (!ctx) return BYO_EINVAL;
  return gen_uniform_pairs(ctx, seed, n, first, count, d_src, d_dst);
}
int byo_gen_uniform_keys_device(byo_ctx *ctx, uint64_t seed, uint64_t n, uint64_t count, uint64_t *d_keys) {
  if (!ctx) return BYO_EINVAL;
  return gen_uniform_keys(ctx, seed, n, count, d_keys);
}

// ---------------------------------------------------------------- algorithms

int byo_bfs_device(byo_graph *g, uint32_t src, uint32_t *d_parent, uint32_t *d_level, int policy,
                   uint32_t *rounds) {
  if (!g) return BYO_EINVAL;
  BYO_TRY(need(g->ctx, policy >= 0 && policy <= BYO_POLICY_M20_BLOCKED, "unknown policy"));
  byo_graph *t = nullptr;
  BYO_TRY(traversal_view(g, &t));
  return bfs_run(t, src, d_parent, d_level, policy, rounds);
}

int byo_bfs(byo_graph *g, uint32_t src, uint32_t *h_parent, uint32_t *h_level, int policy,
            uint32_t *rounds) {
  if (!g) return BYO_EINVAL;
  byo_ctx *ctx = g->ctx;
  uint32_t *d = nullptr;
  BYO_TRY(ws(g, WS_LABEL, 2 * g->n + 2, &d));
  uint32_t *dp = h_parent ? d : nullptr, *dl = h_level ? d + g->n : nullptr;
  BYO_TRY(byo_bfs_device(g, src, dp, dl, policy, rounds));
  if (h_parent) BYO_TRY(copy_to_host(ctx, h_parent, dp, g->n * 4));
  if (h_level) BYO_TRY(copy_to_host(ctx, h_level, dl, g->n * 4));
  return BYO_OK;
}

int byo_bfs_multi_device(byo_graph *g, const uint32_t *h_srcs, uint32_t k, uint32_t *d_levels, uint32_t *rounds) {
  if (!g || !h_srcs || !d_levels) return BYO_EINVAL;
  byo_graph *t = nullptr;
  BYO_TRY(traversal_view(g, &t));
  return bfs_multi_run(t, h_srcs, k, d_levels, rounds);
}

int byo_bfs_multi(byo_graph *g, const uint32_t *h_srcs, uint32_t k, uint32_t *h_levels, uint32_t *rounds) {
  if (!g || !h_srcs || !h_levels) return BYO_EINVAL;
  uint32_t *d = nullptr;
  BYO_TRY(ws(g, WS_TC_NBR, (uint64_t)k * g->n + 1, &d));
  byo_graph *t = nullptr;
  BYO_TRY(traversal_view(g, &t));
  BYO_TRY(bfs_multi_run(t, h_srcs, k, d, rounds));
  return copy_to_host(g->ctx, h_levels, d, (uint64_t)k * g->n * 4);
}

int byo_graph_get_tuning(byo_graph *g, byo_tuning *out) {
  if (!g || !out) return BYO_EINVAL;
  *out = effective_tuning(g);
  return BYO_OK;
}

int byo_graph_set_tuning(byo_graph *g, const byo_tuning *t) {
  if (!g || !t) return BYO_EINVAL;
  BYO_TRY(check_tuning(g->ctx, t));
  g->tune = *t;
  return BYO_OK;
}

int byo_graph_autotune(byo_graph *g, uint32_t what, uint32_t trials, byo_tuning *out) {
  if (!g) return BYO_EINVAL;
  BYO_TRY(need(g->ctx, what != 0 && (what & ~(BYO_TUNE_BFS | BYO_TUNE_MULTI)) == 0, "autotune: unknown flags"));
  BYO_TRY(autotune(g, what, trials));
  if (out) *out = effective_tuning(g);
  return BYO_OK;
}

int byo_cc_device(byo_graph *g, uint32_t *d_label) {
  if (!g || !d_label) return BYO_EINVAL;
  byo_graph *t = nullptr;
  BYO_TRY(traversal_view(g, &t));
  return cc_run(t, d_label);
}

int byo_cc(byo_graph *g, uint32_t *h_label) {
  if (!g || !h_label) return BYO_EINVAL;
  uint32_t *d = nullptr;
  BYO_TRY(ws(g, WS_PR_A, g->n + 1, &d));
  byo_graph *t = nullptr;
  BYO_TRY(traversal_view(g, &t));
  BYO_TRY(cc_run(t, d));
  return copy_to_host(g->ctx, h_label, d, g->n * 4);
}

int byo_bfs_cc(byo_graph *g, uint32_t *h_label) {
  if (!g || !h_label) return BYO_EINVAL;
  uint32_t *d = nullptr;
  BYO_TRY(ws(g, WS_PR_B, g->n + 1, &d));
  byo_graph *t = nullptr;
  BYO_TRY(traversal_view(g, &t));
  BYO_TRY(bfs_cc_run(t, d));
  return copy_to_host(g->ctx, h_label, d, g->n * 4);
}

int byo_pagerank_device(byo_graph *g, double eps, uint32_t max_iters, int precision, double *d_p,
                        uint32_t *iters, double *l1) {
  if (!g || !d_p) return BYO_EINVAL;
  byo_graph *t = nullptr;
  BYO_TRY(traversal_view(g, &t));
  return pagerank_run(t, eps, max_iters, precision, d_p, iters, l1);
}

int byo_pagerank_edgemap(byo_graph *g, double eps, uint32_t max_iters, double *h_p, uint32_t *iters,
                         double *l1) {
  if (!g || !h_p) return BYO_EINVAL;
  if (g->n == 0) return BYO_OK;
  double *d = nullptr;
  BYO_TRY(host_out_buffer(g, g->n, &d));
  BYO_TRY(pagerank_edgemap_run(g, eps, max_iters, d, iters, l1));
  return copy_to_host(g->ctx, h_p, d, g->n * 8);
}

int byo_pagerank_delta_device(byo_graph *g, double eps, double local_eps, uint32_t max_iters, double *d_p,
                              uint32_t *rounds, double *l1) {
  if (!g || !d_p) return BYO_EINVAL;
  byo_graph *t = nullptr;
  BYO_TRY(traversal_view(g, &t));
  return pagerank_delta_run(t, eps, local_eps, max_iters, d_p, rounds, l1);
}

int byo_pagerank_delta(byo_graph *g, double eps, double local_eps, uint32_t max_iters, double *h_p,
                       uint32_t *rounds, double *l1) {
  if (!g || !h_p) return BYO_EINVAL;
  double *d = nullptr;
  BYO_TRY(ws(g, WS_TC_CNT, 2 * g->n + 2, (uint32_t **)&d));
  byo_graph *t = nullptr;
  BYO_TRY(traversal_view(g, &t));
  BYO_TRY(pagerank_delta_run(t, eps, local_eps, max_iters, d, rounds, l1));
  return copy_to_host(g->ctx, h_p, d, g->n * 8);
}

int byo_pagerank(byo_graph *g, double eps, uint32_t max_iters, int precision, double *h_p, uint32_t *iters,
                 double *l1) {
  if (!g || !h_p) return BYO_EINVAL;
  double *d = nullptr;
  BYO_TRY(ws(g, WS_TC_CNT, 2 * g->n + 2, (uint32_t **)&d));
  byo_graph *t = nullptr;
  BYO_TRY(traversal_view(g, &t));
  BYO_TRY(pagerank_run(t, eps, max_iters, precision, d, iters, l1));
  return copy_to_host(g->ctx, h_p, d, g->n * 8);
}

int byo_triangle_count(byo_graph *g, uint64_t *count) {
  if (!g || !count) return BYO_EINVAL;
  byo_graph *t = nullptr;
  BYO_TRY(traversal_view(g, &t));
  return tc_run(t, count);
}

// ---------------------------------------------------------------- neighbour maps

int byo_map_sum(byo_graph *g, uint64_t *sum) {
  if (!g || !sum) return BYO_EINVAL;
  return map_run(g, -1, nullptr, sum);
}

int byo_map_remote_device(byo_graph *g, const void *d_remote, uint32_t width, uint64_t *sum) {
  if (!g || !sum || (!d_remote && g->n)) return BYO_EINVAL;
  return map_run(g, (int)width, d_remote, sum);
}

int byo_map_remote(byo_graph *g, const void *h_remote, uint32_t width, uint64_t *sum) {
  if (!g || !sum || (!h_remote && g->n)) return BYO_EINVAL;
  if (width > 32 || (width & (width - 1)))
    return set_error(g->ctx, BYO_EINVAL, "map: remote width must be 0, 1, 2, 4, 8, 16 or 32");
  const uint64_t bytes = map_remote_bytes(g->n, width);
  uint64_t *d = nullptr;
  BYO_TRY(ws(g, WS_TC_NBR, bytes / 8 + 1, &d));
  if (bytes) BYO_CU(g->ctx, cudaMemcpyAsync(d, h_remote, bytes, cudaMemcpyHostToDevice, g->ctx->stream));
  return map_run(g, (int)width, d, sum);
}

// ---------------------------------------------------------------- edgeMap API

int byo_functor_bfs_create(byo_graph *g, uint32_t src, byo_functor **out) {
  if (!g || !out) return BYO_EINVAL;
  *out = nullptr;
  if (src >= g->n) return set_error(g->ctx, BYO_EINVAL, "src >= n");
  byo_functor *f = new (std::nothrow) byo_functor();
  if (!f) return BYO_ENOMEM;
  f->g = g;
  const uint64_t W = (g->n + 31) / 32;
  int rc = ensure(g->ctx, f->lp, g->n * 8);
  if (rc == BYO_OK) rc = ensure(g->ctx, f->visited, W * 4);
  if (rc == BYO_OK) {
    f->st.lp = (uint64_t *)f->lp.p;
    f->st.visited = (uint32_t *)f->visited.p;
    rc = trav_init(g, f->st, src);
  }
  if (rc != BYO_OK) {
    byo_functor_destroy(f);
    return rc;
  }
  *out = f;
  return BYO_OK;
}

int byo_functor_bfs_parents(byo_functor *f, uint32_t *h_parents) {
  if (!f || !h_parents) return BYO_EINVAL;
  byo_graph *g = f->g;
  uint32_t *d = nullptr;
  BYO_TRY(ws(g, WS_LABEL, g->n + 1, &d));
  BYO_TRY(trav_extract(g, f->st, d, nullptr));
  return copy_to_host(g->ctx, h_parents, d, g->n * 4);
}

static int functor_new(byo_graph *g, const FunctorArgs &fa, byo_functor **out) {
  byo_functor *f = new (std::nothrow) byo_functor();
  if (!f) return set_error(g->ctx, BYO_ENOMEM, "functor");
  f->g = g;
  f->kind = fa.kind;
  f->fa = fa;
  *out = f;
  return BYO_OK;
}

int byo_functor_bfs_label_create(byo_graph *g, uint32_t src, uint32_t *d_parents, byo_functor **out) {
  if (!g || !out || !d_parents) return BYO_EINVAL;
  *out = nullptr;
  if (src >= g->n) return set_error(g->ctx, BYO_EINVAL, "src >= n");
  FunctorArgs fa;
  fa.kind = BYO_F_BFS_LABEL;
  fa.parents = d_parents;
  fa.src = src;
  return functor_new(g, fa, out);
}

int byo_functor_pr_create(byo_graph *g, const double *d_p_curr, double *d_p_next, byo_functor **out) {
  if (!g || !out || !d_p_curr || !d_p_next) return BYO_EINVAL;
  *out = nullptr;
  FunctorArgs fa;
  fa.kind = BYO_F_PR;
  fa.p_curr = d_p_curr;
  fa.p_next = d_p_next;
  return functor_new(g, fa, out);
}

int byo_functor_pr_delta_create(byo_graph *g, const double *d_delta, double *d_ngh_sum, byo_functor **out) {
  if (!g || !out || !d_delta || !d_ngh_sum) return BYO_EINVAL;
  *out = nullptr;
  FunctorArgs fa;
  fa.kind = BYO_F_PR_DELTA;
  fa.delta = d_delta;
  fa.ngh = d_ngh_sum;
  return functor_new(g, fa, out);
}

int byo_functor_kind(const byo_functor *f) { return f ? f->kind : BYO_EINVAL; }

void byo_functor_destroy(byo_functor *f) {
  if (!f) return;
  if (f->g && f->g->ctx) cudaStreamSynchronize(f->g->ctx->stream);
  free_buf(f->lp);
  free_buf(f->visited);
  delete f;
}

static int vs_alloc(byo_graph *g, byo_vertex_subset **out) {
  byo_vertex_subset *vs = new (std::nothrow) byo_vertex_subset();
  if (!vs) return BYO_ENOMEM;
  vs->g = g;
  const uint64_t W = (g->n + 31) / 32;
  int rc = ensure(g->ctx, vs->list, g->n * 4);
  if (rc == BYO_OK) rc = ensure(g->ctx, vs->bits, W * 4);
  if (rc != BYO_OK) {
    byo_vs_destroy(vs);
    return rc;
  }
  vs->f.list = (uint32_t *)vs->list.p;
  vs->f.bits = (uint32_t *)vs->bits.p;
  *out = vs;
  return BYO_OK;
}

__global__ void k_sum_deg(const uint32_t *__restrict__ list, uint64_t cnt, const uint32_t *__restrict__ deg,
                          unsigned long long *out) {
  unsigned long long s = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt;
       i += (uint64_t)gridDim.x * blockDim.x)
    s += deg[list[i]];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, s);
}

int byo_vs_create_list(byo_graph *g, const uint32_t *h_ids, uint64_t count, byo_vertex_subset **out) {
  if (!g || !out || (count && !h_ids)) return BYO_EINVAL;
  *out = nullptr;
  byo_ctx *ctx = g->ctx;
  if (count > g->n) return set_error(ctx, BYO_EINVAL, "subset larger than n");
  for (uint64_t i = 0; i < count; i++)
    if (h_ids[i] >= g->n) return set_error(ctx, BYO_EINVAL, "vertex id >= n");
  byo_vertex_subset *vs = nullptr;
  BYO_TRY(vs_alloc(g, &vs));
  int rc = BYO_OK;
  if (count) {
    cudaError_t e = cudaMemcpyAsync(vs->f.list, h_ids, count * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) rc = set_error(ctx, BYO_EDEVICE, "upload subset", e);
  }
  unsigned long long *d_sum = nullptr;
  if (rc == BYO_OK) rc = ws(g, WS_MISC, 4, (uint32_t **)&d_sum);
  if (rc == BYO_OK) {
    cudaMemsetAsync(d_sum, 0, 8, ctx->stream);
    if (count)
      launch(ctx, k_sum_deg, dim3(grid_for(ctx, count, 256)), dim3(256), 0, (const uint32_t *)vs->f.list, count,
             (const uint32_t *)g->d_deg, d_sum);
    unsigned long long h = 0;
    cudaMemcpyAsync(&h, d_sum, 8, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = set_error(ctx, BYO_EDEVICE, "subset degrees", e);
    vs->f.outdeg = h;
  }
  if (rc != BYO_OK) {
    byo_vs_destroy(vs);
    return rc;
  }
  vs->f.size = count;
  vs->f.has_list = true;
  vs->f.has_bits = false;
  vs->f.dense = false;
  *out = vs;
  return BYO_OK;
}

int byo_vs_create_single(byo_graph *g, uint32_t v, byo_vertex_subset **out) {
  return byo_vs_create_list(g, &v, 1, out);
}

int byo_vs_create_bitmap(byo_graph *g, const uint32_t *d_bits, byo_vertex_subset **out) {
  if (!g || !out) return BYO_EINVAL;
  *out = nullptr;
  byo_vertex_subset *vs = nullptr;
  BYO_TRY(vs_alloc(g, &vs));
  int rc = frontier_from_bits(g, d_bits, vs->f);
  if (rc != BYO_OK) {
    byo_vs_destroy(vs);
    return rc;
  }
  *out = vs;
  return BYO_OK;
}

int byo_vs_create_all(byo_graph *g, byo_vertex_subset **out) { return byo_vs_create_bitmap(g, nullptr, out); }

void byo_vs_destroy(byo_vertex_subset *vs) {
  if (!vs) return;
  if (vs->g && vs->g->ctx) cudaStreamSynchronize(vs->g->ctx->stream);
  free_buf(vs->list);
  free_buf(vs->bits);
  delete vs;
}

uint64_t byo_vs_size(const byo_vertex_subset *vs) { return vs ? vs->f.size : 0; }
int byo_vs_is_dense(const byo_vertex_subset *vs) { return vs ? (vs->f.dense ? 1 : 0) : BYO_EINVAL; }

int byo_vs_to_list(byo_vertex_subset *vs, uint32_t *h_out, uint64_t cap) {
  if (!vs || (vs->f.size && !h_out)) return BYO_EINVAL;
  byo_ctx *ctx = vs->g->ctx;
  if (cap < vs->f.size) return set_error(ctx, BYO_EINVAL, "output smaller than the subset");
  if (!vs->f.size) return BYO_OK;
  // toSparse order: increasing ids
  uint64_t *keys = nullptr, *tmp = nullptr, *sorted = nullptr;
  BYO_TRY(ws(vs->g, WS_TC_OFF, 2 * vs->f.size + 2, &keys));
  tmp = keys + vs->f.size + 1;
  std::vector<uint32_t> h(vs->f.size);
  BYO_TRY(copy_to_host(ctx, h.data(), vs->f.list, vs->f.size * 4));
  std::vector<uint64_t> k(h.begin(), h.end());
  BYO_CU(ctx, cudaMemcpyAsync(keys, k.data(), k.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
  BYO_TRY(sort_u64(ctx, keys, tmp, vs->f.size, sig_mask_for(vs->g->n) & 0xFFFFFFFFull, &sorted));
  BYO_TRY(copy_to_host(ctx, k.data(), sorted, k.size() * 8));
  for (uint64_t i = 0; i < vs->f.size; i++) h_out[i] = (uint32_t)k[i];
  return BYO_OK;
}

int byo_edge_map(byo_graph *g, byo_vertex_subset *vs, byo_functor *f, int64_t threshold, uint32_t flags,
                 byo_vertex_subset **out) {
  if (!g || !vs || !f || !out) return BYO_EINVAL;
  *out = nullptr;
  byo_ctx *ctx = g->ctx;
  if (vs->g != g || f->g != g) return set_error(ctx, BYO_EINVAL, "subset / functor of another graph");
  byo_vertex_subset *o = nullptr;
  BYO_TRY(vs_alloc(g, &o));
  const uint64_t W = (g->n + 31) / 32;
  int rc = memset_async(ctx, o->f.bits, 0, W * 4);
  // edgeMapData, edge_map_data.h:254-307
  int mode = MODE_PUSH;
  bool empty = vs->f.size == 0;
  if (!empty) {
    if ((flags & BYO_FL_DENSE_ONLY) || (vs->f.dense && vs->f.size > g->n / 10)) {
      mode = (flags & BYO_FL_DENSE_FORWARD) ? MODE_DENSE_FWD : MODE_PULL;
    } else if (vs->f.outdeg == 0) {
      empty = true;
    } else {
      const int sparse = (flags & BYO_FL_SPARSE_BLOCKED) ? MODE_BLOCKED : MODE_PUSH;
      mode = m20_mode(g, vs->f, threshold, sparse);
      if (mode == MODE_PULL && (flags & BYO_FL_NO_DENSE)) mode = sparse;
      if (mode == MODE_PULL && (flags & BYO_FL_DENSE_FORWARD)) mode = MODE_DENSE_FWD;
    }
  }
  if (rc == BYO_OK && !empty) {
    if (f->kind == BYO_F_BFS) {
      EngineTuning tune = default_tuning(g);
      rc = edge_map_round(g, f->st, vs->f, o->f, mode, tune);
    } else {
      rc = generic_edge_map(g, f->fa, vs->f, o->f, mode, !(flags & BYO_FL_NO_OUTPUT));
    }
  } else if (rc == BYO_OK) {
    o->f.size = 0;
    o->f.has_list = o->f.has_bits = true;
  }
  if (rc == BYO_OK) rc = check_launch(ctx, "edge_map");
  if (rc != BYO_OK) {
    byo_vs_destroy(o);
    return rc;
  }
  if (flags & BYO_FL_NO_OUTPUT) {
    o->f.size = 0;
    o->f.outdeg = 0;
  }
  *out = o;
  return BYO_OK;
}

static int vop_args(byo_vertex_subset *vs, const byo_vertex_op *op, VertexOpArgs *a) {
  byo_ctx *ctx = vs->g->ctx;
  switch (op->kind) {
    case BYO_VOP_PR_UPDATE:
    case BYO_VOP_ZERO:
      if (!op->d_a) return set_error(ctx, BYO_EINVAL, "vertex op: d_a is null");
      break;
    case BYO_VOP_PR_DELTA_FIRST:
    case BYO_VOP_PR_DELTA:
      if (!op->d_a || !op->d_b || !op->d_c) return set_error(ctx, BYO_EINVAL, "vertex op: null array");
      break;
    default:
      return set_error(ctx, BYO_EINVAL, "vertex op: unknown kind");
  }
  *a = VertexOpArgs{op->kind, op->d_a, op->d_b, op->d_c, op->damping, op->eps2};
  return BYO_OK;
}

int byo_vertex_map(byo_vertex_subset *vs, const byo_vertex_op *op) {
  if (!vs || !op) return BYO_EINVAL;
  VertexOpArgs a;
  BYO_TRY(vop_args(vs, op, &a));
  return vertex_op_run(vs->g, a, vs->f, nullptr);
}

int byo_vertex_filter(byo_vertex_subset *vs, const byo_vertex_op *op, byo_vertex_subset **out) {
  if (!vs || !op || !out) return BYO_EINVAL;
  *out = nullptr;
  byo_graph *g = vs->g;
  VertexOpArgs a;
  BYO_TRY(vop_args(vs, op, &a));
  byo_vertex_subset *o = nullptr;
  BYO_TRY(vs_alloc(g, &o));
  int rc = memset_async(g->ctx, o->f.bits, 0, (g->n + 31) / 32 * 4);
  if (rc == BYO_OK) rc = vertex_op_run(g, a, vs->f, &o->f);
  if (rc != BYO_OK) {
    byo_vs_destroy(o);
    return rc;
  }
  *out = o;
  return BYO_OK;
}

int byo_last_rounds(byo_ctx *ctx, byo_round_log *out, uint64_t cap, uint64_t *count) {
  if (!ctx) return BYO_EINVAL;
  uint64_t n = ctx->rounds.size();
  if (count) *count = n;
  if (out)
    for (uint64_t i = 0; i < n && i < cap; i++) out[i] = ctx->rounds[i];
  return BYO_OK;
}

int byo_ctx_kernel_timing(byo_ctx *ctx, const char *tag) {
  if (!ctx) return BYO_EINVAL;
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->ktag = tag ? tag : "";
  ctx->kev_used = 0;
  ctx->ktags.clear();
  return BYO_OK;
}

int byo_ctx_kernel_time(byo_ctx *ctx, const char *tag, uint64_t *launches, double *ms) {
  if (!ctx) return BYO_EINVAL;
  BYO_CU(ctx, cudaStreamSynchronize(ctx->stream));
  double tot = 0.0;
  uint64_t cnt = 0;
  for (size_t i = 0; i + 1 < ctx->kev_used; i += 2) {
    if (tag && std::strcmp(tag, ctx->ktags[i / 2]) != 0) continue;
    float t = 0.f;
    BYO_CU(ctx, cudaEventElapsedTime(&t, ctx->kev[i], ctx->kev[i + 1]));
    tot += t;
    cnt++;
  }
  if (launches) *launches = cnt;
  if (ms) *ms = tot;
  return BYO_OK;
}

int byo_ctx_set_update_policy(byo_ctx *ctx, int policy) {
  if (!ctx) return BYO_EINVAL;
  if (policy != BYO_UPDATE_MERGE && policy != BYO_UPDATE_LEARNED && policy != BYO_UPDATE_REBUILD)
    return set_error(ctx, BYO_EINVAL, "unknown update policy");
  ctx->update_policy = policy;
  return BYO_OK;
}

// Times one batch both ways (in-place merge and rebuild), as insert and as
// remove, restoring the contents in between; two samples for the policy.
int byo_update_sample(byo_graph *g, const uint64_t *h_keys, uint64_t count, float *h_x, float *h_y,
                      uint8_t *h_mask) {
  if (!g || !h_keys || !count || !h_x || !h_y || !h_mask) return BYO_EINVAL;
  byo_ctx *ctx = g->ctx;
  if (g->container != BYO_CONTAINER_PMA) return set_error(ctx, BYO_ENOTSUP, "needs the PMA container");
  const int saved = ctx->update_policy;
  float t[4] = {0, 0, 0, 0};
  uint64_t m0 = g->m, slots0 = g->nslots;
  // an untimed merge pair first sizes every update buffer for this batch, so
  // no allocation falls inside a timed update
  ctx->update_policy = BYO_UPDATE_MERGE;
  int rc = update_common(g, h_keys, count, 0, 1, 1, nullptr);
  if (rc == BYO_OK) rc = update_common(g, h_keys, count, 0, 0, 1, nullptr);
  for (int k = 0; k < 4 && rc == BYO_OK; k++) {
    const int insert = (k % 2) == 0;
    ctx->update_policy = k < 2 ? BYO_UPDATE_MERGE : BYO_UPDATE_REBUILD;
    cudaEventRecord(ctx->ev[2], ctx->stream);
    rc = update_common(g, h_keys, count, 0, insert, 1, nullptr);
    cudaEventRecord(ctx->ev[3], ctx->stream);
    cudaEventSynchronize(ctx->ev[3]);
    cudaEventElapsedTime(&t[k], ctx->ev[2], ctx->ev[3]);
  }
  ctx->update_policy = saved;
  if (rc != BYO_OK) return rc;
  for (int s2 = 0; s2 < 2; s2++) {
    update_features(count, m0, slots0, 0, s2 == 0, h_x + 16 * s2);
    for (int o = 0; o < 5; o++) h_y[5 * s2 + o] = 0.f;
    const float merge_ms = t[s2], rebuild_ms = t[2 + s2];
    h_y[5 * s2 + 3] = std::log2(1.f + merge_ms * 1000.f) / 16.f;
    h_y[5 * s2 + 4] = std::log2(1.f + rebuild_ms * 1000.f) / 16.f;
    h_mask[s2] = (uint8_t)((1u << 3) | (1u << 4));
  }
  return BYO_OK;
}

int byo_ctx_last_update_strategy(const byo_ctx *ctx) { return ctx ? ctx->last_update_strategy : BYO_EINVAL; }

int byo_ctx_set_barrier_test(byo_ctx *ctx, uint32_t limit_ms, uint32_t extra_blocks) {
  if (!ctx) return BYO_EINVAL;
  if (limit_ms > 4000 || extra_blocks > 1)
    return set_error(ctx, BYO_EINVAL, "barrier test: limit_ms <= 4000 and extra_blocks <= 1");
  ctx->bar_limit_ms = limit_ms;
  ctx->bar_extra = extra_blocks;
  return BYO_OK;
}

int byo_ctx_set_pagerank_graphs(byo_ctx *ctx, int on) {
  if (!ctx) return BYO_EINVAL;
  ctx->pr_graphs = on != 0;
  return BYO_OK;
}

int byo_gather_roof(byo_ctx *ctx, uint64_t table_bytes, double *gathers_per_s) {
  if (!ctx || !gathers_per_s) return BYO_EINVAL;
  *gathers_per_s = 0.0;
  return gather_roof(ctx, table_bytes, gathers_per_s);
}

int byo_ctx_set_round_timing(byo_ctx *ctx, int on) {
  if (!ctx) return BYO_EINVAL;
  ctx->time_rounds = on != 0;
  return BYO_OK;
}

}  // extern "C"

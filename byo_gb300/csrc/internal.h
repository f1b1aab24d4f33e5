// internal.h -- shared host-side declarations of the byo_gpu library.
//
// Layout in HBM of a graph (both containers):
//   d_off   uint64[n+1]  slot range [d_off[v], d_off[v+1]) of vertex v
//   d_slots uint32[nslots] neighbour ids; the PMA leaves gaps marked kSentinel
//                        inside that range, a CSR has none
//   d_deg   uint32[n]    degree (non-gap entries) of every vertex
// so one family of traversal kernels serves the static CSR and the packed
// memory array alike.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/byo_gpu.h"

namespace byo {

constexpr uint32_t kSentinel = 0xFFFFFFFFu;
constexpr uint64_t kNone64 = ~0ull;

// A device buffer that only grows; freed with its owner.
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
};

struct Pma;  // pma.cu
struct Vos;  // vos.cu
struct Pcsr; // pcsr.cu
struct Mlp;  // mlp.cu

}  // namespace byo

struct byo_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  uint64_t launches = 0;
  void *pinned = nullptr;  // small pinned host staging area
  size_t pinned_bytes = 0;
  cudaEvent_t ev[64];      // per-round timing events
  bool time_rounds = false;
  std::vector<byo_round_log> rounds;
  byo::DevBuf scratch[8];  // context-wide temporaries (sort, scan)
  byo::Mlp *policy = nullptr;
  // per-kernel timing: tagged launches matching `ktag` ("*" = every tag) are
  // bracketed by event pairs; ktags[i] names the pair i
  std::string ktag;
  std::vector<cudaEvent_t> kev;
  std::vector<const char *> ktags;
  size_t kev_used = 0;
  int update_policy = BYO_UPDATE_MERGE;  // container update strategy
  int last_update_strategy = 0;          // 0 merge, 1 rebuild (last batch)
  // grid-barrier test hook (byo_ctx_set_barrier_test): limit in ms (0 = the
  // default) and arrivals awaited beyond the launched blocks
  uint32_t bar_limit_ms = 0, bar_extra = 0;
  // PageRank iterations as one CUDA graph (default) or one stream launch per
  // kernel with a host check per iteration (byo_ctx_set_pagerank_graphs)
  bool pr_graphs = true;
};

// What the last batch update did (PMA): batch keys, keys changed, leaves the
// merge rewrote and the keys they held before it; path 0 merge, 1 rebuild,
// 2 merge then window redistribution.
struct UpdateStats {
  uint64_t keys = 0, changed = 0, leaves = 0, entries = 0;
  uint32_t path = 0;
};

struct byo_graph {
  byo_ctx *ctx = nullptr;
  int container = BYO_CONTAINER_CSR;
  uint64_t n = 0, m = 0;
  uint64_t *d_off = nullptr;
  uint32_t *d_slots = nullptr;
  uint64_t nslots = 0;
  uint32_t *d_deg = nullptr;
  byo::Pma *pma = nullptr;
  byo::Vos *vos = nullptr;  // vector of per-vertex runs (BYO_CONTAINER_VOS)
  byo::Pcsr *pcsr = nullptr;  // packed CSR (BYO_CONTAINER_PCSR); d_off is its vertex index
  byo::DevBuf ws[24];  // per-graph workspaces, indexed by the Ws enum
  byo_tuning tune = {};  // launch shapes set by the caller or the autotuner (0 = automatic)
  // A PMA keeps a compact CSR snapshot of its contents for the read-only
  // algorithms, rebuilt on first use after an update (version counts updates).
  uint64_t version = 0;
  byo_graph *snap = nullptr;
  uint64_t snap_version = 0;
  uint64_t slots_cap = 0;  // snapshot: capacity of d_slots
  UpdateStats upd;         // the last batch update (PMA)
};

namespace byo {

enum Ws {
  WS_LP = 0,        // uint64[n]   BFS level<<32 | parent
  WS_VISITED,       // uint32[W]
  WS_FRONT_LIST_A,  // uint32[n]
  WS_FRONT_LIST_B,
  WS_FRONT_BITS_A,  // uint32[W]
  WS_FRONT_BITS_B,
  WS_DEFER,         // uint32[n]   pull long-list / hub list
  WS_SCAN,          // uint64[n+1] frontier degree prefix (blocked push)
  WS_STATS,         // small device stats block
  WS_LABEL,         // uint32[n]   CC
  WS_PR_A,          // PageRank state
  WS_PR_B,
  WS_PR_C,
  WS_PR_D,
  WS_TC_RANK,
  WS_TC_OFF,
  WS_TC_NBR,
  WS_TC_CNT,
  WS_BUCKETS,
  WS_MISC,
  WS_STREAM,        // update stream: batch offsets and operations
  WS_MS_LEVELS,     // uint64[16][n] 64-source BFS: bit b of each pair's level
  WS_STREAM_Q,      // mixed stream: query numbering, sources, descriptors, op times
  WS_COUNT
};
static_assert(WS_COUNT <= 24, "byo_graph::ws holds 24 workspaces");

// ---------------------------------------------------------------- errors
int set_error(byo_ctx *ctx, int code, const char *what, cudaError_t e = cudaSuccess);
#define BYO_CU(ctx, call)                                             \
  do {                                                                \
    cudaError_t e_ = (call);                                          \
    if (e_ != cudaSuccess) return byo::set_error(ctx, BYO_EDEVICE, #call, e_); \
  } while (0)
#define BYO_TRY(call)            \
  do {                           \
    int rc_ = (call);            \
    if (rc_ != BYO_OK) return rc_; \
  } while (0)
int check_launch(byo_ctx *ctx, const char *what);

// Launch on the context's stream and count it.
template <typename Kern, typename... Args>
inline void launch(byo_ctx *ctx, Kern kernel, dim3 grid, dim3 block, size_t smem, Args... args) {
  kernel<<<grid, block, smem, ctx->stream>>>(args...);
  ctx->launches++;
}

// As launch(), and when `tag` is the context's timed tag, brackets the launch
// with a pair of CUDA events on the same stream.
bool ktimer_begin(byo_ctx *ctx, const char *tag);
void ktimer_end(byo_ctx *ctx);
template <typename Kern, typename... Args>
inline void launch_t(byo_ctx *ctx, const char *tag, Kern kernel, dim3 grid, dim3 block, size_t smem,
                     Args... args) {
  bool timed = !ctx->ktag.empty() && ktimer_begin(ctx, tag);
  kernel<<<grid, block, smem, ctx->stream>>>(args...);
  ctx->launches++;
  if (timed) ktimer_end(ctx);
}

// ---------------------------------------------------------------- memory
int ensure(byo_ctx *ctx, DevBuf &b, size_t bytes);
template <typename T>
int ws(byo_graph *g, int slot, size_t count, T **out) {
  BYO_TRY(ensure(g->ctx, g->ws[slot], count * sizeof(T)));
  *out = static_cast<T *>(g->ws[slot].p);
  return BYO_OK;
}
template <typename T>
int scratch(byo_ctx *ctx, int slot, size_t count, T **out) {
  BYO_TRY(ensure(ctx, ctx->scratch[slot], count * sizeof(T)));
  *out = static_cast<T *>(ctx->scratch[slot].p);
  return BYO_OK;
}
void free_buf(DevBuf &b);
int pinned(byo_ctx *ctx, size_t bytes, void **out);
int grid_for(byo_ctx *ctx, uint64_t work, int block, int per_sm = 8);

// ---------------------------------------------------------------- primitives (primitives.cu)
// Exclusive scan of uint32 or uint64 items into uint64 out[count+1]
// (out[count] = total).  Uses scratch slots 6,7.
int scan_u32_to_u64(byo_ctx *ctx, const uint32_t *in, uint64_t count, uint64_t *out);
int scan_u64(byo_ctx *ctx, const uint64_t *in, uint64_t count, uint64_t *out);
// Exclusive scan of deg[list[i]] (frontier degree prefix) into out[count+1].
int scan_gather_deg(byo_ctx *ctx, const uint32_t *deg, const uint32_t *list, uint64_t count,
                    uint64_t *out);
// Exclusive scan of off[list[i]+1] - off[list[i]] (slot-range lengths).
int scan_gather_range(byo_ctx *ctx, const uint64_t *off, const uint32_t *list, uint64_t count,
                      uint64_t *out);
// LSD radix sort of uint64 keys restricted to the bytes set in sig_mask;
// returns the buffer that holds the result (keys or tmp).  Scratch slots 4,5.
int sort_u64(byo_ctx *ctx, uint64_t *keys, uint64_t *tmp, uint64_t count, uint64_t sig_mask,
             uint64_t **sorted);
// Sorts an update batch (keys src<<32|dst, src,dst < n) from `in` into `out`
// by a bucket partition on src and per-bucket shared-memory sorts; `tmp`
// (count keys) is used only by buckets too large for shared memory.  A key
// with src or dst >= n is placed without an out-of-bounds access (in an
// unspecified order), so the sort may run before the batch is validated.
int sort_bucketed(byo_ctx *ctx, const uint64_t *in, uint64_t count, uint64_t n, uint64_t *out, uint64_t *tmp);
// Removes adjacent duplicates of a sorted array (and src==dst keys if
// drop_loops) into out; *out_count on the host.  Scratch slots 3.
int unique_u64(byo_ctx *ctx, const uint64_t *in, uint64_t count, int drop_loops, uint64_t *out,
               uint64_t *out_count);
// offsets[v] = first index of keys with src >= v (keys sorted), v in [0,n].
int offsets_from_keys(byo_ctx *ctx, const uint64_t *keys, uint64_t count, uint64_t n,
                      uint64_t *offsets);
int dst_from_keys(byo_ctx *ctx, const uint64_t *keys, uint64_t count, uint32_t *dst);
int degrees_from_offsets(byo_ctx *ctx, const uint64_t *off, uint64_t n, uint32_t *deg);
int reduce_max_u64(byo_ctx *ctx, const uint64_t *in, uint64_t count, uint64_t *out_host);
uint64_t sig_mask_for(uint64_t n);
int memset_async(byo_ctx *ctx, void *p, int v, size_t bytes);

// ---------------------------------------------------------------- graph construction (graph.cu)
int graph_from_sorted_keys(byo_ctx *ctx, int container, uint64_t n, const uint64_t *d_keys,
                           uint64_t m, byo_graph **out);
int graph_from_host_csr(byo_ctx *ctx, int container, uint64_t n, uint64_t m, const uint64_t *h_off,
                        const uint32_t *h_nbrs, byo_graph **out);
int graph_generate(byo_ctx *ctx, int container, const byo_gen_spec *sp, byo_graph **out);
int graph_alloc_view(byo_graph *g);
int gen_rmat_pairs(byo_ctx *ctx, uint64_t seed, uint32_t lg_n, double a, double b, double c,
                   uint64_t first, uint64_t count, uint32_t *src, uint32_t *dst);
int gen_uniform_pairs(byo_ctx *ctx, uint64_t seed, uint64_t n, uint64_t first, uint64_t count,
                      uint32_t *src, uint32_t *dst);
int gen_uniform_keys(byo_ctx *ctx, uint64_t seed, uint64_t n, uint64_t count, uint64_t *keys);

// ---------------------------------------------------------------- traversal (engine.cu)
int bfs_run(byo_graph *g, uint32_t src, uint32_t *d_parent, uint32_t *d_level, int policy,
            uint32_t *rounds);

// ---------------------------------------------------------------- 64-source BFS (msbfs.cu)
int bfs_multi_run(byo_graph *g, const uint32_t *h_srcs, uint32_t k, uint32_t *d_levels, uint32_t *rounds);
int pagerank_delta_run(byo_graph *g, double eps, double local_eps, uint32_t max_iters, double *d_p,
                       uint32_t *rounds, double *l1);
// The graph the read-only algorithms traverse: g itself for a CSR, the
// compact snapshot of a PMA's contents (rebuilt if stale) otherwise.
int traversal_view(byo_graph *g, byo_graph **out);
// Copies the PMA's keys, leaf by leaf, into a compact neighbour array
// (sorted adjacency in CSR order).
int pma_compact(byo_graph *g, uint32_t *d_slots_out);
// Graph files (graphio.cu).  With offsets == NULL only *n and *m are read.
int adj_read_host(byo_ctx *ctx, const char *path, int binary, uint64_t *n, uint64_t *m, uint64_t *offsets,
                  uint32_t *nbrs);
int adj_write_host(byo_ctx *ctx, const char *path, int binary, uint64_t n, uint64_t m, const uint64_t *offsets,
                   const uint32_t *nbrs);
// Launch shapes in effect: g->tune where set, else the defaults for g.
byo_tuning effective_tuning(const byo_graph *g);
int check_tuning(byo_ctx *ctx, const byo_tuning *t);
int autotune(byo_graph *g, uint32_t what, uint32_t trials);

// ---------------------------------------------------------------- algorithms (algos.cu)
int cc_run(byo_graph *g, uint32_t *d_label);
int bfs_cc_run(byo_graph *g, uint32_t *d_label);
int pagerank_run(byo_graph *g, double eps, uint32_t max_iters, int precision, double *d_p,
                 uint32_t *iters, double *l1);
int tc_run(byo_graph *g, uint64_t *count);
int map_run(byo_graph *g, int width, const void *d_remote, uint64_t *sum);
int graph_from_device_csr(byo_ctx *ctx, int container, uint64_t n, uint64_t m, const uint64_t *d_off,
                          const uint32_t *d_nbrs, byo_graph **out);
int graph_from_bytepd_host(byo_ctx *ctx, uint64_t n, const uint64_t *h_bo, const uint32_t *h_deg,
                           const unsigned char *h_bytes, uint64_t nbytes, uint32_t P, int container,
                           byo_graph **out);
int bytepd_read_file(byo_ctx *ctx, const char *path, uint32_t P, int container, byo_graph **out);
int bytepd_write_file(byo_graph *g, const char *path, uint32_t P);
int bytepd_encode_host(byo_graph *g, uint32_t P, uint64_t *h_bo, uint32_t *h_deg, unsigned char *h_bytes,
                       uint64_t *nbytes);
uint64_t map_remote_bytes(uint64_t n, uint32_t width);
int gather_roof(byo_ctx *ctx, uint64_t table_bytes, double *gathers_per_s);

// ---------------------------------------------------------------- PMA (pma.cu)
int pma_build(byo_graph *g, const uint64_t *d_keys, uint64_t m);
int vos_build(byo_graph *g, const uint64_t *d_keys, uint64_t m);
int vos_update(byo_graph *g, const uint64_t *d_keys, uint64_t count, int sorted, int insert, uint64_t *changed);
int vos_compact(byo_graph *g, const uint64_t *offc, uint32_t *out);
void vos_destroy(Vos *v);
int pcsr_build(byo_graph *g, const uint64_t *d_keys, uint64_t m);
int pcsr_update(byo_graph *g, const uint64_t *d_keys, uint64_t count, int sorted, int insert, uint64_t *changed);
int pcsr_compact(byo_graph *g, uint32_t *out);
uint64_t pcsr_leaf_slots();
void pcsr_destroy(Pcsr *p);
// Query ops of a mixed stream (ops[b] == 2): k sources per query, taken in
// order from h_srcs; query q writes its levels to d_levels + q * k * n;
// h_op_ns (may be null) receives each op's device start and end times.
struct StreamQueries {
  const uint32_t *h_srcs;
  uint32_t k;
  uint32_t *d_levels;
  uint64_t *h_op_ns;
};
int pma_update_stream(byo_graph *g, const uint64_t *d_keys, const uint64_t *d_boff, const uint64_t *h_boff,
                      const unsigned char *d_ops, const unsigned char *h_ops, uint64_t nbatch, long long *h_changed,
                      const StreamQueries *qs = nullptr);
uint64_t pma_leaf_slots();
// One CTA sorts up to sort_small_max() (4096) keys in registers; bounds[0],
// bounds[1] receive the largest src and dst.  It does not index by key, so it
// may run before the batch is validated.
uint64_t sort_small_max();
int sort_small_keys(byo_ctx *ctx, const uint64_t *in, uint64_t count, uint64_t *out, unsigned long long *bounds);
int pma_update(byo_graph *g, const uint64_t *d_keys, uint64_t count, int sorted, int insert,
               uint64_t *changed);
int pma_export_keys(byo_graph *g, uint64_t *d_keys_out);
void pma_destroy(Pma *p);

// ---------------------------------------------------------------- policy (mlp.cu)
void policy_destroy(Mlp *p);
// 0 = in-place merge, 1 = rebuild, from the trained network (0 when untrained)
int update_strategy(byo_ctx *ctx, uint64_t batch, uint64_t m, uint64_t slots, int sorted, int insert);
void update_features(uint64_t batch, uint64_t m, uint64_t slots, int sorted, int insert, float *x);

}  // namespace byo

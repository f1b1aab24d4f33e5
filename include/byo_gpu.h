/*
 * byo_gpu.h -- C ABI of the GB300 (sm_103a) graph-container engine.
 *
 * This is the drop-in boundary for BYO's data-parallel hot path: the GBBS
 * edgeMap / vertexSubset traversal engine, the algorithms that BYO's run_all
 * drives through it, and the batched insert/delete of a packed-memory-array
 * graph container.  Everything is plain pointers and sizes; no C++ or torch
 * type crosses it.  Reference interfaces are cited as path:line of the
 * wheatman/BYO tree.
 *
 * Conventions
 *  - vertex ids uint32 (gbbs uintE), edge offsets uint64 (uintT),
 *    BYO_NONE (0xFFFFFFFF) = "unreached / no parent" (UINT_E_MAX).
 *  - update keys are uint64 (src << 32) | dst, the bit pattern of the
 *    std::tuple<uintE,uintE> that PMA_graph bit_casts
 *    (benchmarks/run_structures/run_single_pma.cc:63-70).
 *  - functions return BYO_OK (0) or a negative BYO_E* code; the message of the
 *    last failure is byo_last_error(ctx).  No function aborts the process.
 *  - Arguments named h_* are host memory; d_* are device memory of the
 *    context's device.  Host-memory variants copy through the context's
 *    stream and return when the result is on the host.
 *  - A context owns one CUDA stream; calls on one context are not thread safe
 *    (the reference is likewise driven from one host thread, its parallelism
 *    is internal).
 */
#ifndef BYO_GPU_H
#define BYO_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BYO_NONE 0xFFFFFFFFu

enum byo_status {
  BYO_OK = 0,
  BYO_EINVAL = -1,    /* bad argument (null pointer, id >= n, bad size) */
  BYO_ENOMEM = -2,    /* device allocation failed */
  BYO_EDEVICE = -3,   /* CUDA error; see byo_last_error */
  BYO_ETIMEDOUT = -4, /* a bounded device-side wait gave up */
  BYO_ENOTSUP = -5    /* operation not supported by this container */
};

typedef struct byo_ctx byo_ctx;
typedef struct byo_graph byo_graph;
typedef struct byo_vertex_subset byo_vertex_subset;

/* ------------------------------------------------------------------ context */

/* Opens a context on CUDA device `device`; creates its stream. */
int byo_gpu_init(int device, byo_ctx **out);
void byo_gpu_shutdown(byo_ctx *ctx);
const char *byo_last_error(const byo_ctx *ctx);
/* The context's cudaStream_t, for callers that time or order work around it. */
void *byo_ctx_stream(byo_ctx *ctx);
/* Number of kernels this context has launched so far. */
uint64_t byo_ctx_launches(const byo_ctx *ctx);
int byo_ctx_synchronize(byo_ctx *ctx);
/* Library version string. */
const char *byo_version(void);

/* Device buffers for callers without CUDA bindings (a C++ adapter, a cgo or
 * JNI host): the arrays the edgeMap functors and the mixed stream read and
 * write.  byo_buffer_alloc allocates `bytes` on the context's device;
 * byo_buffer_write / byo_buffer_read copy `bytes` between host memory and the
 * buffer at byte `offset` and return when the copy is done; byo_buffer_fill32
 * sets `count` 32-bit words from byte `offset` to `value`.  No reference
 * counterpart (the reference's arrays are host memory). */
int byo_buffer_alloc(byo_ctx *ctx, uint64_t bytes, void **d_out);
void byo_buffer_free(byo_ctx *ctx, void *d);
int byo_buffer_write(byo_ctx *ctx, void *d, uint64_t offset, const void *h, uint64_t bytes);
int byo_buffer_read(byo_ctx *ctx, const void *d, uint64_t offset, void *h, uint64_t bytes);
int byo_buffer_fill32(byo_ctx *ctx, void *d, uint64_t offset, uint64_t count, uint32_t value);

/* ------------------------------------------------------------------ containers
 * Replaces the container adapters of benchmarks/run_structures: CSR
 * (run_csr.cc:28-175, static) and PMA_graph (run_single_pma.cc:39-141, a
 * packed memory array of (src,dst) keys).  Both constructors take the loader's
 * CSR (graph_io.h:117-123 builds it; run_csr.cc:87-106 and
 * run_single_pma.cc:75-89 consume it): offsets[n+1] and nbrs[m], sorted and
 * duplicate-free per vertex.  The arrays are copied; the caller keeps them. */
/* CSR (static), PMA (one packed-memory array of src << 32 | dst keys, the
 * CPMA / PMA_graph counterpart), VOS (a vector of per-vertex sorted runs
 * with slack, the counterpart of the vector-of-sets containers,
 * run_vector_pma.cc / run_vector_vector.cc) and PCSR (the Packed CSR of
 * run_pcsr.cc:24-99: one packed array of per-vertex sentinels and neighbour
 * ids, 4 bytes a slot, with the vertex index kept up to date by the updates;
 * n below 2^31).  PMA, VOS and PCSR take updates. */
enum byo_container {
  BYO_CONTAINER_CSR = 0,
  BYO_CONTAINER_PMA = 1,
  BYO_CONTAINER_VOS = 2,
  BYO_CONTAINER_PCSR = 3
};

int byo_graph_create_csr(byo_ctx *ctx, uint64_t n, uint64_t m, const uint64_t *h_offsets,
                         const uint32_t *h_nbrs, byo_graph **out);
int byo_graph_create_pma(byo_ctx *ctx, uint64_t n, uint64_t m, const uint64_t *h_offsets,
                         const uint32_t *h_nbrs, byo_graph **out);
/* Either container from a CSR (sorted, duplicate-free lists, copied in). */
int byo_graph_create(byo_ctx *ctx, int container, uint64_t n, uint64_t m, const uint64_t *h_offsets,
                     const uint32_t *h_nbrs, byo_graph **out);
void byo_graph_destroy(byo_graph *g);
int byo_graph_container(const byo_graph *g);
/* G.N() / num_vertices() (graph.h:2627; run_csr.cc:31) */
uint64_t byo_graph_num_vertices(const byo_graph *g);
/* G.M() / num_edges(): directed entries currently stored (run_csr.cc:32) */
uint64_t byo_graph_num_edges(const byo_graph *g);
/* Slots of the traversal view (= num_edges for a CSR; the PMA counts gaps). */
uint64_t byo_graph_num_slots(const byo_graph *g);
/* degree(i) for every vertex (run_csr.cc:34-36; Graph::finilize
 * graph.h:2559-2588 for containers without a native degree). */
int byo_graph_degrees(byo_graph *g, uint32_t *h_out);
/* Sorted adjacency of every vertex, the content Graph::write_adj dumps
 * (graph.h:3018-3044); the parity view of a container after updates. */
int byo_graph_export_csr(byo_graph *g, uint64_t *h_offsets, uint32_t *h_nbrs);
/* Neighbours of one vertex, sorted (map_neighbors, run_csr.cc:38-43). Writes
 * at most cap ids and the degree to *deg. */
int byo_graph_neighbors(byo_graph *g, uint32_t v, uint32_t *h_out, uint64_t cap, uint64_t *deg);

/* Batched updates: Graph::insert_batch / remove_batch (graph.h:3071-3124) ->
 * PMA_graph::insert_sorted_batch / remove_sorted_batch (run_single_pma.cc:63-70).
 * keys may be unsorted and contain duplicates unless `sorted` is 1 (then they
 * must be strictly increasing).  Inserting a present key and removing an
 * absent key are no-ops.  A batch with a key whose src or dst is >= n, or one
 * passed as sorted that is not strictly increasing, is rejected whole
 * (BYO_EINVAL) and leaves the container unchanged.  BYO_ENOMEM or
 * BYO_EDEVICE from an update (a grow or rebuild that could not allocate, after
 * the merge had started) leaves the contents unspecified: destroy the graph.
 * (The reference aborts on a failed allocation.)
 * *changed (may be NULL) receives the number of keys actually inserted or
 * removed.  The PMA, VOS and PCSR containers take updates (CSR: BYO_ENOTSUP). */
int byo_graph_insert_batch(byo_graph *g, const uint64_t *h_keys, uint64_t count, int sorted,
                           uint64_t *changed);
int byo_graph_remove_batch(byo_graph *g, const uint64_t *h_keys, uint64_t count, int sorted,
                           uint64_t *changed);
int byo_graph_insert_batch_device(byo_graph *g, const uint64_t *d_keys, uint64_t count, int sorted,
                                  uint64_t *changed);
int byo_graph_remove_batch_device(byo_graph *g, const uint64_t *d_keys, uint64_t count, int sorted,
                                  uint64_t *changed);

/* What the last insert/remove batch on g did, for the update path's byte
 * accounting (the reference's Batch_insert_runner times the batch,
 * benchmarks/run_unweighted.h:832-873; it reports no byte counts).  keys: the
 * batch's keys (duplicates included); changed: keys inserted or removed;
 * touched_leaves: PMA leaves the merge rewrote; touched_entries: keys those
 * leaves held before the merge; leaf_slots: slots per PMA leaf (0 for other
 * containers); path: 0 in-place merge, 1 rebuild, 2 merge then window
 * redistribution of overflowing leaves (whose extra traffic is not counted). */
typedef struct byo_update_stats {
  uint64_t keys;
  uint64_t changed;
  uint64_t touched_leaves;
  uint64_t touched_entries;
  uint64_t leaf_slots;
  uint32_t path;
  uint32_t reserved;
} byo_update_stats;
int byo_graph_last_update_stats(const byo_graph *g, byo_update_stats *out);

/* ------------------------------------------------------------------ graph files
 * The reference's input formats (gbbs/graph_io.cc:35-95, read by
 * read_unweighted_symmetric_graph, gbbs/graph_io.h:98-124):
 *   text    "AdjacencyGraph", n, m, n offsets, m neighbour ids (whitespace
 *           separated); binary = 0
 *   binary  int64 n, int64 m, int64 file size, uint64 offsets[n+1],
 *           uint32 ids[m] (the layout of the reference's -DLONG build);
 *           binary = 1
 * byo_adj_read parses on the host without a device: call it with offsets =
 * nbrs = NULL for *n and *m, then with arrays of n+1 and m entries.  Offsets
 * must run from 0 to m without decreasing and ids must be below n (BYO_EINVAL
 * otherwise).  byo_graph_read_adj loads a file into a new container (which
 * also requires each adjacency sorted, as the loaders do);
 * byo_graph_write_adj writes the sorted adjacency in either format (text =
 * Graph::write_adj, gbbs/graph.h:3018-3044). */
int byo_adj_read(const char *path, int binary, uint64_t *n, uint64_t *m, uint64_t *offsets, uint32_t *nbrs);
int byo_graph_read_adj(byo_ctx *ctx, const char *path, int binary, int container, byo_graph **out);
int byo_graph_write_adj(byo_graph *g, const char *path, int binary);

/* ------------------------------------------------------------------ generators
 * Synthetic graphs built on the device (counter-based streams; a slice of any
 * stream is reproducible on the host bit for bit).  Pairs are symmetrised,
 * sorted, deduplicated and self loops dropped, as the workloads specify. */
enum byo_gen_kind { BYO_GEN_RMAT = 0, BYO_GEN_ER = 1, BYO_GEN_GRID = 2, BYO_GEN_CHUNG_LU = 3 };
typedef struct byo_gen_spec {
  int kind;          /* byo_gen_kind */
  uint64_t seed;
  uint32_t lg_n;     /* RMAT: n = 2^lg_n */
  uint64_t n;        /* ER / Chung-Lu: vertices; GRID: rows */
  uint64_t draws;    /* RMAT / ER / Chung-Lu: pairs drawn; GRID: columns */
  double a, b, c;    /* RMAT quadrant probabilities */
  double exponent;   /* Chung-Lu power-law exponent */
} byo_gen_spec;
int byo_graph_generate(byo_ctx *ctx, int container, const byo_gen_spec *spec, byo_graph **out);
/* Raw pair streams into device buffers (RMAT thresholds as in the oracle). */
int byo_gen_rmat_pairs_device(byo_ctx *ctx, uint64_t seed, uint32_t lg_n, double a, double b,
                              double c, uint64_t first, uint64_t count, uint32_t *d_src,
                              uint32_t *d_dst);
int byo_gen_uniform_pairs_device(byo_ctx *ctx, uint64_t seed, uint64_t n, uint64_t first,
                                 uint64_t count, uint32_t *d_src, uint32_t *d_dst);
/* Symmetrised update keys for a uniform batch: 2*count keys (u<<32|v, v<<32|u). */
int byo_gen_uniform_keys_device(byo_ctx *ctx, uint64_t seed, uint64_t n, uint64_t count,
                                uint64_t *d_keys);

/* ------------------------------------------------------------------ traversal
 * Direction policy for edgeMap rounds (the choice never changes a result). */
enum byo_policy {
  BYO_POLICY_M20 = 0,          /* GBBS rule, edge_map_data.h:254-307 (sparse = push) */
  BYO_POLICY_LEARNED = 1,      /* MLP over frontier statistics, falls back to M20 */
  BYO_POLICY_PUSH = 2,         /* force sparse push every round */
  BYO_POLICY_PULL = 3,         /* force dense pull every round */
  BYO_POLICY_BLOCKED = 4,      /* force edge-balanced blocked push every round */
  BYO_POLICY_M20_BLOCKED = 5   /* GBBS rule with blocked push for sparse rounds */
};

/* BFS (benchmarks/BFS/NonDeterministicBFS/BFS.h:47-64).  parent[v]: the
 * smallest-id neighbour of v one level closer to src (a valid outcome of the
 * reference's nondeterministic CAS, and exactly what its dense pull produces on
 * sorted adjacency); parent[src] = src; BYO_NONE if unreached.  level may be
 * NULL.  *rounds (may be NULL) = edgeMap rounds run. */
int byo_bfs(byo_graph *g, uint32_t src, uint32_t *h_parent, uint32_t *h_level, int policy,
            uint32_t *rounds);
int byo_bfs_device(byo_graph *g, uint32_t src, uint32_t *d_parent, uint32_t *d_level, int policy,
                   uint32_t *rounds);

/* Batched BFS from k <= 64 sources at once, bit lanes of one traversal run
 * by a persistent kernel.  levels[s * n + v] is the BFS level of v from
 * srcs[s] (BYO_NONE if unreached), identical to byo_bfs's levels; sources may
 * repeat.  *rounds (may be NULL) = rounds run.  No reference counterpart:
 * the reference answers one source per BFS call
 * (benchmarks/BFS/NonDeterministicBFS/BFS.h:47-64). */
int byo_bfs_multi(byo_graph *g, const uint32_t *h_srcs, uint32_t k, uint32_t *h_levels,
                  uint32_t *rounds);
int byo_bfs_multi_device(byo_graph *g, const uint32_t *h_srcs, uint32_t k, uint32_t *d_levels,
                         uint32_t *rounds);

/* Launch shapes of the traversal kernels, kept per graph: the degree
 * boundaries at which work per vertex moves from a thread to a group of lanes,
 * a warp or a CTA, and tile sizes.  Results never depend on them.  In
 * byo_graph_set_tuning a zero field means "automatic"; byo_graph_get_tuning
 * reports the values in effect.  No reference counterpart (the reference's
 * shapes are compile-time constants: kEMBlockSize gbbs/macros.h:80,
 * vertex_ops::kBlockSize gbbs/vertex.h:35). */
typedef struct byo_tuning {
  uint32_t push_group;   /* single-source push: lanes per frontier vertex (4, 8, 16 or 32) */
  uint32_t hub_min;      /* single-source push: degree from which one CTA takes a vertex (>= 32) */
  uint32_t pull_cap;     /* single-source pull: slots a thread scans before a warp takes over (1..4096) */
  uint32_t blocked_tile; /* blocked push: slots per tile (64..65536) */
  uint32_t ms_heavy_deg; /* 64-source pull: slots above which a warp takes a vertex (1..65536) */
  uint32_t ms_hub_deg;   /* 64-source push: frontier vertices above this many slots are cut into
                            chunks of this size, a warp each (32..2^20) */
  uint32_t ms_push_div;  /* 64-source: push while the frontier's slots < all slots / ms_push_div */
  uint32_t pull_stage_words; /* single-source pull: frontier bitmap words staged in shared memory
                                (256..49152; fewer words let two CTAs share an SM) */
  uint32_t tc_stage;     /* triangle counting: DAG out-lists up to this many entries are staged in
                            a CTA's shared memory, longer ones are searched in place (512..49152) */
  uint32_t reserved;     /* zero */
} byo_tuning;
int byo_graph_get_tuning(byo_graph *g, byo_tuning *out);
int byo_graph_set_tuning(byo_graph *g, const byo_tuning *t);
/* Picks the tuning fields by timing the kernels on this graph: coordinate
 * descent over candidate values of each field, BFS from `trials` seeded
 * sources per candidate.  what: BYO_TUNE_BFS and/or BYO_TUNE_MULTI.  The
 * result is installed on the graph and copied to *out (may be NULL). */
#define BYO_TUNE_BFS 1u
#define BYO_TUNE_MULTI 2u
int byo_graph_autotune(byo_graph *g, uint32_t what, uint32_t trials, byo_tuning *out);

/* Connectivity, SimpleUnionAsync semantics
 * (benchmarks/Connectivity/SimpleUnionAsync/Connectivity.h:122-136): label[v]
 * = smallest vertex id in v's component. */
int byo_cc(byo_graph *g, uint32_t *h_label);
int byo_cc_device(byo_graph *g, uint32_t *d_label);
/* BFS-based connectivity (benchmarks/Connectivity/BFSCC/Connectivity.h:33-88);
 * same labels as byo_cc. */
int byo_bfs_cc(byo_graph *g, uint32_t *h_label);

/* PageRank (benchmarks/PageRank/PageRank.h:125-193): damping 0.85, p0 = 1/n,
 * stop when the L1 change < eps or after max_iters; no dangling
 * redistribution.  Output p_out in FP64. */
enum byo_precision {
  BYO_PR_FP32_KAHAN = 0, /* FP32 state, compensated per-vertex sums, FP64 residual */
  BYO_PR_FP64 = 1,       /* FP64 throughout */
  BYO_PR_FP32 = 2        /* FP32, uncompensated (for the error comparison) */
};
int byo_pagerank(byo_graph *g, double eps, uint32_t max_iters, int precision, double *h_p,
                 uint32_t *iters, double *l1);
int byo_pagerank_device(byo_graph *g, double eps, uint32_t max_iters, int precision, double *d_p,
                        uint32_t *iters, double *l1);

/* PageRank_edgeMap (benchmarks/PageRank/PageRank.h:80-123), its loop through
 * the edgeMap API: frontier = every vertex; per iteration edgeMap(PR_F,
 * threshold 0, no_output) (always the dense round), vertexMap(PR_Vertex_F),
 * the L1 change, reset and swap; FP64.  Returns the last computed iterate. */
int byo_pagerank_edgemap(byo_graph *g, double eps, uint32_t max_iters, double *h_p, uint32_t *iters,
                         double *l1);

/* delta::PageRankDelta (benchmarks/PageRank/PageRank.h:340-398), FP64: p0 = 0,
 * delta0 = 1/n, frontier0 = all vertices; per round every vertex sums
 * delta/deg of its neighbours in the frontier, the first round adds
 * 0.85*sum + 0.15/n to p (active when the change beyond 1/n exceeds
 * local_eps*p), later rounds add 0.85*sum when its magnitude exceeds
 * local_eps*p (then active); stops when the sum of |delta| < eps or after
 * max_iters rounds.  *rounds, *l1 may be NULL.  Reference defaults: eps 1e-4
 * in run_all (run_unweighted.h:920), local_eps 0.01, 20 rounds. */
int byo_pagerank_delta(byo_graph *g, double eps, double local_eps, uint32_t max_iters, double *h_p,
                       uint32_t *rounds, double *l1);
int byo_pagerank_delta_device(byo_graph *g, double eps, double local_eps, uint32_t max_iters, double *d_p,
                              uint32_t *rounds, double *l1);

/* Triangle counting, degree ordering
 * (benchmarks/TriangleCounting/ShunTangwongsan15/Triangle.h:167-204). */
int byo_triangle_count(byo_graph *g, uint64_t *count);

/* A stream of update batches (Batch_insert_runner's loop,
 * benchmarks/run_unweighted.h:781-893, as one call): batch b is keys
 * [offsets[b], offsets[b+1]) (src << 32 | dst, unsorted, duplicates allowed),
 * inserted when ops[b] != 0 and removed otherwise, in order.  Runs of small
 * batches (at most 4096 keys and at most half as many as the container has
 * leaves) are drained by one persistent kernel -- sort, segment search,
 * merge and offset refresh per batch between grid barriers, one host
 * synchronisation for the run; a batch that overflows a leaf stops the
 * kernel, is finished on the windowed path and the run resumes after it;
 * larger batches take byo_graph_insert/remove_batch.  changed[b] (may be NULL)
 * receives each batch's count of keys inserted or removed.  A key with src or
 * dst >= n gives BYO_EINVAL with the batches before it applied.  offsets and
 * ops are host arrays; keys are host (byo_graph_update_stream) or device
 * (_device) memory. */
int byo_graph_update_stream(byo_graph *g, const uint64_t *h_keys, const uint64_t *offsets, const uint8_t *ops,
                            uint64_t nbatch, uint64_t *changed);
int byo_graph_update_stream_device(byo_graph *g, const uint64_t *d_keys, const uint64_t *offsets, const uint8_t *ops,
                                   uint64_t nbatch, uint64_t *changed);

/* A mixed stream of update batches and 64-source BFS queries, in order
 * (the serving pattern of a dynamic graph: batches arrive between queries);
 * PMA, packed CSR or vector-of-runs container.  ops[i]: BYO_OP_REMOVE /
 * BYO_OP_INSERT (keys
 * [offsets[i], offsets[i+1]) as in byo_graph_update_stream) or BYO_OP_QUERY
 * (an empty key range): the q-th query op runs a k-source bit-lane BFS
 * (k <= 64, sources h_srcs[q*k .. q*k+k)) over the contents at that point of
 * the stream and writes levels as byo_bfs_multi does to
 * d_levels + q*k*n (device memory of nq*k*n entries).  On the PMA, runs of
 * queries and small batches (as for byo_graph_update_stream) are drained by
 * one persistent kernel under one bounded grid barrier: per query its state is
 * cleared, the traversal runs over the container's own slots and the levels
 * are written, with no host round trip; a larger batch, or one whose merge
 * overflows a leaf, is finished by the host and the kernel resumes after it.
 * The other containers run the ops one by one (each batch through its own
 * update, each query as byo_bfs_multi on the contents at that point).
 * changed[i] (may be NULL): keys inserted or removed by op i.  op_ns (may be
 * NULL, 2*nops entries): device start and end time of each op run inside the
 * PMA's kernel, in ns of one clock (0 for ops run otherwise).  No
 * reference counterpart: the reference runs queries and batches as separate
 * calls (benchmarks/run_unweighted.h:781-893 for batches, BFS.h:47-64 for a
 * query). */
enum byo_stream_op { BYO_OP_REMOVE = 0, BYO_OP_INSERT = 1, BYO_OP_QUERY = 2 };
int byo_graph_mixed_stream(byo_graph *g, const uint64_t *h_keys, const uint64_t *offsets, const uint8_t *ops,
                           uint64_t nops, const uint32_t *h_srcs, uint32_t k, uint32_t *d_levels, uint64_t *changed,
                           uint64_t *op_ns);
int byo_graph_mixed_stream_device(byo_graph *g, const uint64_t *d_keys, const uint64_t *offsets, const uint8_t *ops,
                                  uint64_t nops, const uint32_t *h_srcs, uint32_t k, uint32_t *d_levels,
                                  uint64_t *changed, uint64_t *op_ns);

/* ------------------------------------------------------------------ byte-PD graphs
 * The reference's compressed graphs: neighbour lists in the bytepd_amortized
 * encoding (gbbs/encodings/byte_pd_amortized.h:1100-1155,
 * byte_pd_amortized.cc:7-55) and its file (gbbs/graph_io.h:351-390: int64 n,
 * m, total bytes; uint64 byte offsets[n+1]; uint32 degrees[n]; the bytes).
 * `block` is the encoder's block size, the reader's PARALLEL_DEGREE
 * (gbbs/macros.h:83); 0 = 1000.  Decoding and encoding run on the GPU; the
 * graph is held decoded (CSR or PMA container).  Malformed data, or lists
 * that are not strictly increasing, give BYO_EINVAL. */
int byo_graph_from_bytepd(byo_ctx *ctx, uint64_t n, const uint64_t *byte_offsets, const uint32_t *degrees,
                          const uint8_t *bytes, uint64_t nbytes, uint32_t block, int container, byo_graph **out);
int byo_graph_read_bytepd(byo_ctx *ctx, const char *path, uint32_t block, int container, byo_graph **out);
int byo_graph_write_bytepd(byo_graph *g, const char *path, uint32_t block);
/* Encodes g into host arrays: byte_offsets[n+1], degrees[n], bytes[*nbytes].
 * *nbytes is the capacity of `bytes` on entry and the size on return; with
 * bytes NULL only the size (and the offsets and degrees, when given) are
 * returned. */
int byo_graph_encode_bytepd(byo_graph *g, uint32_t block, uint64_t *byte_offsets, uint32_t *degrees, uint8_t *bytes,
                            uint64_t *nbytes);

/* ------------------------------------------------------------------ neighbour maps
 * Test_Map (benchmarks/Map/Base/Map.h:8-18): the sum over every edge (u, v)
 * of v, by one scan of the container's own slots (a PMA's leaves as they lie,
 * gaps skipped). */
int byo_map_sum(byo_graph *g, uint64_t *sum);
/* Test_Map_Remote (benchmarks/Map/RemoteRead/Map.h:21-33, as run by
 * Map_Remote_runner<G, W>, benchmarks/run_unweighted.h:50-126): the sum over
 * every edge (u, v) of remote[v], remote an n-entry array of `width`-byte
 * elements.  width 0: a bitmap, bit v of 64-bit word v/64 (std::vector<bool>
 * packs least significant bit first); 1, 2, 4, 8: unsigned integers; 16, 32:
 * an unsigned 64-bit value at the start of each element (wide_int<size_t, W>).
 * byo_map_remote copies h_remote (host) in; the _device form reads d_remote. */
int byo_map_remote(byo_graph *g, const void *h_remote, uint32_t width, uint64_t *sum);
int byo_map_remote_device(byo_graph *g, const void *d_remote, uint32_t width, uint64_t *sum);

/* ------------------------------------------------------------------ edgeMap API
 * vertexSubset (gbbs/vertex_subset.h:202-371), edgeMap
 * (gbbs/edge_map_data.h:254-315), vertexMap and vertexFilter
 * (gbbs/vertex_subset.h:382-485) over device functors.  A device kernel cannot
 * call a host lambda, so the functor set is closed; each kind mirrors one GBBS
 * functor struct {update, updateAtomic, cond} over arrays the caller owns
 * (d_*: device memory of the graph's context, n entries unless stated). */
enum byo_functor_kind {
  BYO_F_BFS = 0,       /* BFS_F, BFS.h:30-45, over a parents array owned by the functor */
  BYO_F_BFS_LABEL = 1, /* BFS_ComponentLabel_F, benchmarks/Connectivity/BFSCC/Connectivity.h:31-50:
                          cond(d) = Parents[d] == BYO_NONE; update writes src into Parents[d]
                          (returns 1 if it changed); updateAtomic = CAS(BYO_NONE -> src) */
  BYO_F_PR = 2,        /* PR_F, benchmarks/PageRank/PageRank.h:33-50: p_next[d] += p_curr[s] /
                          degree(s); cond true; updateAtomic adds atomically */
  BYO_F_PR_DELTA = 3   /* delta::PR_Delta_F, PageRank.h:200-226: nghSum[d] += delta_over_degree[s],
                          returns whether nghSum[d] was 0 before; d_delta holds n pairs
                          {delta, delta / degree} (struct delta_and_degree) */
};
/* edgeMap flags, values as gbbs/flags.h:8-19 */
enum byo_edge_map_flags {
  BYO_FL_NO_OUTPUT = 1,
  BYO_FL_SPARSE_BLOCKED = 4,
  BYO_FL_DENSE_FORWARD = 8,
  BYO_FL_DENSE_PARALLEL = 16,
  BYO_FL_NO_DENSE = 64,
  BYO_FL_DENSE_ONLY = 1024
};
typedef struct byo_functor byo_functor;
/* BFS_F over a fresh Parents array (all BYO_NONE but Parents[src] = src). */
int byo_functor_bfs_create(byo_graph *g, uint32_t src, byo_functor **out);
int byo_functor_bfs_parents(byo_functor *f, uint32_t *h_parents);
/* The functors over caller arrays (kept by pointer; they must outlive it). */
int byo_functor_bfs_label_create(byo_graph *g, uint32_t src, uint32_t *d_parents, byo_functor **out);
int byo_functor_pr_create(byo_graph *g, const double *d_p_curr, double *d_p_next, byo_functor **out);
int byo_functor_pr_delta_create(byo_graph *g, const double *d_delta, double *d_ngh_sum, byo_functor **out);
int byo_functor_kind(const byo_functor *f);
void byo_functor_destroy(byo_functor *f);

/* vertexSubset(n, v) and vertexSubset(n, list) (vertex_subset.h:240-262). */
int byo_vs_create_single(byo_graph *g, uint32_t v, byo_vertex_subset **out);
int byo_vs_create_list(byo_graph *g, const uint32_t *h_ids, uint64_t count,
                       byo_vertex_subset **out);
/* vertexSubset(n, m, BitArray&&) (vertex_subset.h:263-270): the members are
 * the set bits of d_bits (ceil(n/32) words, bit v of word v/32; bits of ids
 * >= n ignored), copied in.  _all: BitArray(n, true), every vertex. */
int byo_vs_create_bitmap(byo_graph *g, const uint32_t *d_bits, byo_vertex_subset **out);
int byo_vs_create_all(byo_graph *g, byo_vertex_subset **out);
void byo_vs_destroy(byo_vertex_subset *vs);
uint64_t byo_vs_size(const byo_vertex_subset *vs);
int byo_vs_is_dense(const byo_vertex_subset *vs);
/* Members in increasing id order (toSparse + sort). */
int byo_vs_to_list(byo_vertex_subset *vs, uint32_t *h_out, uint64_t cap);
/* edgeMap(G, vs, F, threshold, flags): threshold -1 => M/20.  Direction as
 * edgeMapData (edge_map_data.h:254-307); sparse and blocked rounds apply cond
 * and updateAtomic from the members, dense rounds apply update to each vertex
 * whose cond holds, neighbours in increasing id order, until cond fails.  The
 * output holds each vertex once (as with gbbs's remove_duplicates flag);
 * BYO_FL_NO_OUTPUT gives an empty subset. */
int byo_edge_map(byo_graph *g, byo_vertex_subset *vs, byo_functor *f, int64_t threshold,
                 uint32_t flags, byo_vertex_subset **out);

/* vertexMap / vertexFilter (vertex_subset.h:382-485) with one of the
 * reference's vertex functions, applied to every member i:
 *   BYO_VOP_PR_UPDATE      PR_Vertex_F (PageRank.h:53-68):
 *                          d_a[i] = damping * d_a[i] + (1 - damping) / n
 *   BYO_VOP_ZERO           PR_Vertex_Reset (PageRank.h:71-78): d_a[i] = 0
 *   BYO_VOP_PR_DELTA_FIRST delta::PR_Vertex_F_FirstRound (PageRank.h:252-281):
 *                          pre = damping * d_c[i] + (1 - damping) / n;
 *                          d_a[i] += pre; delta = pre - 1/n; d_b[2i] = delta,
 *                          d_b[2i+1] = delta / degree(i); keeps i when
 *                          delta > eps2 * d_a[i]
 *   BYO_VOP_PR_DELTA       delta::PR_Vertex_F (PageRank.h:294-318):
 *                          delta = d_c[i] * damping; d_b[2i], d_b[2i+1] as
 *                          above; when |delta| > eps2 * d_a[i], d_a[i] +=
 *                          delta and i is kept
 * (d_a: p, d_b: the delta pairs, d_c: nghSum).  vertexMap ignores the
 * results; vertexFilter returns the members kept. */
enum byo_vertex_op_kind {
  BYO_VOP_PR_UPDATE = 0,
  BYO_VOP_ZERO = 1,
  BYO_VOP_PR_DELTA_FIRST = 2,
  BYO_VOP_PR_DELTA = 3
};
typedef struct byo_vertex_op {
  int kind;
  double *d_a, *d_b, *d_c;
  double damping, eps2;
} byo_vertex_op;
int byo_vertex_map(byo_vertex_subset *vs, const byo_vertex_op *op);
int byo_vertex_filter(byo_vertex_subset *vs, const byo_vertex_op *op, byo_vertex_subset **out);

/* ------------------------------------------------------------------ statistics
 * Per-round log of the last traversal (the learned policy's training data). */
typedef struct byo_round_log {
  uint32_t round;
  uint32_t mode;          /* 0 push, 1 pull, 2 blocked */
  uint64_t frontier;      /* |F| */
  uint64_t frontier_deg;  /* sum of out-degrees of F */
  uint64_t unvisited;     /* vertices not yet reached before the round */
  float ms;               /* device time of the round (with round timing on) */
  float features[16];     /* policy features of F (learned policy or timing on) */
} byo_round_log;
int byo_last_rounds(byo_ctx *ctx, byo_round_log *out, uint64_t cap, uint64_t *count);
/* Times every round with CUDA events (adds one host wait per round). */
int byo_ctx_set_round_timing(byo_ctx *ctx, int on);
/* PageRank's iterations run as one CUDA graph whose conditional nodes test
 * the residual on the device (on = 1, the default), or as one stream launch
 * per kernel with the residual checked on the host after each iteration
 * (on = 0; the same kernels in the same order, so the same results; for
 * profilers that cannot look inside conditional graphs).  No reference
 * counterpart. */
int byo_ctx_set_pagerank_graphs(byo_ctx *ctx, int on);
/* The device's rate of random 4-byte gathers from a table of table_bytes
 * (allocated and freed by the call): uniform indices from a counter-based
 * hash, 16 independent loads per thread in flight, best of 5 timed launches.
 * The second roof of kernels bound by one-word random gathers from an
 * L2-resident array (PageRank's pull).  No reference counterpart. */
int byo_gather_roof(byo_ctx *ctx, uint64_t table_bytes, double *gathers_per_s);
/* Test hook for the bounded device waits: the grid barriers of the persistent
 * kernels (small BFS rounds, 64-source BFS, the update stream) give up after
 * limit_ms (<= 4000; 0 = the default 4 s) and wait for extra_blocks (0 or 1)
 * more arrivals than blocks launched.  With extra_blocks = 1 no barrier can
 * complete: the kernel's blocks leave after limit_ms and the call returns
 * BYO_ETIMEDOUT with the context still usable.  (0, 0) restores the default.
 * No reference counterpart (the reference's waits are host-side, in
 * parlaylib's scheduler). */
int byo_ctx_set_barrier_test(byo_ctx *ctx, uint32_t limit_ms, uint32_t extra_blocks);
/* Brackets every launch of the kernels tagged `tag` ("*": all tags, NULL: off)
 * with CUDA events on the context's stream; byo_ctx_kernel_time sums the
 * launches of one tag (NULL: all) since the last byo_ctx_kernel_timing call.
 * Tags: "bfs_push", "bfs_pull", "bfs_blocked", "bfs_multi", "cc_finish",
 * "pr_pull", "pr_delta", "tc_intersect", "sort_scatter", "pma_merge",
 * "pma_redistribute". */
int byo_ctx_kernel_timing(byo_ctx *ctx, const char *tag);
int byo_ctx_kernel_time(byo_ctx *ctx, const char *tag, uint64_t *launches, double *ms);

/* ------------------------------------------------------------------ learned policy
 * A 16-32-32-5 FP32 MLP predicting log2(1 + microseconds)/16 of five actions:
 * 0 push, 1 pull, 2 blocked (per edgeMap round) and 3 in-place merge,
 * 4 rebuild (per container update).  Trained on the device by the library's
 * own kernels on samples the engine logs (round logs with round timing on,
 * byo_update_sample).  BYO_POLICY_LEARNED rounds and BYO_UPDATE_LEARNED
 * batches use it; the m/20 rule (edge_map_data.h:254-307) and in-place merge
 * remain the fallback and arbiter.  No counterpart in the reference beyond the
 * rule it learns around. */
#define BYO_POLICY_NFEATURES 16
#define BYO_POLICY_NOUTPUTS 5
#define BYO_POLICY_NPARAMS 1765
enum byo_update_policy { BYO_UPDATE_MERGE = 0, BYO_UPDATE_LEARNED = 1, BYO_UPDATE_REBUILD = 2 };
int byo_ctx_set_update_policy(byo_ctx *ctx, int policy);
/* strategy of the last batch: 0 merge, 1 rebuild */
int byo_ctx_last_update_strategy(const byo_ctx *ctx);
/* Seeded Xavier initialisation of the 1765 parameters (W1,b1,W2,b2,W3,b3). */
int byo_policy_init_params(uint64_t seed, float *h_params);
int byo_policy_set_params(byo_ctx *ctx, const float *h_params);
int byo_policy_get_params(byo_ctx *ctx, float *h_params);
/* Forget the network: learned policies fall back to the rules. */
int byo_policy_clear(byo_ctx *ctx);
int byo_policy_forward(byo_ctx *ctx, const float *h_params, const float *h_x, uint64_t n, float *h_y);
/* Mean squared error over the observed targets (bit o of mask[i] marks
 * y[i][o]) and its gradient with respect to the 1765 parameters. */
int byo_policy_loss_grad(byo_ctx *ctx, const float *h_params, const float *h_x, const float *h_y,
                         const uint8_t *h_mask, uint64_t n, float *loss, float *h_grad);
/* Adam on the device for `epochs` passes from h_init (NULL: seeded init);
 * installs the result as the context's policy. */
int byo_policy_train(byo_ctx *ctx, const float *h_init, const float *h_x, const float *h_y,
                     const uint8_t *h_mask, uint64_t n, uint32_t epochs, float lr, uint64_t seed,
                     float *h_loss_per_epoch);
/* Times the batch as in-place merge and as rebuild, for insert and remove
 * (contents restored in between); writes 2 samples (x[2][16], y[2][5], mask[2]). */
int byo_update_sample(byo_graph *g, const uint64_t *h_keys, uint64_t count, float *h_x, float *h_y,
                      uint8_t *h_mask);

/* ------------------------------------------------------------------ allocation-free BFS
 * No counterpart in the reference.  For callers that cannot let a library
 * allocate device memory: hosts whose memory manager reserves the whole GPU
 * up front and hands out sub-ranges itself (a buffer pool, a managed runtime
 * that owns one device arena), where a cudaMalloc inside the library would
 * fail or take memory the manager does not track.  BFS from src over the
 * caller's device CSR (d_offsets[n+1], d_nbrs[m], symmetric, sorted), on the
 * caller's stream (cudaStream_t, NULL = default) of the current device,
 * writing the same parents and levels as byo_bfs into the caller's device
 * arrays (either may be NULL, not both).  Calls no cudaMalloc / cudaFree:
 * the traversal state lives in one static device array sized for
 * BYO_NOALLOC_MAX_VERTICES vertices (16.4 MiB per GPU, held until exit);
 * n above that, src >= n or n == 0 return BYO_EINVAL.  The array is shared
 * by all calls: calls that overlap on the GPU race and must be serialised by
 * the caller.  The call is host-synchronous: it reads each round's frontier
 * size back and synchronises `stream` every round, and returns when the
 * result is in the output arrays.  The array's device address is looked up
 * on the first call in each CUDA context of a device and cached. */
#define BYO_NOALLOC_MAX_VERTICES (1u << 20)
int byo_bfs_csr_noalloc(const uint64_t *d_offsets, const uint32_t *d_nbrs, uint64_t n, uint64_t m,
                        uint32_t src, uint32_t *d_parent, uint32_t *d_level, void *stream,
                        uint32_t *rounds);

#ifdef __cplusplus
}
#endif
#endif

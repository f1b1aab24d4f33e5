/*
 * oracle.h -- CPU restatement of BYO's data-parallel hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path in
 * byo_gb300/ and the CPU baseline timed by bench.py.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU legs may load it.  The product
 * library (libbyo_gpu.so) never links, loads or calls it.
 *
 * Each function cites the reference file:line it restates (paths relative to
 * the wheatman/BYO tree).  The reference itself cannot be compiled here: every
 * GBBS header pulls parlaylib through gbbs/bridge.h:9-21 and parlaylib, the CPMA
 * and ParallelTools are un-vendored submodules.  Parity is pinned instead on the
 * reference's own unit-test vectors (test_bfs.cc, test_cc.cc) and on an
 * independent implementation (networkx) over the reference's inputs/ graphs;
 * see tests/golden/make_golden.py.
 *
 * Conventions (as in the reference): vertex ids are uint32 (uintE,
 * gbbs/macros.h), edge offsets uint64 (uintT), UINT32_MAX marks "unreached".
 * Update keys are uint64 src<<32 | dst (run_single_pma.cc:63-70 bit_casts a
 * std::tuple<uint32,uint32> to uint64, libstdc++ puts get<1> at the low word).
 *
 * Threading: functions parallelise with OpenMP; every result is independent of
 * the thread count.
 */
#ifndef BYO_ORACLE_H
#define BYO_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_NONE 0xFFFFFFFFu

/* ---------------------------------------------------------------- generators
 * Counter-based, so that any slice of the edge stream can be produced
 * independently (host or device) and bit-exactly.  The stream for a seed is
 *   key      = mix64(seed)
 *   draw(c)  = mix64(key + c * 0x9E3779B97F4A7C15)       (c = 64-bit counter)
 * where mix64 is the SplitMix64 output function (Steele, Lea & Flood,
 * "Fast splittable pseudorandom number generators", OOPSLA 2014).
 *
 * RMAT (Chakrabarti, Zhan & Faloutsos 2004) edge i uses counters i*32 + j:
 * level l (most significant bit first) takes the 32-bit word (l&1) of draw
 * j = l>>1 and compares it with the integer thresholds ta < tab < tabc
 * (probabilities scaled by 2^32); quadrant a = (0,0), b = (0,1) (dst bit),
 * c = (1,0) (src bit), d = (1,1).  This plays the role of the reference's
 * batch generator rMat (benchmarks/run_unweighted.h:730-778), with the
 * a/b/c/d split of the workload and an exact integer comparison.
 */
uint64_t orc_mix64(uint64_t x);
void orc_rmat_thresholds(double a, double b, double c, uint32_t out[3]);
void orc_rmat_edges(uint64_t seed, uint32_t lg_n, uint64_t first, uint64_t count,
                    const uint32_t thr[3], uint32_t *src, uint32_t *dst);
/* Uniform pairs in [0,n): draw(i) low word -> src, high word -> dst, each
 * reduced by multiply-shift ((w * n) >> 32).  Used for Erdos-Renyi G(n,m)
 * graphs and the insert/delete batches. */
void orc_uniform_pairs(uint64_t seed, uint64_t n, uint64_t first, uint64_t count,
                       uint32_t *src, uint32_t *dst);
/* rows x cols 4-neighbour grid: vertex r*cols+c, edges right and down. Returns
 * the number of pairs written (2*rows*cols - rows - cols). */
uint64_t orc_grid_pairs(uint32_t rows, uint32_t cols, uint32_t *src, uint32_t *dst);
/* Chung-Lu: endpoint i drawn with probability proportional to (i+1)^(-1/(g-1)).
 * cdf is the integer table built by orc_chung_lu_cdf (n entries, cdf[n-1] =
 * 2^63); endpoint = first i with (draw >> 1) < cdf[i]. */
void orc_chung_lu_cdf(uint64_t n, double exponent, uint64_t *cdf);
void orc_chung_lu_pairs(uint64_t seed, uint64_t n, const uint64_t *cdf, uint64_t first,
                        uint64_t count, uint32_t *src, uint32_t *dst);

/* ---------------------------------------------------------------- CSR build
 * Symmetrise (optional), drop self loops (optional), sort, deduplicate.
 * Mirrors graph_test::MakeUnweightedSymmetricGraph
 * (gbbs/unit_tests/graph_test_utils.h:35-60) and the sorted, duplicate-free
 * adjacency that run_csr.cc:87-106 expects.  offsets has n+1 entries; nbrs must
 * hold count*(symmetrise?2:1) entries.  Returns m (directed entries). */
uint64_t orc_build_csr(uint64_t n, const uint32_t *src, const uint32_t *dst, uint64_t count,
                       int symmetrise, int drop_self_loops, uint64_t *offsets, uint32_t *nbrs);

/* Sorts keys ascending (LSD radix) and removes duplicates; returns new count.
 * Restates parlay::unique(parlay::sort(...)) in Graph::insert_batch
 * (gbbs/graph.h:3090-3092). */
uint64_t orc_sort_unique_u64(uint64_t *keys, uint64_t count);

/* ---------------------------------------------------------------- algorithms */

/* BFS (benchmarks/BFS/NonDeterministicBFS/BFS.h:47-64) driven by edgeMap's
 * direction rule (gbbs/edge_map_data.h:254-307): dense pull when the frontier
 * is dense and larger than n/10, or |F| + sum deg(F) > m/20; sparse push
 * otherwise.  parent[v] is the canonical parent: the smallest neighbour of v at
 * level[v]-1 (what the dense pull returns on sorted adjacency), parent[src] =
 * src, ORC_NONE when unreached.  level may be NULL.  Returns the number of
 * rounds (levels discovered + 1). */
uint32_t orc_bfs(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs, uint32_t src,
                 uint32_t *parent, uint32_t *level);

/* Connectivity, SimpleUnionAsync (benchmarks/Connectivity/SimpleUnionAsync/
 * Connectivity.h:32-136): union-find hooking the larger root under the smaller
 * one, so each label is the minimum vertex id of its component. */
void orc_cc(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs, uint32_t *label);

/* BFS-based connectivity (benchmarks/Connectivity/BFSCC/Connectivity.h:33-88):
 * components discovered in increasing order of their smallest vertex; label =
 * that vertex.  Equal to orc_cc on every graph. */
void orc_bfs_cc(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs, uint32_t *label);

/* PageRank, dense pull (benchmarks/PageRank/PageRank.h:125-193 with
 * EdgeMap::edgeMapReduce_dense, gbbs/edge_map_reduce.h:458-487): p0 = 1/n,
 * p_div = p/deg, p_next[v] = 0.85 * sum_{u in N(v)} p_div[u] + 0.15/n (sum
 * left to right over sorted neighbours), stop when L1(p_curr, p_next) < eps or
 * after max_iters iterations; returns p_next.  No dangling redistribution.
 * iters_out (may be NULL) receives the number of iterations run; l1_out (may be
 * NULL) the last L1 norm. */
void orc_pagerank(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs, double eps,
                  uint32_t max_iters, double *p_out, uint32_t *iters_out, double *l1_out);

/* PageRank, delta variant (benchmarks/PageRank/PageRank.h:340-398,
 * delta::PageRankDelta): p0 = 0, delta0 = 1/n, frontier0 = all; each round
 * nghSum[v] = sum over neighbours u in the frontier of delta[u]/deg(u); first
 * round p += 0.85 nghSum + 0.15/n and delta = that - 1/n (active when delta >
 * local_eps p), later rounds delta = 0.85 nghSum, applied (and active) when
 * |delta| > local_eps p; stop when sum |delta| < eps or after max_iters rounds.
 * rounds_out / l1_out may be NULL. */
void orc_pagerank_delta(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs, double eps, double local_eps,
                        uint32_t max_iters, double *p, uint32_t *rounds_out, double *l1_out);

/* ---------------------------------------------------------------- byte-PD
 * The bytepd_amortized encoding of neighbour lists
 * (gbbs/encodings/byte_pd_amortized.h:1100-1155 sequentialCompressEdgeSet,
 * byte_pd_amortized.cc:7-55 compressFirstEdge / compressEdge, the reader
 * iter at byte_pd_amortized.h:180-260) and the compressed graph file
 * (gbbs/graph_io.h:351-390; utils/converter.h:671-760 writes it):
 *   file: int64 n, m, total bytes; uint64 byte offsets[n + 1]; uint32
 *   degrees[n]; the bytes.  A vertex of degree d > 0 starts with uint32 d,
 *   then uint32 byte offsets (from the vertex start) of blocks 1 .. nb-1,
 *   nb = 1 + (d-1)/P; block i holds uint32 i*P and then up to P neighbours:
 *   the first as (neighbour - source): byte 0 = bit 7 "more bytes", bit 6
 *   sign, bits 0-5 the low six bits of |difference|, further bytes 7 bits
 *   each (bit 7 "more"); the others as the positive difference to the
 *   previous neighbour, 7 bits per byte, bit 7 "more".  The reader uses
 *   P = PARALLEL_DEGREE = 1000 (gbbs/macros.h:83).  Neighbour lists must be
 *   strictly increasing (a zero difference has no encoding).
 * orc_bytepd_sizes: per-vertex byte counts into sizes[n]; returns the total.
 * orc_bytepd_encode: writes every vertex at byte_offsets[v] (exclusive prefix
 * of the sizes, byte_offsets[n] = total) into bytes.
 * orc_bytepd_decode: the CSR back (offsets from the degrees); returns 0, or -1
 * on a malformed run. */
uint64_t orc_bytepd_sizes(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs, uint32_t P, uint64_t *sizes);
void orc_bytepd_encode(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs, uint32_t P,
                       const uint64_t *byte_offsets, unsigned char *bytes);
int orc_bytepd_decode(uint64_t n, const uint64_t *byte_offsets, const uint32_t *degrees, const unsigned char *bytes,
                      uint64_t nbytes, uint32_t P, uint64_t *offsets, uint32_t *nbrs);

/* Test_Map (benchmarks/Map/Base/Map.h:8-18): sum over every edge of its
 * destination id.  Test_Map_Remote (benchmarks/Map/RemoteRead/Map.h:21-33):
 * sum over every edge (u, v) of remote[v], remote an n-entry array of
 * `width`-byte elements (0: bitmap of 64-bit words, least significant bit
 * first; 1, 2, 4, 8: unsigned integers; 16, 32: a uint64 at the start of the
 * element). */
uint64_t orc_map_sum(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs);
uint64_t orc_map_remote(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs, const void *remote,
                        uint32_t width);

/* Triangle counting, degree ordering (benchmarks/TriangleCounting/
 * ShunTangwongsan15/Triangle.h:57-68,99-150,167-204): rank by (degree, id),
 * orient u->v when rank[u] < rank[v], count |N+(u) cap N+(v)| over DAG edges by
 * sorted merge (gbbs/intersect.h:111-134). */
uint64_t orc_triangle_count(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs);

/* ---------------------------------------------------------------- container model
 * The container's observable contents as a set of (src,dst) keys held in
 * per-vertex sorted arrays.  insert = set union, remove = set difference,
 * after sort+unique of the batch, which is what Graph::insert_batch /
 * remove_batch (gbbs/graph.h:3071-3124) feed PMA_graph::insert_sorted_batch /
 * remove_sorted_batch (benchmarks/run_structures/run_single_pma.cc:63-70).
 * The batch is taken as given (keys are not symmetrised; self loops allowed). */
typedef struct orc_store orc_store;
orc_store *orc_store_create(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs);
void orc_store_destroy(orc_store *s);
uint64_t orc_store_num_edges(const orc_store *s);
/* keys are copied; returns the number of keys newly inserted / removed */
uint64_t orc_store_insert_batch(orc_store *s, const uint64_t *keys, uint64_t count);
uint64_t orc_store_remove_batch(orc_store *s, const uint64_t *keys, uint64_t count);
/* writes offsets[n+1], nbrs[m] (sorted adjacency) */
void orc_store_export_csr(const orc_store *s, uint64_t *offsets, uint32_t *nbrs);

int orc_num_threads(void);
void orc_set_num_threads(int t);

#ifdef __cplusplus
}
#endif
#endif

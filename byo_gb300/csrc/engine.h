// engine.h -- the edgeMap / vertexSubset engine shared by BFS, BFS-CC and the
// public edgeMap API.
//
// One traversal state (the BFS_F functor of BFS.h:30-45 with its Parents
// array) is a packed word per vertex, lp[v] = level << 32 | parent, plus a
// "visited before this round" bitmap (cond(v) of the functor).  A round reads
// frontier F (list and/or bitmap) and writes the next frontier as both a list
// and a bitmap, so no sparse<->dense conversion pass is ever needed.
//
//   push     (edgeMapSparse, edge_map_blocked.h:18-92): groups of lanes per
//            frontier vertex, coalesced neighbour loads, atomicMin on lp so the
//            smallest-id parent of this level wins; hubs go to one CTA each.
//   blocked  (edgeMapBlocked, edge_map_blocked.h:130-246): edge-balanced tiles
//            over the exclusive scan of frontier degrees (merge-path split).
//   pull     (edgeMapDense, edge_map_data.h:47-175): one thread per unvisited
//            vertex, warp per 32-vertex bitmap word, early exit at the first
//            frontier neighbour (= smallest id, adjacency is sorted), frontier
//            bitmap prefix staged in shared memory; long scans deferred to a
//            warp-cooperative pass.
#pragma once

#include "internal.h"

namespace byo {

// MODE_DENSE_FWD (edgeMapDenseForward) is asked for only through the edgeMap
// API's flag; the direction policies choose among the first three.
enum Mode { MODE_PUSH = 0, MODE_PULL = 1, MODE_BLOCKED = 2, MODE_DENSE_FWD = 3 };

struct RoundStats {
  unsigned long long count;   // |next frontier|
  unsigned long long outdeg;  // sum of degrees of the next frontier
  unsigned long long ndefer;  // pull: deferred long scans; push: hubs
  unsigned long long edges;   // edges examined (diagnostic)
  unsigned long long hist[8]; // degree sketch of the next frontier (log4 bins)
  unsigned long long mode;    // next round's mode chosen by the policy kernel
  float feat[16];             // the features that choice was made from
};

struct Frontier {
  uint32_t *list = nullptr;  // uint32[n]
  uint32_t *bits = nullptr;  // uint32[W]
  uint64_t size = 0;
  uint64_t outdeg = 0;
  bool dense = false;        // produced by a dense round
  bool has_list = false, has_bits = false;
  unsigned long long hist[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int next_mode = 0;    // policy kernel's choice for the round consuming this frontier
  float feat[16] = {0}; // its features
};

struct TravState {
  uint64_t *lp = nullptr;        // level<<32 | parent
  uint32_t *visited = nullptr;   // uint32[W]
  uint32_t round = 0;            // level being discovered next
  uint64_t reached = 0;          // vertices with a level so far
};

struct EngineTuning {
  int push_group = 8;        // lanes per frontier vertex in push
  uint32_t hub_min = 4096;   // degree at which push hands a vertex to a CTA
  int pull_cap = 32;         // neighbours a pull thread scans before deferring
  int pull_stage_words = 32768;  // frontier bitmap words staged in shared memory
  int blocked_tile = 2048;   // edges per blocked tile
};

// Decision of the GBBS rule for the next round (edge_map_data.h:254-307).
int m20_mode(const byo_graph *g, const Frontier &f, int64_t threshold, int sparse_mode);

// Runs one edgeMap round over BFS_F semantics: reads `in`, writes `out`
// (out.bits must be all zero; out.list capacity n).  Updates st.
int edge_map_round(byo_graph *g, TravState &st, Frontier &in, Frontier &out, int mode,
                   const EngineTuning &tune, bool run_policy = false);
// Zeroes a frontier bitmap using its list when that is cheaper.
int clear_frontier_bits(byo_graph *g, Frontier &f);
int ensure_bits(byo_graph *g, Frontier &f);
int trav_init(byo_graph *g, TravState &st, uint32_t src);
int trav_extract(byo_graph *g, const TravState &st, uint32_t *d_parent, uint32_t *d_level);
EngineTuning default_tuning(const byo_graph *g);
// Runs push rounds from *cur in one persistent kernel while the frontier
// stays within `limit` edges (and, with gate_hub, holds no vertex of degree
// >= 4^5); on return *cur is the frontier reached and *nxt a clean buffer
// (bfs_small.cu).  With d_st, the final frontier's statistics are written
// there for the policy.
int bfs_small_rounds(byo_graph *g, TravState &st, Frontier *&cur, Frontier *&nxt, uint64_t limit, bool gate_hub,
                     RoundStats *d_st, uint32_t *rounds_run);

// ---- the edgeMap functors other than BFS_F, vertexMap / vertexFilter (edgemap.cu)
struct FunctorArgs {
  int kind = 0;                   // BYO_F_BFS_LABEL, BYO_F_PR, BYO_F_PR_DELTA
  uint32_t *parents = nullptr;    // BFS_LABEL: Parents
  uint32_t src = 0;               // BFS_LABEL: the label written
  const double *p_curr = nullptr; // PR
  double *p_next = nullptr;
  const double *delta = nullptr;  // PR_DELTA: [2n] delta, delta / degree
  double *ngh = nullptr;          // PR_DELTA: nghSum
};
struct VertexOpArgs {
  int kind;           // BYO_VOP_*
  double *a, *b, *c;  // per kind (include/byo_gpu.h)
  double damping, eps2;
};
// One edgeMap round of a generic functor: reads `in`, writes `out` (out.bits
// all zero, list capacity n) unless !output.
int generic_edge_map(byo_graph *g, const FunctorArgs &f, Frontier &in, Frontier &out, int mode, bool output);
// vertexMap (out == nullptr) or vertexFilter (out: bits all zero) over `in`.
int vertex_op_run(byo_graph *g, const VertexOpArgs &op, Frontier &in, Frontier *out);
// Builds f.list (and size, outdeg) from f.bits when only the bitmap is held.
int ensure_list(byo_graph *g, Frontier &f);
// f.bits = d_bits (every vertex when null), then its list, size and outdeg.
int frontier_from_bits(byo_graph *g, const uint32_t *d_bits, Frontier &f);
int pagerank_edgemap_run(byo_graph *g, double eps, uint32_t max_iters, double *d_p, uint32_t *iters, double *l1);

// Arguments of the policy epilogue fused into a round's last kernel
// (policy.cuh); on == 0 disables it.
struct PolicyTail {
  const float *P = nullptr;
  float n = 0, m = 0, reached_before = 0;
  int dense = 0, has_net = 0, on = 0, log = 0, prefetch = 0;
  unsigned int *done = nullptr;  // blocks finished; the last one resets it
};
// Fills pt for a round reading a frontier of the given kind (mlp.cu).
int policy_tail_args(byo_graph *g, unsigned int *done, uint64_t reached_before, bool this_round_dense,
                     PolicyTail *pt);

// Policy kernel after a round (mlp.cu): features of the frontier in d_st,
// the m/20 rule's choice, and the network's choice when one is trained;
// writes d_st->mode and d_st->feat.
int round_policy(byo_graph *g, RoundStats *d_st, uint64_t reached_before, bool this_round_dense);
bool policy_trained(const byo_ctx *ctx);

}  // namespace byo

// byo_gpu_graph.hpp -- C++ container adapters over the byo_gpu C ABI, in the
// shape BYO's gbbs::Graph<Rep, symmetric, API> consumes
// (gbbs/graph.h:2154-2421), so that a benchmarks/run_structures target can
// put a GB300-resident graph where run_csr.cc / run_single_pma.cc put theirs.
//
//   GPU_CSR            replaces CSR<node_t, edge_t>   (run_csr.cc:28-175)
//   GPU_PMA_graph<W>   replaces PMA_graph<W>          (run_single_pma.cc:39-141)
//
// Both expose the container concept: num_vertices()/N(), num_edges(),
// degree(i), map_neighbors(i, f), map_neighbors_early_exit(i, f),
// parallel_map_neighbors(i, f), parallel_map_neighbors_early_exit(i, f), the
// loader constructor Rep(v_data, n, m, deleter, edges) and, for the PMA,
// insert_sorted_batch / remove_sorted_batch(std::tuple<uint32_t,uint32_t>*, n).
// Neighbour maps run on the host over a mirror of the device adjacency that is
// refreshed after every update, so any GBBS algorithm still works; the hot
// algorithms run on the GPU through the free functions gpu_bfs, gpu_bfs_multi,
// gpu_cc, gpu_bfs_cc, gpu_pagerank, gpu_pagerank_delta, gpu_triangle_count,
// gpu_map and gpu_map_remote.
//
// The edgeMap / vertexSubset API (gbbs/edge_map_data.h:254-315,
// gbbs/vertex_subset.h:202-485) runs on the device: vertexSubset, the
// functors BFS_F, BFS_ComponentLabel_F, PR_F and PR_Delta_F over
// DeviceVector arrays, edgeMap, vertexMap and vertexFilter.
//
// Errors from the C ABI throw byo::Error (the reference aborts instead).
#pragma once

#include <cstdint>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "byo_gpu.h"

namespace byo {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// One process-wide context per device (the reference drives its graph from
// one host thread as well).
class Context {
 public:
  static Context &get(int device = 0) {
    static Context c(device);
    return c;
  }
  byo_ctx *h() const { return ctx_; }
  void check(int rc, const char *what) const {
    if (rc != BYO_OK) throw Error(rc, std::string(what) + ": " + byo_last_error(ctx_));
  }
  ~Context() {
    if (ctx_) byo_gpu_shutdown(ctx_);
  }

 private:
  explicit Context(int device) {
    int rc = byo_gpu_init(device, &ctx_);
    if (rc != BYO_OK) throw Error(rc, "byo_gpu_init failed");
  }
  byo_ctx *ctx_ = nullptr;
};

namespace detail {

// Shared body of both adapters: the device graph plus a host mirror.
class DeviceGraph {
 public:
  using weight_type = struct empty_w {};

  DeviceGraph() = default;
  DeviceGraph(int container, const uint64_t *off, const uint32_t *nbrs, uint64_t n, uint64_t m) {
    Context &c = Context::get();
    c.check(byo_graph_create(c.h(), container, n, m, off, nbrs, &g_), "create graph");
    refresh();
  }
  DeviceGraph(const DeviceGraph &) = delete;
  DeviceGraph &operator=(const DeviceGraph &) = delete;
  DeviceGraph(DeviceGraph &&o) noexcept { *this = std::move(o); }
  DeviceGraph &operator=(DeviceGraph &&o) noexcept {
    std::swap(g_, o.g_);
    off_.swap(o.off_);
    nbrs_.swap(o.nbrs_);
    return *this;
  }
  ~DeviceGraph() {
    if (g_) byo_graph_destroy(g_);
  }

  byo_graph *handle() const { return g_; }
  size_t num_vertices() const { return byo_graph_num_vertices(g_); }
  size_t N() const { return num_vertices(); }
  size_t num_edges() const { return byo_graph_num_edges(g_); }
  size_t degree(size_t i) const { return off_[i + 1] - off_[i]; }

  template <class F>
  void map_neighbors(size_t i, F f) const {
    weight_type w{};
    for (uint64_t j = off_[i]; j < off_[i + 1]; j++) f(i, nbrs_[j], w);
  }
  template <class F>
  void map_neighbors_early_exit(size_t i, F f) const {
    weight_type w{};
    for (uint64_t j = off_[i]; j < off_[i + 1]; j++)
      if (f(i, nbrs_[j], w)) break;
  }
  template <class F>
  void parallel_map_neighbors(size_t i, F f) const {
    map_neighbors(i, f);
  }
  template <class F, typename Block_F = std::nullptr_t>
  void parallel_map_neighbors_early_exit(size_t i, F f, Block_F = {}) const {
    map_neighbors_early_exit(i, f);
  }

  // device-side views of the mirror refresh
  void refresh() {
    off_.assign(num_vertices() + 1, 0);
    nbrs_.assign(num_edges() ? num_edges() : 1, 0);
    Context::get().check(byo_graph_export_csr(g_, off_.data(), nbrs_.data()), "export adjacency");
  }
  const std::vector<uint64_t> &offsets() const { return off_; }
  const std::vector<uint32_t> &edges() const { return nbrs_; }

 protected:
  byo_graph *g_ = nullptr;
  std::vector<uint64_t> off_;
  std::vector<uint32_t> nbrs_;
};

template <class VData, class Edge>
void loader_csr(const VData *v_data, size_t n, const Edge *e0, std::vector<uint64_t> &off,
                std::vector<uint32_t> &nbrs) {
  off.assign(n + 1, 0);
  for (size_t i = 0; i < n; i++) off[i + 1] = off[i] + v_data[i].degree;
  nbrs.resize(off[n]);
  for (size_t i = 0; i < n; i++)
    for (size_t j = 0; j < v_data[i].degree; j++) nbrs[off[i] + j] = std::get<0>(e0[v_data[i].offset + j]);
}

}  // namespace detail

// Static CSR on the GPU (run_csr.cc:28-175).
class GPU_CSR : public detail::DeviceGraph {
 public:
  using vertex_weight_type = double;
  GPU_CSR() = default;
  GPU_CSR(const uint64_t *off, const uint32_t *nbrs, uint64_t n, uint64_t m)
      : DeviceGraph(BYO_CONTAINER_CSR, off, nbrs, n, m) {}
  // the loader constructor of run_csr.cc:87-106
  template <class VData, class Edge>
  GPU_CSR(VData *v_data, size_t n, size_t, std::function<void()> deletion_fn, Edge *e0,
          vertex_weight_type * = nullptr) {
    std::vector<uint64_t> off;
    std::vector<uint32_t> nbrs;
    detail::loader_csr(v_data, n, e0, off, nbrs);
    static_cast<DeviceGraph &>(*this) = DeviceGraph(BYO_CONTAINER_CSR, off.data(), nbrs.data(), n, nbrs.size());
    if (deletion_fn) deletion_fn();
  }
};

// Packed-memory-array graph on the GPU (run_single_pma.cc:39-141).
template <class W>
class GPU_PMA_graph : public detail::DeviceGraph {
 public:
  using vertex_weight_type = double;
  using edge_type = std::tuple<uint32_t, W>;
  GPU_PMA_graph() = default;
  GPU_PMA_graph(const uint64_t *off, const uint32_t *nbrs, uint64_t n, uint64_t m)
      : DeviceGraph(BYO_CONTAINER_PMA, off, nbrs, n, m) {}
  template <class VData, class Edge>
  GPU_PMA_graph(VData *v_data, size_t n, size_t m, std::function<void()> deletion_fn, Edge *e0,
                vertex_weight_type *w = nullptr)
      : GPU_PMA_graph(BYO_CONTAINER_PMA, v_data, n, m, deletion_fn, e0, w) {}

 protected:
  // the same loader path into another updatable container (GPU_VOS_graph)
  template <class VData, class Edge>
  GPU_PMA_graph(int container, VData *v_data, size_t n, size_t, std::function<void()> deletion_fn, Edge *e0,
                vertex_weight_type *) {
    std::vector<uint64_t> off;
    std::vector<uint32_t> nbrs;
    detail::loader_csr(v_data, n, e0, off, nbrs);
    static_cast<DeviceGraph &>(*this) = DeviceGraph(container, off.data(), nbrs.data(), n, nbrs.size());
    if (deletion_fn) deletion_fn();
  }
  GPU_PMA_graph(int container, const uint64_t *off, const uint32_t *nbrs, uint64_t n, uint64_t m)
      : DeviceGraph(container, off, nbrs, n, m) {}

 public:

  // PMA_graph::insert_sorted_batch / remove_sorted_batch: the tuple array is
  // read as uint64 (src << 32 | dst) keys, as the reference bit_casts it.
  void insert_sorted_batch(std::tuple<uint32_t, uint32_t> *es, size_t n) { update(es, n, true); }
  void remove_sorted_batch(std::tuple<uint32_t, uint32_t> *es, size_t n) { update(es, n, false); }
  // Graph::insert_batch / remove_batch with unsorted, duplicated input
  void insert_batch(std::tuple<uint32_t, uint32_t> *es, size_t n) { update_unsorted(es, n, true); }
  void remove_batch(std::tuple<uint32_t, uint32_t> *es, size_t n) { update_unsorted(es, n, false); }

 private:
  static std::vector<uint64_t> keys_of(const std::tuple<uint32_t, uint32_t> *es, size_t n) {
    std::vector<uint64_t> k(n);
    for (size_t i = 0; i < n; i++) k[i] = ((uint64_t)std::get<0>(es[i]) << 32) | std::get<1>(es[i]);
    return k;
  }
  void update(const std::tuple<uint32_t, uint32_t> *es, size_t n, bool ins) {
    std::vector<uint64_t> k = keys_of(es, n);
    int rc = ins ? byo_graph_insert_batch(g_, k.data(), n, 1, nullptr)
                 : byo_graph_remove_batch(g_, k.data(), n, 1, nullptr);
    Context::get().check(rc, ins ? "insert_sorted_batch" : "remove_sorted_batch");
    refresh();
  }
  void update_unsorted(const std::tuple<uint32_t, uint32_t> *es, size_t n, bool ins) {
    std::vector<uint64_t> k = keys_of(es, n);
    int rc = ins ? byo_graph_insert_batch(g_, k.data(), n, 0, nullptr)
                 : byo_graph_remove_batch(g_, k.data(), n, 0, nullptr);
    Context::get().check(rc, ins ? "insert_batch" : "remove_batch");
    refresh();
  }
};

// Vector of per-vertex sorted sets on the GPU (run_vector_pma.cc,
// run_vector_vector.cc: gbbs::symmetric_set_graph over one set per vertex):
// the same interface as GPU_PMA_graph over BYO_CONTAINER_VOS.
template <class W>
class GPU_VOS_graph : public GPU_PMA_graph<W> {
 public:
  using typename GPU_PMA_graph<W>::vertex_weight_type;
  GPU_VOS_graph() = default;
  GPU_VOS_graph(const uint64_t *off, const uint32_t *nbrs, uint64_t n, uint64_t m)
      : GPU_PMA_graph<W>(BYO_CONTAINER_VOS, off, nbrs, n, m) {}
  template <class VData, class Edge>
  GPU_VOS_graph(VData *v_data, size_t n, size_t m, std::function<void()> deletion_fn, Edge *e0,
                vertex_weight_type *w = nullptr)
      : GPU_PMA_graph<W>(BYO_CONTAINER_VOS, v_data, n, m, deletion_fn, e0, w) {}
};

// The PCSR target (run_pcsr.cc:24-99, symmetric_PCSR_graph) over
// BYO_CONTAINER_PCSR: one packed array of per-vertex sentinels and sorted
// neighbour ids with gaps, and a per-vertex index into it that the batch
// updates keep current; the same interface as GPU_PMA_graph.
template <class W>
class GPU_PCSR_graph : public GPU_PMA_graph<W> {
 public:
  using typename GPU_PMA_graph<W>::vertex_weight_type;
  GPU_PCSR_graph() = default;
  GPU_PCSR_graph(const uint64_t *off, const uint32_t *nbrs, uint64_t n, uint64_t m)
      : GPU_PMA_graph<W>(BYO_CONTAINER_PCSR, off, nbrs, n, m) {}
  template <class VData, class Edge>
  GPU_PCSR_graph(VData *v_data, size_t n, size_t m, std::function<void()> deletion_fn, Edge *e0,
                 vertex_weight_type *w = nullptr)
      : GPU_PMA_graph<W>(BYO_CONTAINER_PCSR, v_data, n, m, deletion_fn, e0, w) {}
};

// ---------------------------------------------------------------- GPU algorithms
// BFS (BFS.h:47-64): Parents with UINT_E_MAX for unreached, parent[src] = src.
inline std::vector<uint32_t> gpu_bfs(const detail::DeviceGraph &G, uint32_t src, int policy = BYO_POLICY_M20) {
  std::vector<uint32_t> parents(G.num_vertices());
  Context::get().check(byo_bfs(G.handle(), src, parents.data(), nullptr, policy, nullptr), "bfs");
  return parents;
}
// SimpleUnionAsync (Connectivity.h:122-136): minimum vertex id per component.
inline std::vector<uint32_t> gpu_cc(const detail::DeviceGraph &G) {
  std::vector<uint32_t> label(G.num_vertices());
  Context::get().check(byo_cc(G.handle(), label.data()), "cc");
  return label;
}
// PageRank (PageRank.h:125-193).
inline std::vector<double> gpu_pagerank(const detail::DeviceGraph &G, double eps = 1e-6, uint32_t iters = 100,
                                        int precision = BYO_PR_FP32_KAHAN) {
  std::vector<double> p(G.num_vertices());
  Context::get().check(byo_pagerank(G.handle(), eps, iters, precision, p.data(), nullptr, nullptr), "pagerank");
  return p;
}
// Triangle_degree_ordering (Triangle.h:167-204).
inline uint64_t gpu_triangle_count(const detail::DeviceGraph &G) {
  uint64_t c = 0;
  Context::get().check(byo_triangle_count(G.handle(), &c), "triangle_count");
  return c;
}
// Test_Map (benchmarks/Map/Base/Map.h:8-18).
inline uint64_t gpu_map(const detail::DeviceGraph &G) {
  uint64_t s = 0;
  Context::get().check(byo_map_sum(G.handle(), &s), "map");
  return s;
}
// Test_Map_Remote (benchmarks/Map/RemoteRead/Map.h:21-33) over a host array of
// W-byte elements (W = 1, 2, 4, 8; wider elements through byo_map_remote).
template <class T>
inline uint64_t gpu_map_remote(const detail::DeviceGraph &G, const std::vector<T> &remote) {
  static_assert(sizeof(T) <= 8 && (sizeof(T) & (sizeof(T) - 1)) == 0, "1, 2, 4 or 8-byte elements");
  uint64_t s = 0;
  Context::get().check(byo_map_remote(G.handle(), remote.data(), (uint32_t)sizeof(T), &s), "map_remote");
  return s;
}
// delta::PageRankDelta (PageRank.h:340-398).
inline std::vector<double> gpu_pagerank_delta(const detail::DeviceGraph &G, double eps = 1e-6, double local_eps = 0.01,
                                              uint32_t iters = 100) {
  std::vector<double> p(G.num_vertices());
  Context::get().check(byo_pagerank_delta(G.handle(), eps, local_eps, iters, p.data(), nullptr, nullptr),
                       "pagerank_delta");
  return p;
}
// BFS levels from up to 64 sources in one traversal: levels[s * n + v].
inline std::vector<uint32_t> gpu_bfs_multi(const detail::DeviceGraph &G, const std::vector<uint32_t> &sources) {
  std::vector<uint32_t> levels(sources.size() * G.num_vertices());
  Context::get().check(byo_bfs_multi(G.handle(), sources.data(), (uint32_t)sources.size(), levels.data(), nullptr),
                       "bfs_multi");
  return levels;
}
// SimpleUnionAsync's labels through BFS-CC (Connectivity.h:33-88 of BFSCC).
inline std::vector<uint32_t> gpu_bfs_cc(const detail::DeviceGraph &G) {
  std::vector<uint32_t> label(G.num_vertices());
  Context::get().check(byo_bfs_cc(G.handle(), label.data()), "bfs_cc");
  return label;
}

// ---------------------------------------------------------------- edgeMap API
// A device array of T on the context's device (the arrays the functors read
// and write).
template <class T>
class DeviceVector {
 public:
  explicit DeviceVector(size_t n, T init = T()) : n_(n) {
    Context &c = Context::get();
    c.check(byo_buffer_alloc(c.h(), n * sizeof(T), &d_), "device vector");
    std::vector<T> h(n, init);
    c.check(byo_buffer_write(c.h(), d_, 0, h.data(), n * sizeof(T)), "device vector fill");
  }
  DeviceVector(const DeviceVector &) = delete;
  DeviceVector &operator=(const DeviceVector &) = delete;
  ~DeviceVector() { byo_buffer_free(Context::get().h(), d_); }
  T *data() const { return static_cast<T *>(d_); }
  size_t size() const { return n_; }
  std::vector<T> to_host() const {
    std::vector<T> h(n_);
    Context::get().check(byo_buffer_read(Context::get().h(), d_, 0, h.data(), n_ * sizeof(T)), "device vector read");
    return h;
  }
  void swap(DeviceVector &o) noexcept {
    std::swap(d_, o.d_);
    std::swap(n_, o.n_);
  }
  void assign(const std::vector<T> &h) {
    Context::get().check(byo_buffer_write(Context::get().h(), d_, 0, h.data(), n_ * sizeof(T)), "device vector write");
  }

 private:
  void *d_ = nullptr;
  size_t n_;
};

// vertexSubset (vertex_subset.h:240-270): one vertex, a list, every vertex
// (BitArray(n, true)) or the set bits of a device bitmap.
class vertexSubset {
 public:
  vertexSubset(const detail::DeviceGraph &G, uint32_t v) { check(byo_vs_create_single(G.handle(), v, &h_)); }
  vertexSubset(const detail::DeviceGraph &G, const std::vector<uint32_t> &ids) {
    check(byo_vs_create_list(G.handle(), ids.data(), ids.size(), &h_));
  }
  static vertexSubset all(const detail::DeviceGraph &G) {
    vertexSubset s;
    s.check(byo_vs_create_all(G.handle(), &s.h_));
    return s;
  }
  static vertexSubset from_bitmap(const detail::DeviceGraph &G, const DeviceVector<uint32_t> &bits) {
    vertexSubset s;
    s.check(byo_vs_create_bitmap(G.handle(), bits.data(), &s.h_));
    return s;
  }
  explicit vertexSubset(byo_vertex_subset *h) : h_(h) {}
  vertexSubset(vertexSubset &&o) noexcept : h_(o.h_) { o.h_ = nullptr; }
  vertexSubset &operator=(vertexSubset &&o) noexcept {
    std::swap(h_, o.h_);
    return *this;
  }
  vertexSubset(const vertexSubset &) = delete;
  ~vertexSubset() {
    if (h_) byo_vs_destroy(h_);
  }
  size_t size() const { return byo_vs_size(h_); }
  bool isEmpty() const { return size() == 0; }
  bool isDense() const { return byo_vs_is_dense(h_) == 1; }
  std::vector<uint32_t> toSparse() const {
    std::vector<uint32_t> ids(size());
    check(byo_vs_to_list(h_, ids.data(), ids.size()));
    return ids;
  }
  byo_vertex_subset *handle() const { return h_; }

 private:
  vertexSubset() = default;
  void check(int rc) const { Context::get().check(rc, "vertexSubset"); }
  byo_vertex_subset *h_ = nullptr;
};

// The device functors (a GBBS functor struct's update / updateAtomic / cond).
class Functor {
 public:
  Functor(Functor &&o) noexcept : h_(o.h_) { o.h_ = nullptr; }
  Functor(const Functor &) = delete;
  ~Functor() {
    if (h_) byo_functor_destroy(h_);
  }
  byo_functor *handle() const { return h_; }

 protected:
  Functor() = default;
  byo_functor *h_ = nullptr;
};
// BFS_F (BFS.h:30-45) over its own Parents array.
class BFS_F : public Functor {
 public:
  BFS_F(const detail::DeviceGraph &G, uint32_t src) {
    Context::get().check(byo_functor_bfs_create(G.handle(), src, &h_), "BFS_F");
  }
  std::vector<uint32_t> parents(size_t n) const {
    std::vector<uint32_t> p(n);
    Context::get().check(byo_functor_bfs_parents(h_, p.data()), "BFS_F parents");
    return p;
  }
};
// BFS_ComponentLabel_F (benchmarks/Connectivity/BFSCC/Connectivity.h:31-50).
class BFS_ComponentLabel_F : public Functor {
 public:
  BFS_ComponentLabel_F(const detail::DeviceGraph &G, DeviceVector<uint32_t> &parents, uint32_t src) {
    Context::get().check(byo_functor_bfs_label_create(G.handle(), src, parents.data(), &h_), "BFS_ComponentLabel_F");
  }
};
// PR_F (benchmarks/PageRank/PageRank.h:33-50).
class PR_F : public Functor {
 public:
  PR_F(const detail::DeviceGraph &G, const DeviceVector<double> &p_curr, DeviceVector<double> &p_next) {
    Context::get().check(byo_functor_pr_create(G.handle(), p_curr.data(), p_next.data(), &h_), "PR_F");
  }
};
// delta::PR_Delta_F (PageRank.h:200-226): delta holds n {delta, delta/degree} pairs.
class PR_Delta_F : public Functor {
 public:
  PR_Delta_F(const detail::DeviceGraph &G, const DeviceVector<double> &delta, DeviceVector<double> &ngh_sum) {
    Context::get().check(byo_functor_pr_delta_create(G.handle(), delta.data(), ngh_sum.data(), &h_), "PR_Delta_F");
  }
};

// edgeMap (edge_map_data.h:312-315); flags as gbbs/flags.h (BYO_FL_*).
inline vertexSubset edgeMap(const detail::DeviceGraph &G, const vertexSubset &vs, const Functor &f,
                            int64_t threshold = -1, uint32_t flags = 0) {
  byo_vertex_subset *out = nullptr;
  Context::get().check(byo_edge_map(G.handle(), vs.handle(), f.handle(), threshold, flags, &out), "edgeMap");
  return vertexSubset(out);
}
// vertexMap / vertexFilter (vertex_subset.h:382-485) with the reference's
// vertex functions (BYO_VOP_*, arrays as byo_vertex_op describes).
inline void vertexMap(const vertexSubset &vs, const byo_vertex_op &op) {
  Context::get().check(byo_vertex_map(vs.handle(), &op), "vertexMap");
}
inline vertexSubset vertexFilter(const vertexSubset &vs, const byo_vertex_op &op) {
  byo_vertex_subset *out = nullptr;
  Context::get().check(byo_vertex_filter(vs.handle(), &op, &out), "vertexFilter");
  return vertexSubset(out);
}

}  // namespace byo

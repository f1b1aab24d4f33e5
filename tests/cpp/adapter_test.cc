// Exercises include/byo_gpu_graph.hpp the way a benchmarks/run_structures
// target would: the loader's (vertex_data, edges) arrays into GPU_CSR and
// GPU_PMA_graph, the container concept, batch updates and the GPU algorithms.
// Graph: test_bfs.cc:26-50 (0-1, 2-3, 3-4, 3-5, 4-5, 5-6).
#include <cstdio>
#include <cstdlib>
#include <tuple>
#include <vector>

#include "byo_gpu_graph.hpp"

struct vertex_data {
  uint64_t offset;
  uint64_t degree;
};

#define CHECK(c)                                              \
  do {                                                        \
    if (!(c)) {                                               \
      std::fprintf(stderr, "check failed line %d: %s\n", __LINE__, #c); \
      return 1;                                               \
    }                                                         \
  } while (0)

int main() {
  const size_t n = 7;
  std::vector<std::vector<uint32_t>> adj = {{1}, {0}, {3}, {2, 4, 5}, {3, 5}, {3, 4, 6}, {5}};
  std::vector<vertex_data> vd(n);
  std::vector<std::tuple<uint32_t, int>> edges;
  for (size_t v = 0; v < n; v++) {
    vd[v] = {edges.size(), adj[v].size()};
    for (uint32_t u : adj[v]) edges.emplace_back(u, 0);
  }
  bool deleted = false;
  byo::GPU_CSR csr(vd.data(), n, edges.size(), [&] { deleted = true; }, edges.data());
  CHECK(deleted);
  CHECK(csr.num_vertices() == 7 && csr.num_edges() == 12);
  CHECK(csr.degree(3) == 3 && csr.degree(6) == 1);
  std::vector<uint32_t> seen;
  csr.map_neighbors(5, [&](size_t, uint32_t u, auto) { seen.push_back(u); });
  CHECK((seen == std::vector<uint32_t>{3, 4, 6}));
  int visits = 0;
  csr.map_neighbors_early_exit(3, [&](size_t, uint32_t u, auto) { visits++; return u == 4; });
  CHECK(visits == 2);
  // BFS(2): parents {NONE, NONE, 2, 2, 3, 3, 5} (canonical min-id parents)
  auto par = byo::gpu_bfs(csr, 2);
  const uint32_t X = BYO_NONE;
  CHECK((par == std::vector<uint32_t>{X, X, 2, 2, 3, 3, 5}));
  auto lab = byo::gpu_cc(csr);
  CHECK((lab == std::vector<uint32_t>{0, 0, 2, 2, 2, 2, 2}));
  CHECK(byo::gpu_triangle_count(csr) == 1);
  auto pr = byo::gpu_pagerank(csr, 1e-9, 200, BYO_PR_FP64);
  double sum = 0;
  for (double x : pr) sum += x;
  CHECK(sum > 0.5 && sum < 1.01);
  auto prd = byo::gpu_pagerank_delta(csr);
  CHECK(prd.size() == n && prd[3] > 0);
  CHECK((byo::gpu_bfs_cc(csr) == lab));
  // edge destination sum: 1+0+3+2+4+5+3+5+3+4+6+5 = 41; remote[3] = 1 counts 3's in-edges
  CHECK(byo::gpu_map(csr) == 41);
  std::vector<uint16_t> remote(n, 0);
  remote[3] = 1;
  CHECK(byo::gpu_map_remote(csr, remote) == 3);
  // levels from 2 and 0 in one traversal
  auto lv = byo::gpu_bfs_multi(csr, {2, 0});
  CHECK((std::vector<uint32_t>(lv.begin(), lv.begin() + n) == std::vector<uint32_t>{X, X, 0, 1, 2, 2, 3}));
  CHECK((std::vector<uint32_t>(lv.begin() + n, lv.end()) == std::vector<uint32_t>{0, 1, X, X, X, X, X}));

  byo::GPU_PMA_graph<int> pma(vd.data(), n, edges.size(), nullptr, edges.data());
  CHECK(pma.num_edges() == 12);
  std::vector<std::tuple<uint32_t, uint32_t>> batch = {{1, 2}, {2, 1}, {0, 6}, {6, 0}, {1, 2}};
  pma.insert_batch(batch.data(), batch.size());
  CHECK(pma.num_edges() == 16);
  CHECK(pma.degree(1) == 2 && pma.degree(6) == 2);
  par = byo::gpu_bfs(pma, 0);
  CHECK((par == std::vector<uint32_t>{0, 0, 1, 2, 5, 6, 0}));
  std::vector<std::tuple<uint32_t, uint32_t>> sorted = {{0, 6}, {6, 0}};
  pma.remove_sorted_batch(sorted.data(), sorted.size());
  CHECK(pma.num_edges() == 14 && pma.degree(6) == 1);
  lab = byo::gpu_cc(pma);
  CHECK((lab == std::vector<uint32_t>{0, 0, 0, 0, 0, 0, 0}));

  // the vector-of-sets container answers the same calls
  byo::GPU_VOS_graph<int> vos(vd.data(), n, edges.size(), nullptr, edges.data());
  CHECK(vos.num_edges() == 12);
  vos.insert_batch(batch.data(), batch.size());
  CHECK(vos.num_edges() == 16 && vos.degree(1) == 2 && vos.degree(6) == 2);
  CHECK((byo::gpu_bfs(vos, 0) == std::vector<uint32_t>{0, 0, 1, 2, 5, 6, 0}));
  vos.remove_sorted_batch(sorted.data(), sorted.size());
  CHECK(vos.num_edges() == 14 && vos.degree(6) == 1);
  CHECK((vos.offsets() == pma.offsets()) && (vos.edges() == pma.edges()));
  // the packed CSR: the same calls, its own layout
  byo::GPU_PCSR_graph<int> pcsr(vd.data(), n, edges.size(), nullptr, edges.data());
  CHECK(pcsr.num_edges() == 12);
  pcsr.insert_batch(batch.data(), batch.size());
  CHECK(pcsr.num_edges() == 16 && pcsr.degree(1) == 2 && pcsr.degree(6) == 2);
  CHECK((byo::gpu_bfs(pcsr, 0) == std::vector<uint32_t>{0, 0, 1, 2, 5, 6, 0}));
  {
    std::vector<uint32_t> nb6;
    pcsr.map_neighbors(6, [&](size_t, uint32_t v, auto) { nb6.push_back(v); });
    CHECK((nb6 == std::vector<uint32_t>{0, 5}));
  }
  pcsr.remove_sorted_batch(sorted.data(), sorted.size());
  CHECK(pcsr.num_edges() == 14 && pcsr.degree(6) == 1);
  CHECK((pcsr.offsets() == pma.offsets()) && (pcsr.edges() == pma.edges()));
  CHECK((byo::gpu_cc(pcsr) == std::vector<uint32_t>{0, 0, 0, 0, 0, 0, 0}));

  // the reference's own edgeMap loops through the adapter: bfs_cc::CC with
  // BFS_ComponentLabel_F (BFSCC/Connectivity.h:52-88) and PageRank_edgeMap
  // (PageRank.h:80-123), on the CSR of test_bfs.cc's graph
  {
    byo::DeviceVector<uint32_t> parents(n, BYO_NONE);
    std::vector<uint32_t> host(n, BYO_NONE);
    for (uint32_t i = 0; i < n; i++) {
      if (host[i] != BYO_NONE || csr.degree(i) == 0) continue;
      host[i] = i;
      parents.assign(host);
      byo::vertexSubset F(csr, i);
      byo::BFS_ComponentLabel_F f(csr, parents, i);
      while (!F.isEmpty()) F = byo::edgeMap(csr, F, f, -1, BYO_FL_SPARSE_BLOCKED | BYO_FL_DENSE_PARALLEL);
      host = parents.to_host();
    }
    CHECK((host == std::vector<uint32_t>{0, 0, 2, 2, 2, 2, 2}));
    byo::DeviceVector<double> pc(n, 1.0 / n), pn(n, 0.0);
    byo::vertexSubset all = byo::vertexSubset::all(csr);
    CHECK(all.size() == n && all.isDense());
    for (int it = 0; it < 200; it++) {
      byo::PR_F f(csr, pc, pn);
      byo::vertexSubset none = byo::edgeMap(csr, all, f, 0, BYO_FL_NO_OUTPUT);
      CHECK(none.isEmpty());
      byo::vertexMap(all, byo_vertex_op{BYO_VOP_PR_UPDATE, pn.data(), nullptr, nullptr, 0.85, 0.0});
      std::vector<double> a = pc.to_host(), b = pn.to_host();
      double l1 = 0;
      for (size_t v = 0; v < n; v++) l1 += a[v] > b[v] ? a[v] - b[v] : b[v] - a[v];
      if (l1 < 1e-9) break;
      byo::vertexMap(all, byo_vertex_op{BYO_VOP_ZERO, pc.data(), nullptr, nullptr, 0.0, 0.0});
      pc.swap(pn);
    }
    std::vector<double> got = pn.to_host();
    double diff = 0;
    for (size_t v = 0; v < n; v++) diff += got[v] > pr[v] ? got[v] - pr[v] : pr[v] - got[v];
    CHECK(diff < 1e-8);
  }
  std::printf("adapter ok\n");
  return 0;
}

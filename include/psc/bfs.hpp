// psc/bfs.hpp — drop-in for the reference's src/bfs.hpp (class BFS,
// src/bfs.hpp:18-57), running on a GB300.
//
//   BFS(Graph&)                                uploads the graph once
//   size_t bfs(NodeId src, sequence<NodeId>& dst)    bfs.hpp:200-238
//   void bfs_seq(NodeId src, sequence<NodeId>& dst)  bfs.hpp:59-76
//   size_t num_round
// dst[v] = hop distance from src along out-edges, UINT_N_MAX if unreached.
// Link with -lpsc_cuda -lpsc_host.
#pragma once
#include "device_graph.hpp"

class BFS {
 private:
  Graph& graph;
  psc_graph_t h = nullptr;

 public:
  size_t num_round = 0;
  BFS() = delete;
  explicit BFS(Graph& G) : graph(G) { h = psc_detail::upload(graph); }
  BFS(const BFS&) = delete;
  BFS& operator=(const BFS&) = delete;
  ~BFS() { psc_graph_free(h); }

  size_t bfs(NodeId source, psc::sequence<NodeId>& dst) {
    if (dst.size() < graph.n) dst = psc::sequence<NodeId>(graph.n);
    uint32_t r = 0;
    psc_detail::check(psc_bfs(h, source, dst.data(), &r), "psc_bfs");
    num_round = r;
    return r;
  }
  // The sequential BFS of the reference gives the same distances.
  void bfs_seq(NodeId source, psc::sequence<NodeId>& dst) { bfs(source, dst); }
};

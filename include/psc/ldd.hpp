// psc/ldd.hpp — drop-in for the reference's src/ldd.hpp (class LDD,
// src/ldd.hpp:38-56), running on a GB300.
//
//   LDD(const Graph&, pred = all edges)
//   tuple<sequence<NodeId>, sequence<NodeId>> ldd(double beta, bool spanning_tree)
//                                              ldd.hpp:325-417
//   size_t num_round
// label[v] = centre of v's cluster; parent (only with spanning_tree) = BFS
// parent inside the cluster, parent[v] = v for centres.  The graph must be
// symmetric.  A predicate other than the default keeps only the edges (u, v)
// with pred(u, v); they are selected on the host before the upload.
// Link with -lpsc_cuda -lpsc_host.
#pragma once
#include <functional>
#include <tuple>

#include "device_graph.hpp"

namespace psc_detail {

// Edges (u, v) of g with pred(u, v), as a new CSR graph (transpose = itself).
inline Graph filter_edges(const Graph& g, const std::function<bool(NodeId, NodeId)>& pred) {
  Graph f;
  f.n = g.n;
  f.symmetric = true;
  f.offset = psc::sequence<EdgeId>(g.n + 1, 0);
  psc::sequence<NodeId> tmp(g.m);
  size_t k = 0;
  for (size_t u = 0; u < g.n; u++) {
    f.offset[u] = k;
    for (EdgeId j = g.offset[u]; j < g.offset[u + 1]; j++)
      if (pred((NodeId)u, g.E[j])) tmp[k++] = g.E[j];
  }
  f.offset[g.n] = k;
  f.m = k;
  f.E = psc::sequence<NodeId>(k);
  for (size_t j = 0; j < k; j++) f.E[j] = tmp[j];
  f.in_offset = f.offset;
  f.in_E = f.E;
  return f;
}

}  // namespace psc_detail

class LDD {
 private:
  psc_graph_t h = nullptr;
  size_t n = 0;

 public:
  size_t num_round = 0;
  LDD() = delete;
  explicit LDD(const Graph& G) : n(G.n) { h = upload_sym(G); }
  LDD(const Graph& G, std::function<bool(NodeId, NodeId)> pred) : n(G.n) {
    Graph f = psc_detail::filter_edges(G, pred);
    h = upload_sym(f);
  }
  LDD(const LDD&) = delete;
  LDD& operator=(const LDD&) = delete;
  ~LDD() { psc_graph_free(h); }

  std::tuple<psc::sequence<NodeId>, psc::sequence<NodeId>> ldd(double beta,
                                                               bool spanning_tree = false) {
    psc::sequence<NodeId> label(n), parent;
    if (spanning_tree) parent = psc::sequence<NodeId>(n);
    psc_detail::check(psc_ldd(h, beta, label.data(), spanning_tree ? parent.data() : nullptr),
                      "psc_ldd");
    psc_stats_t st;
    psc_last_stats(h, &st);
    num_round = st.reach_rounds;
    return {std::move(label), std::move(parent)};
  }

 private:
  static psc_graph_t upload_sym(const Graph& g) {
    psc_graph_t hh = nullptr;
    psc_detail::check(psc_graph_upload(g.offset.data(), g.E.data(), nullptr, nullptr, g.n, g.m, &hh),
                      "psc_graph_upload");
    return hh;
  }
};

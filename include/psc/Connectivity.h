// psc/Connectivity.h — drop-in for the reference's src/Connectivity.h,
// running on a GB300.
//
//   tuple<sequence<NodeId>, sequence<pair<NodeId, NodeId>>>
//   Connectivity(const Graph& G, double beta,
//                function<bool(NodeId, NodeId)> pred = all edges,
//                bool spanning_forest = false)      Connectivity.h:37-119
// Returns each vertex's component root (a vertex id of the component) and,
// with spanning_forest, the tree edges.  The graph must be symmetric.  A
// predicate other than the default keeps only the edges (u, v) with
// pred(u, v); they are selected on the host before the upload.
// Link with -lpsc_cuda -lpsc_host.
#pragma once
#include <functional>
#include <tuple>
#include <utility>

#include "ldd.hpp"

namespace psc_detail {

inline std::tuple<psc::sequence<NodeId>, psc::sequence<std::pair<NodeId, NodeId>>> connectivity(
    const Graph& G, double beta, bool spanning_forest) {
  psc_graph_t h = nullptr;
  check(psc_graph_upload(G.offset.data(), G.E.data(), nullptr, nullptr, G.n, G.m, &h),
        "psc_graph_upload");
  psc::sequence<NodeId> label(G.n);
  psc::sequence<std::pair<NodeId, NodeId>> edges;
  if (spanning_forest) {
    psc::sequence<NodeId> f(2 * (G.n ? G.n : 1));
    uint64_t k = 0;
    check(psc_cc(h, beta, label.data(), f.data(), &k), "psc_cc");
    edges = psc::sequence<std::pair<NodeId, NodeId>>(k);
    for (uint64_t i = 0; i < k; i++) edges[i] = {f[2 * i], f[2 * i + 1]};
  } else {
    check(psc_cc(h, beta, label.data(), nullptr, nullptr), "psc_cc");
  }
  psc_graph_free(h);
  return {std::move(label), std::move(edges)};
}

}  // namespace psc_detail

inline std::tuple<psc::sequence<NodeId>, psc::sequence<std::pair<NodeId, NodeId>>> Connectivity(
    const Graph& G, double beta) {
  return psc_detail::connectivity(G, beta, false);
}

inline std::tuple<psc::sequence<NodeId>, psc::sequence<std::pair<NodeId, NodeId>>> Connectivity(
    const Graph& G, double beta, std::function<bool(NodeId, NodeId)> pred,
    bool spanning_forest = false) {
  Graph f = psc_detail::filter_edges(G, pred);
  return psc_detail::connectivity(f, beta, spanning_forest);
}

// psc/reach.hpp — drop-in for the reference's src/reach.hpp (class REACH,
// src/reach.hpp:21-55), running on a GB300.
//
//   REACH(Graph&)                       uploads the graph once
//   int reach(src, sequence<bool>& dst, bool local)   reach.hpp:208-243
//   void reach_seq(src, sequence<bool>& dst)          reach.hpp:57-74
//   void swap_graph()                   reach.hpp:51-54: swaps the caller's
//                                       E/in_E and offset/in_offset, and later
//                                       searches follow the swapped direction
// `tau` is the global of psc/scc.hpp.  Link with -lpsc_cuda -lpsc_host.
#pragma once
#include <utility>

#include "device_graph.hpp"
#include "scc.hpp"

class REACH {
 private:
  Graph& graph;
  psc_graph_t h = nullptr;
  bool swapped = false;

 public:
  size_t num_round = 0;
  REACH() = delete;
  explicit REACH(Graph& G) : graph(G) {
    // the device copy is uploaded in the unswapped orientation
    h = psc_detail::upload(graph);
  }
  REACH(const REACH&) = delete;
  REACH& operator=(const REACH&) = delete;
  ~REACH() { psc_graph_free(h); }

  int reach(NodeId source, psc::sequence<bool>& dst, bool local) {
    if (dst.size() < graph.n) dst = psc::sequence<bool>(graph.n);
    uint32_t r = 0;
    static_assert(sizeof(bool) == 1, "bool flags are bytes");
    psc_detail::check(psc_reach(h, source, swapped ? 1 : 0, local ? 1 : 0, (uint32_t)tau,
                                reinterpret_cast<uint8_t*>(dst.data()), &r),
                      "psc_reach");
    num_round = r;
    return (int)r;
  }

  void reach_seq(NodeId source, psc::sequence<bool>& dst) { reach(source, dst, false); }

  void swap_graph() {
    std::swap(graph.in_E, graph.E);
    std::swap(graph.in_offset, graph.offset);
    swapped = !swapped;
  }
};

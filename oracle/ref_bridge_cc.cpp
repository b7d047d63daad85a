// C entry points over the reference's own connectivity code (src/Connectivity.h,
// src/ldd.hpp, src/union_find_rules.h), compiled unmodified against the
// ParlayLib-API stand-in in oracle/ref_shim/.  Built by oracle/ref.mk into
// oracle/_ref/libref_cc.so.
//
// TEST INFRASTRUCTURE ONLY (tests and the fixture generator); the product
// never loads it.
#include "Connectivity.h"

#include "ref_bridge_common.hpp"

extern "C" {

// Connectivity(G, beta) (src/Connectivity.h:37-119) on a symmetric graph;
// labels_out[v] = the reference's component label of v.  With forest_out
// non-null the spanning forest's edges are written there (n entries of two
// u32) and their number returned.
int64_t ref_cc(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E, double beta,
               uint32_t* labels_out, uint32_t* forest_out) {
  if (n == 0) return 0;
  Graph g = ref_graph(n, m, off, E, off, E);
  sequence<NodeId> label;
  sequence<pair<NodeId, NodeId>> forest;
  tie(label, forest) = Connectivity(g, beta, [](NodeId, NodeId) { return true; },
                                    forest_out != nullptr);
  for (uint64_t i = 0; i < n; i++) labels_out[i] = label[i];
  if (forest_out) {
    for (size_t i = 0; i < forest.size(); i++) {
      forest_out[2 * i] = forest[i].first;
      forest_out[2 * i + 1] = forest[i].second;
    }
  }
  return (int64_t)forest.size();
}

// LDD::ldd (src/ldd.hpp:325-417): cluster labels (centre ids); returns the
// number of rounds.
int64_t ref_ldd(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E, double beta,
                uint32_t* labels_out, uint32_t* parent_out) {
  if (n == 0) return 0;
  Graph g = ref_graph(n, m, off, E, off, E);
  LDD l(g);
  sequence<NodeId> label, parent;
  tie(label, parent) = l.ldd(beta, parent_out != nullptr);
  for (uint64_t i = 0; i < n; i++) labels_out[i] = label[i];
  if (parent_out)
    for (uint64_t i = 0; i < n; i++) parent_out[i] = parent[i];
  return (int64_t)l.num_round;
}

}  // extern "C"

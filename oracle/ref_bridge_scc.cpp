// C entry points over the reference's own SCC, REACH, BFS, graph-building and
// Tarjan code (src/scc.hpp, src/reach.hpp, src/bfs.hpp, src/graph.hpp,
// baselines/tarjan_scc/tarjan_scc.hpp), compiled unmodified against the
// ParlayLib-API stand-in in oracle/ref_shim/.  Built by oracle/ref.mk into
// oracle/_ref/libref_scc.so.
//
// TEST INFRASTRUCTURE ONLY: used by the tests and by the fixture generator
// tests/golden/make_ref_golden.py to pin the C oracle and the CUDA library to
// the reference's code.  The product never loads it.
#include "scc.hpp"
#include "bfs.hpp"
#include "tarjan_scc.hpp"

#include "ref_bridge_common.hpp"

extern "C" {

// SCC::scc (src/scc.hpp:277-476) with the CLI's globals set first
// (src/scc.cpp:45-46); labels_out[v] = the reference's raw label of v.
int ref_scc(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E, const uint64_t* in_off,
            const uint32_t* in_E, double beta, uint64_t tau_, uint64_t lambda, int local_reach,
            int local_scc, uint64_t seed, uint64_t* labels_out) {
  if (n == 0) return 0;
  Graph g = ref_graph(n, m, off, E, in_off, in_E);
  parlay::shim_seed() = seed;
  tau = tau_;
  _min_bag_size_ = lambda;
  sequence<size_t> labels(n);
  SCC s(g);
  s.scc(labels, beta, local_reach != 0, local_scc != 0);
  for (uint64_t i = 0; i < n; i++) labels_out[i] = labels[i];
  return 0;
}

// REACH::reach from src over the graph (forward) or its transpose
// (src/reach.hpp:208-243, swap_graph :51-54).
int ref_reach(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E, const uint64_t* in_off,
              const uint32_t* in_E, uint32_t src, int forward, uint64_t tau_, int local,
              uint8_t* out) {
  Graph g = ref_graph(n, m, off, E, in_off, in_E);
  tau = tau_;
  sequence<bool> dst(n);
  REACH r(g);
  if (!forward) r.swap_graph();
  r.reach(src, dst, local != 0);
  for (uint64_t i = 0; i < n; i++) out[i] = dst[i] ? 1 : 0;
  return (int)r.num_round;
}

// BFS::bfs distances from src (src/bfs.hpp:200-238).
int ref_bfs(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E, uint32_t src,
            uint32_t* dist_out) {
  Graph g = ref_graph(n, m, off, E, off, E);
  sequence<NodeId> dst(n);
  BFS b(g);
  b.bfs(src, dst);
  for (uint64_t i = 0; i < n; i++) dist_out[i] = dst[i];
  return (int)b.num_round;
}

// make_directed (src/graph.hpp:222-245): the transpose CSR.
int ref_make_directed(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E,
                      uint64_t* in_off_out, uint32_t* in_E_out) {
  Graph g = ref_graph(n, m, off, E, nullptr, nullptr);
  make_directed(g);
  for (uint64_t i = 0; i <= n; i++) in_off_out[i] = g.in_offset[i];
  for (uint64_t i = 0; i < m; i++) in_E_out[i] = g.in_E[i];
  return 0;
}

// make_symmetric (src/graph.hpp:187-220): both directions, duplicates and
// self-loops dropped.  E_out holds at least 2m entries; returns the new m.
int64_t ref_make_symmetric(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E,
                           uint64_t* off_out, uint32_t* E_out) {
  Graph g = ref_graph(n, m, off, E, nullptr, nullptr);
  make_symmetric(g);
  for (uint64_t i = 0; i <= n; i++) off_out[i] = g.offset[i];
  for (uint64_t i = 0; i < g.m; i++) E_out[i] = g.E[i];
  return (int64_t)g.m;
}

// TARJAN_SCC::tarjan (baselines/tarjan_scc/tarjan_scc.hpp:39-76): component
// ids 1..k in completion order; returns k.
int64_t ref_tarjan(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E,
                   uint32_t* comp_out) {
  Graph g = ref_graph(n, m, off, E, off, E);
  TARJAN_SCC t(g);
  t.clear();
  t.tarjan();
  uint32_t k = 0;
  for (uint64_t i = 0; i < n; i++) {
    comp_out[i] = t.scc[i];
    k = std::max<uint32_t>(k, t.scc[i]);
  }
  return k;
}

}  // extern "C"

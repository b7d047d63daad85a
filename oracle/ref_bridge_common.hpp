// Shared helpers of the reference bridges (test infrastructure only); each
// bridge is its own shared library and includes this file once.
#pragma once
#include <omp.h>
#include <stdint.h>

// A reference Graph (src/graph.hpp:35-43) holding copies of the caller's CSR
// and, when given, its transpose.
inline Graph ref_graph(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E,
                       const uint64_t* in_off, const uint32_t* in_E) {
  Graph g;
  g.n = n;
  g.m = m;
  g.symmetric = (in_off == off && in_E == E);
  g.offset = sequence<EdgeId>(n + 1);
  g.E = sequence<NodeId>(m);
  for (uint64_t i = 0; i <= n; i++) g.offset[i] = off[i];
  for (uint64_t i = 0; i < m; i++) g.E[i] = E[i];
  if (in_off) {
    g.in_offset = sequence<EdgeId>(n + 1);
    g.in_E = sequence<NodeId>(m);
    for (uint64_t i = 0; i <= n; i++) g.in_offset[i] = in_off[i];
    for (uint64_t i = 0; i < m; i++) g.in_E[i] = in_E[i];
  }
  return g;
}

extern "C" void ref_set_threads(int t) {
  if (t > 0) omp_set_num_threads(t);
}

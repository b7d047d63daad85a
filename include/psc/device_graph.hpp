// psc/device_graph.hpp — internal helper of the drop-in headers: owns the
// device copy (psc_graph_t) of a caller's Graph, as the reference's algorithm
// objects hold the caller's Graph by reference (src/scc.hpp:40,
// src/reach.hpp:23).  Errors print and abort(), matching the reference, which
// has no error returns.
#pragma once
#include <cstdio>
#include <cstdlib>

#include "../psc.h"
#include "graph.hpp"

namespace psc_detail {

inline void check(int st, const char* what) {
  if (st != PSC_OK) {
    std::fprintf(stderr, "Error: %s: %s\n", what, psc_strerror(st));
    std::abort();
  }
}

inline psc_graph_t upload(const Graph& g) {
  psc_graph_t h = nullptr;
  const bool sym = g.symmetric || g.in_offset.size() == 0;
  check(psc_graph_upload(g.offset.data(), g.E.data(), sym ? nullptr : g.in_offset.data(),
                         sym ? nullptr : g.in_E.data(), g.n, g.m, &h),
        "psc_graph_upload");
  return h;
}

}  // namespace psc_detail

// Host entry points of the device engines, shared between translation units.
#pragma once
#include "common.cuh"

namespace psc {

int ensure_keep(psc_graph_s* g, int b, size_t bytes, size_t keep, void** out);
int call_begin(psc_graph_s* g);
int call_end(psc_graph_s* g);

// Builds in_off/in_E from off/E on the device (in-lists sorted by source).
int build_transpose(psc_graph_s* g);

// Single-source reachability into the bitmap vis (u32[ceil(n/32)], cleared
// here).  backward = expand over the transpose.  rounds receives the number
// of frontier rounds.
int reach_run(psc_graph_s* g, uint32_t src, bool backward, bool local, uint32_t tau,
              uint32_t pull_div, uint32_t* vis, uint32_t* rounds);

// Forward and backward reachability from one source, run together.
int reach_pair(psc_graph_s* g, uint32_t src, bool local, uint32_t tau, uint32_t pull_div,
               uint32_t* vis_f, uint32_t* vis_b, uint32_t* rounds_f, uint32_t* rounds_b);

// Multi-search (SCC::multi_search, src/scc.hpp:144-275) of one batch in both
// directions at once: closure of the pivots front[i] (labels label_offset + i)
// inside their subproblems, left in table slots B_TF (forward) and B_TB
// (backward).  prev_ne: table sizes of the previous batch (sizing hint).
struct MsResult {
  uint64_t cap = 0;  // table capacity (power of two)
  uint64_t ne = 0;   // entries
};
int ms_pair(psc_graph_s* g, const uint32_t* front, uint64_t n_front, uint64_t label_offset,
            const uint64_t* labels, const psc_params_t* p, const uint64_t prev_ne[2],
            MsResult out[2]);

// SCC into device labels (u64[n]).
int scc_run(psc_graph_s* g, const psc_params_t* p, uint64_t* d_labels);

}  // namespace psc

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

// SCC into device labels (u64[n]).
int scc_run(psc_graph_s* g, const psc_params_t* p, uint64_t* d_labels);

}  // namespace psc

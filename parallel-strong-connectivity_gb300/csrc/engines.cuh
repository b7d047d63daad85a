// Host entry points of the device engines, shared between translation units.
#pragma once
#include "common.cuh"

namespace psc {

int ensure_keep(psc_graph_s* g, int b, size_t bytes, size_t keep, void** out);
// A handle with its stream, counters and events for a graph of n vertices
// and m edges, and its graph arrays from the stream-ordered pool
// (in_off/in_E alias off/E when symmetric).
// priority: of the handle's stream (0 = default; lower numbers run first)
int make_handle(uint64_t n, uint64_t m, psc_graph_s** out, int priority = 0);
int alloc_graph_arrays(psc_graph_s* g, bool symmetric);
// Attaches a graph-offset table (vertex bases, host u64[G+1]) to g: the
// per-vertex graph ids and, when check is set, the test that no edge crosses
// two graphs.
int batch_attach(psc_graph_s* g, const uint64_t* vbase, uint32_t num_graphs, bool check);
int call_begin(psc_graph_s* g);
int call_end(psc_graph_s* g);

// g->max_deg (largest out- / in-degree), computed once per handle.
int ensure_max_degrees(psc_graph_s* g);

// Builds in_off/in_E from off/E on the device (in-lists sorted by source).
int build_transpose(psc_graph_s* g);
// Replaces off/E by their symmetrisation on the device (both directions,
// lists sorted, duplicates and self-loops dropped; g->m becomes the new edge
// count) and makes g symmetric.
int build_symmetric(psc_graph_s* g);

// Single-source reachability into the bitmap vis (u32[ceil(n/32)], cleared
// here).  backward = expand over the transpose.  rounds receives the number
// of frontier rounds.
int reach_run(psc_graph_s* g, uint32_t src, bool backward, bool local, uint32_t tau,
              uint32_t pull_div, uint32_t* vis, uint32_t* rounds);

// Forward and backward reachability from one source, run together.
int reach_pair(psc_graph_s* g, uint32_t src, bool local, uint32_t tau, uint32_t pull_div,
               uint32_t* vis_f, uint32_t* vis_b, uint32_t* rounds_f, uint32_t* rounds_b);

// Forward and backward reachability from n_srcs device sources at once (the
// first pivots of a batch of disjoint graphs share one search).  vgc_max:
// largest frontier expanded by VGC rounds (0: one vertex per resident warp).
int reach_pair_multi(psc_graph_s* g, const uint32_t* d_srcs, uint64_t n_srcs, bool local,
                     uint32_t tau, uint32_t pull_div, uint32_t* vis_f, uint32_t* vis_b,
                     uint32_t* rounds_f, uint32_t* rounds_b, uint64_t vgc_max = 0);

// Multi-search (SCC::multi_search, src/scc.hpp:144-275) of one batch in both
// directions at once: closure of the pivots front[i] (labels label_offset + i)
// inside their subproblems, left in table slots B_TF (forward) and B_TB
// (backward).  prev_ne: table sizes of the previous batch (sizing hint).
// front_labels, when given, holds each pivot's label instead of
// label_offset + i.  vgc_max: largest pair frontier expanded by VGC
// sub-rounds (0: one pair per resident warp).
struct MsResult {
  uint64_t cap = 0;  // table capacity (power of two)
  uint64_t ne = 0;   // entries
};
// Asynchronous start of a batch (MsAsync given): the pivot count is read on
// the device at *nf_dev (n_front is only its upper bound), so the seeds and
// the first sub-round are launched without waiting for the compaction that
// wrote front.  On return n_front holds the pivot count.  (The partition
// cannot start early: later sub-rounds test subproblems on the labels it
// writes.)
struct MsAsync {
  const unsigned long long* nf_dev = nullptr;
  uint64_t n_front = 0;
};
int ms_pair(psc_graph_s* g, const uint32_t* front, uint64_t n_front, uint64_t label_offset,
            const uint64_t* labels, const psc_params_t* p, const uint64_t prev_ne[2],
            MsResult out[2], const uint32_t* front_labels = nullptr, uint64_t vgc_max = 0,
            MsAsync* async = nullptr);

// Partition of one batch (src/scc.hpp:437-464): (v, l) in both tables left by
// ms_pair -> labels[v] = max(l | TOP), else max(l).
int scc_partition(psc_graph_s* g, const MsResult res[2], uint64_t* labels);

// Runs phases(g) between the SCC phase events and fills stats.phase_ms
// (trim, first pivot, multi-search, table growth).  phases records ph[1] and
// ph[2] itself.
template <class Phases>
int scc_timed(psc_graph_s* g, Phases phases);
int scc_phase_times(psc_graph_s* g);
void scc_clear_grow_events(psc_graph_s* g);

template <class Phases>
int scc_timed(psc_graph_s* g, Phases phases) {
  scc_clear_grow_events(g);
  PSC_CUDA(cudaEventRecord(g->ph[0], g->stream));
  PSC_TRY(phases(g));
  return scc_phase_times(g);
}

// SCC into device labels (u64[n]).
int scc_run(psc_graph_s* g, const psc_params_t* p, uint64_t* d_labels);

// SCC of every graph of a batch (graph-offset table set by psc_batch_set)
// into device labels u64[n] holding each graph's own labels (vertex ids local
// to the graph); seeds: per-graph pivot-order seeds (null: p->seed for all).
int scc_batch_run(psc_graph_s* g, const psc_params_t* p, const uint64_t* seeds, uint64_t* d_labels);

// Connectivity labels u32[n] of the union (cc.cu).
int cc_run(psc_graph_s* g, double beta, uint32_t* d_label, uint32_t* d_forest, uint64_t* n_forest);

// Connectivity of every graph of a batch: component roots local to each graph.
int cc_batch_run(psc_graph_s* g, double beta, uint32_t* d_labels);

}  // namespace psc

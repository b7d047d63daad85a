// Autotuner of the SCC parameters on the caller's own graph or batch.  No
// counterpart in the reference, whose knobs are command-line flags
// (src/scc.cpp:40-55, `-tau`, `-beta`).
//
// Coordinate descent over the knobs in the order that matters most for the
// round structure: tau (VGC local-search budget), the push/pull threshold
// (pull when frontier edges exceed m / pull_div), the block size of the
// expansion kernels, then beta (prefix-doubling growth).  Each candidate is
// timed `reps` times with CUDA events around the whole solve (best kept) and
// replaces the current setting only if it is at least 2 % faster.
// tau, pull_div and block never change the labels; beta changes the label
// values (the batch schedule) but never the partition.
#include <cfloat>

#include "common.cuh"
#include "engines.cuh"

namespace psc {
namespace {

const uint32_t kTaus[] = {32, 64, 128, 256, 512};
const uint32_t kPullDivs[] = {5, 10, 20, 40, 80};
const uint32_t kBlocks[] = {128, 256, 512};
const double kBetas[] = {1.5, 2.0, 3.0, 4.0};

}  // namespace
}  // namespace psc

using namespace psc;

extern "C" int psc_tune_scc(psc_graph_t g, const uint64_t* seeds, uint32_t reps, psc_params_t* p,
                            psc_tune_report_t* report) {
  if (!g || !p || !(p->beta > 0)) return PSC_ERR_INVALID;
  if (reps == 0) reps = 2;
  PSC_CUDA(cudaSetDevice(g->device));
  uint64_t* d;
  PSC_TRY(ensure_t(g, B_LABELS, g->n, &d));
  uint32_t trials = 0;
  auto time_one = [&](const psc_params_t& q, double* ms) -> int {
    double best = DBL_MAX;
    for (uint32_t r = 0; r < reps; r++) {
      PSC_TRY(call_begin(g));
      PSC_TRY(g->num_graphs ? scc_batch_run(g, &q, seeds, d) : scc_run(g, &q, d));
      PSC_TRY(call_end(g));
      best = std::min(best, g->stats.total_ms);
    }
    trials++;
    *ms = best;
    return PSC_OK;
  };
  psc_params_t cur = *p;
  if (cur.tau == 0) cur.tau = 512;
  if (cur.pull_div == 0) cur.pull_div = 20;
  if (cur.block == 0) cur.block = 256;
  double cur_ms = 0;
  PSC_TRY(time_one(cur, &cur_ms));
  const double start_ms = cur_ms;
  auto try_knob = [&](auto set, const auto& cands) -> int {
    psc_params_t best = cur;
    double best_ms = cur_ms;
    for (const auto c : cands) {
      psc_params_t q = cur;
      if (!set(q, c)) continue;  // the current value
      double ms = 0;
      PSC_TRY(time_one(q, &ms));
      if (ms < best_ms * 0.98) {
        best = q;
        best_ms = ms;
      }
    }
    cur = best;
    cur_ms = best_ms;
    return PSC_OK;
  };
  PSC_TRY(try_knob([&](psc_params_t& q, uint32_t v) { return q.tau != v ? (q.tau = v, true) : false; },
                   kTaus));
  PSC_TRY(try_knob(
      [&](psc_params_t& q, uint32_t v) { return q.pull_div != v ? (q.pull_div = v, true) : false; },
      kPullDivs));
  PSC_TRY(try_knob(
      [&](psc_params_t& q, uint32_t v) { return q.block != v ? (q.block = v, true) : false; },
      kBlocks));
  PSC_TRY(try_knob([&](psc_params_t& q, double v) { return q.beta != v ? (q.beta = v, true) : false; },
                   kBetas));
  *p = cur;
  if (report) {
    report->start_ms = start_ms;
    report->best_ms = cur_ms;
    report->trials = trials;
  }
  return PSC_OK;
}

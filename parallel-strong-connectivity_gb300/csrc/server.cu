// Request server: SCC and connectivity solves of many independent graphs
// served with continuous batching under a device-memory budget.  No
// counterpart in the reference, whose drivers solve one graph per process
// (src/scc.cpp:57-67, src/Connectivity.cpp:28-33).
//
// Requests wait in one FIFO queue.  Each of `workers` threads owns a CUDA
// stream; whenever it is free it admits, in arrival order, the queued
// requests of the kind at the head of the queue while their estimated device
// footprint fits the budget left by the batches still running, packs them
// into one disjoint-union graph on the device (the members' CSR arrays are
// copied into slices and rebased by one kernel; the transpose of an SCC batch
// is built on the device), solves the batch with the lockstep batched
// SCC / connectivity path, copies every member's labels to its caller and
// releases the memory.  Requests that arrive while batches are running are
// admitted as soon as a worker and enough budget are free, so their work
// overlaps the running batches on the device.
//
// A batch of few edges (up to kUrgentEdges) runs on a high-priority stream: its
// solve is a chain of small, latency-bound rounds that would otherwise wait
// behind the wide kernels of the large batches running beside it.
//
// A request's result does not depend on the batch it lands in: SCC labels
// equal psc_scc on the graph alone with the request's seed, connectivity
// labels give the same partition as psc_cc on the graph alone.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "engines.cuh"

namespace psc {
namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t id = 0;
  int kind = PSC_REQ_SCC;
  uint64_t n = 0, m = 0;
  const uint64_t* off = nullptr;
  const uint32_t* E = nullptr;
  const uint64_t* in_off = nullptr;  // transpose of an SCC request (optional)
  const uint32_t* in_E = nullptr;
  uint64_t seed = 0;
  void* out = nullptr;
  uint64_t bytes = 0;
  Clock::time_point t_submit, t_start, t_done;
  bool done = false;
  int status = PSC_OK;
  uint32_t batch_size = 0;
};

// Device bytes a request may need while its batch runs: graph arrays (and for
// SCC the transpose, plus its build scratch when it is not sent along),
// labels and the solver's scratch (pivot order, queues, bitmaps, label
// tables) per vertex.
uint64_t request_bytes(int kind, uint64_t n, uint64_t m, bool with_t) {
  if (kind == PSC_REQ_SCC) return 16 * (n + 1) + (with_t ? 8 : 22) * m + 168 * n;
  return 8 * (n + 1) + 4 * m + 64 * n;
}

// Adds the batch's vertex / edge bases to the packed arrays (one request's
// slice each: offsets get its edge base, targets its vertex base).

__global__ void k_rebase(uint64_t* off, uint64_t n, uint32_t* E, uint64_t m,
                         const uint64_t* __restrict__ vbase, const uint64_t* __restrict__ ebase,
                         uint32_t R) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n + m;
       i += (uint64_t)gridDim.x * blockDim.x) {
    if (i < n) {
      off[i] += ebase[last_le(vbase, R, i)];
    } else {
      const uint64_t j = i - n;
      E[j] += (uint32_t)vbase[last_le(ebase, R, j)];
    }
  }
}

// Before the rebase: every request's own offsets run from 0 to its edge count
// without decreasing and its targets are its vertex ids.  Only the packed
// arrays are read (no access is indexed by their values).  A malformed item
// sets its request's flag (bad[r]) and the any-flag (*any), so that only the
// requests that hold one fail and the rest of the batch runs without them.
__global__ void k_validate_batch(const uint64_t* __restrict__ off, uint64_t n,
                                 const uint32_t* __restrict__ E, uint64_t m,
                                 const uint64_t* __restrict__ vbase,
                                 const uint64_t* __restrict__ ebase, uint32_t R,
                                 unsigned long long* bad, unsigned long long* any) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool b = false;
  for (uint64_t i = t; i < n; i += stride) {
    const uint32_t r = last_le(vbase, R, i);
    const uint64_t mr = ebase[r + 1] - ebase[r];
    const uint64_t o = off[i], o2 = i + 1 < vbase[r + 1] ? off[i + 1] : mr;
    if ((i == vbase[r] && o != 0) || o > o2 || o2 > mr) {
      atomicOr(&bad[r], 1ull);
      b = true;
    }
  }
  for (uint64_t j = t; j < m; j += stride) {
    const uint32_t r = last_le(ebase, R, j);
    if (E[j] >= vbase[r + 1] - vbase[r]) {
      atomicOr(&bad[r], 1ull);
      b = true;
    }
  }
  if (__any_sync(kFull, b) && lane_id() == 0) atomicOr(any, 1ull);
}

__global__ void k_put_u64(uint64_t* p, uint64_t v) { *p = v; }

}  // namespace
}  // namespace psc

struct psc_server_s {
  psc_server_config_t cfg{};
  int device = 0;
  std::mutex mu;
  std::condition_variable work_cv;  // queue or budget changed
  std::condition_variable done_cv;  // a request completed
  std::deque<psc::Request*> queue;
  std::unordered_map<uint64_t, psc::Request*> requests;
  std::vector<std::thread> workers;
  uint64_t next_id = 1;
  uint64_t used = 0;      // bytes admitted by running batches
  uint32_t running = 0;   // batches on the device
  int urgent_priority = 0;  // stream priority of small batches
  // Host-to-device copies of batches go in the order the batches were taken:
  // a batch waits for its ticket's turn, copies, then passes the turn on, so
  // the first batches reach the device at full link speed and solve while
  // later ones copy (instead of every batch sharing the link and finishing
  // its copy at the same late time).
  std::condition_variable upload_cv;
  uint64_t next_ticket = 0;
  uint64_t upload_turn = 0;
  // Solve slots: cfg.workers batches solve at a time; twice as many worker
  // threads run, so while every slot is busy the others copy their inputs
  // ahead (measured: with one thread per slot the link idled ~24 ms of a
  // 193 ms saturated stream, each time all workers were solving).
  std::condition_variable solve_cv;
  uint32_t solving = 0;
  bool stop = false;
  psc_server_stats_t stats{};
  std::chrono::steady_clock::time_point t_epoch = std::chrono::steady_clock::now();  // trace times
};

namespace psc {
namespace {

constexpr uint64_t kUrgentEdges = 1ull << 26;

// The upload turn of one batch: wait() blocks until the batch's ticket is
// served; the turn passes to the next ticket on release() or when the batch
// leaves run_batch without having released it.  The wait is bounded
// (kTurnWait): a batch whose turn does not come copies anyway (the order is a
// schedule, not a correctness condition) and then passes the turn on only if
// it is still its own, so no batch can block the others for good.
constexpr std::chrono::seconds kTurnWait{30};

struct UploadTurn {
  psc_server_s* S;
  uint64_t ticket;
  bool held = false, done = false;
  void wait() {
    std::unique_lock<std::mutex> lk(S->mu);
    S->upload_cv.wait_for(lk, kTurnWait, [&] { return S->upload_turn >= ticket; });
    held = true;
  }
  void release() {
    if (done) return;
    if (!held) wait();
    {
      std::lock_guard<std::mutex> lk(S->mu);
      if (S->upload_turn <= ticket) S->upload_turn = ticket + 1;
    }
    S->upload_cv.notify_all();
    done = true;
  }
  ~UploadTurn() { release(); }
};

// A solve slot, taken after the batch's copies and released when its labels
// are out.  The wait is bounded like the upload turn's: a batch that waited
// kTurnWait solves anyway.
struct SolveSlot {
  psc_server_s* S;
  bool held = false;
  void take() {
    std::unique_lock<std::mutex> lk(S->mu);
    S->solve_cv.wait_for(lk, kTurnWait, [&] { return S->solving < S->cfg.workers; });
    S->solving++;
    held = true;
  }
  ~SolveSlot() {
    if (!held) return;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->solving--;
    }
    S->solve_cv.notify_one();
  }
};

uint64_t take_ticket(psc_server_s* S) {
  std::lock_guard<std::mutex> lk(S->mu);
  return S->next_ticket++;
}

// Solves one batch of requests of the same kind on a fresh handle.  When the
// device check finds malformed requests, returns PSC_ERR_INVALID with
// bad[k] = 1 for each of them (and nothing solved); the caller runs the rest
// again without them.  ticket: the batch's place in the upload order.
int run_batch(psc_server_s* S, std::vector<Request*>& B, int kind, uint64_t ticket,
              uint64_t* launches, std::vector<char>* bad_out) {
  UploadTurn turn{S, ticket};
  SolveSlot slot{S};
  const uint32_t R = (uint32_t)B.size();
  std::vector<uint64_t> vbase(R + 1, 0), ebase(R + 1, 0);
  for (uint32_t k = 0; k < R; k++) {
    vbase[k + 1] = vbase[k] + B[k]->n;
    ebase[k + 1] = ebase[k] + B[k]->m;
  }
  const uint64_t n = vbase[R], m = ebase[R];
  if (n >= 0xFFFFFFFFull) return PSC_ERR_TOO_LARGE;
  const bool tr = trace_server_on();
  std::vector<std::pair<const char*, double>> marks;
  const auto t_begin = Clock::now();
  psc_graph_s* g = nullptr;
  PSC_TRY(make_handle(n, m, &g, m <= kUrgentEdges ? S->urgent_priority : 0));
  auto stamp = [&](const char* what) -> int {
    if (!tr) return PSC_OK;
    PSC_CUDA(cudaStreamSynchronize(g->stream));
    marks.emplace_back(what, std::chrono::duration<double, std::milli>(Clock::now() - t_begin).count());
    return PSC_OK;
  };
  auto body = [&]() -> int {
    PSC_TRY(stamp("handle"));
    PSC_TRY(alloc_graph_arrays(g, kind == PSC_REQ_CC));
    PSC_TRY(call_begin(g));
    PSC_TRY(stamp("alloc"));
    // every SCC request brought its transpose: copy it instead of building
    bool with_t = kind == PSC_REQ_SCC;
    for (uint32_t k = 0; k < R; k++) with_t = with_t && B[k]->in_off != nullptr;
    turn.wait();
    if (tr)  // host time the upload turn came (no stream wait)
      marks.emplace_back("turn", std::chrono::duration<double, std::milli>(Clock::now() - t_begin).count());
    for (uint32_t k = 0; k < R; k++) {
      PSC_CUDA(cudaMemcpyAsync(g->off + vbase[k], B[k]->off, B[k]->n * 8, cudaMemcpyDefault, g->stream));
      if (B[k]->m)
        PSC_CUDA(cudaMemcpyAsync(g->E + ebase[k], B[k]->E, B[k]->m * 4, cudaMemcpyDefault, g->stream));
      if (with_t) {
        PSC_CUDA(cudaMemcpyAsync(g->in_off + vbase[k], B[k]->in_off, B[k]->n * 8, cudaMemcpyDefault,
                                 g->stream));
        if (B[k]->m)
          PSC_CUDA(cudaMemcpyAsync(g->in_E + ebase[k], B[k]->in_E, B[k]->m * 4, cudaMemcpyDefault,
                                   g->stream));
      }
    }
    // bases: vbase[R+1], ebase[R+1], then one malformed-flag word per request
    uint64_t* bases;
    PSC_TRY(ensure_t(g, B_SCHED, 3 * (size_t)R + 2, &bases));
    std::vector<uint64_t> hb(3 * (size_t)R + 2, 0);
    std::copy(vbase.begin(), vbase.end(), hb.begin());
    std::copy(ebase.begin(), ebase.end(), hb.begin() + R + 1);
    PSC_CUDA(cudaMemcpyAsync(bases, hb.data(), hb.size() * 8, cudaMemcpyHostToDevice, g->stream));
    {
      unsigned long long* any = &g->ctr[2].aux0;  // staging set of the fresh handle
      unsigned long long* flags = (unsigned long long*)(bases + 2 * (size_t)R + 2);
      PSC_CUDA(cudaMemsetAsync(any, 0, sizeof(unsigned long long), g->stream));
      const unsigned vgrid = grid_for(g, std::max(n, m), 256);
      k_validate_batch<<<vgrid, 256, 0, g->stream>>>(g->off, n, g->E, m, bases, bases + R + 1, R,
                                                      flags, any);
      if (with_t)
        k_validate_batch<<<vgrid, 256, 0, g->stream>>>(g->in_off, n, g->in_E, m, bases,
                                                        bases + R + 1, R, flags, any);
      PSC_CUDA(cudaGetLastError());
      PSC_TRY(read_counters(g));  // the copies are done: the link is the next batch's
      turn.release();
      if (tr)
        marks.emplace_back("released",
                           std::chrono::duration<double, std::milli>(Clock::now() - t_begin).count());
      if (g->hctr[2].aux0) {
        std::vector<uint64_t> hf(R);
        PSC_CUDA(cudaMemcpyAsync(hf.data(), flags, R * 8, cudaMemcpyDeviceToHost, g->stream));
        PSC_CUDA(cudaStreamSynchronize(g->stream));
        bad_out->assign(R, 0);
        for (uint32_t k = 0; k < R; k++) (*bad_out)[k] = hf[k] != 0;
        return PSC_ERR_INVALID;
      }
    }
    k_rebase<<<grid_for(g, n + m, 256), 256, 0, g->stream>>>(g->off, n, g->E, m, bases, bases + R + 1,
                                                              R);
    k_put_u64<<<1, 1, 0, g->stream>>>(g->off + n, m);
    if (with_t) {
      k_rebase<<<grid_for(g, n + m, 256), 256, 0, g->stream>>>(g->in_off, n, g->in_E, m, bases,
                                                                bases + R + 1, R);
      k_put_u64<<<1, 1, 0, g->stream>>>(g->in_off + n, m);
    }
    PSC_CUDA(cudaGetLastError());
    PSC_TRY(stamp("upload"));
    slot.take();
    if (tr)
      marks.emplace_back("slot", std::chrono::duration<double, std::milli>(Clock::now() - t_begin).count());
    // SCC needs the in-edges: built on the device when they did not come along
    if (kind == PSC_REQ_SCC && !with_t) PSC_TRY(build_transpose(g));
    PSC_TRY(batch_attach(g, vbase.data(), R, false));
    PSC_TRY(stamp("transpose"));
    if (kind == PSC_REQ_SCC) {
      uint64_t* d;
      PSC_TRY(ensure_t(g, B_LABELS, n, &d));
      std::vector<uint64_t> seeds(R);
      for (uint32_t k = 0; k < R; k++) seeds[k] = B[k]->seed;
      PSC_TRY(scc_batch_run(g, &S->cfg.scc, seeds.data(), d));
      PSC_TRY(stamp("solve"));
      for (uint32_t k = 0; k < R; k++)
        PSC_CUDA(cudaMemcpyAsync(B[k]->out, d + vbase[k], B[k]->n * 8, cudaMemcpyDefault, g->stream));
    } else {
      uint32_t* d;
      PSC_TRY(ensure_t(g, B_AUX0, n + 1, &d));
      PSC_TRY(cc_batch_run(g, S->cfg.cc_beta, d));
      PSC_TRY(stamp("solve"));
      for (uint32_t k = 0; k < R; k++)
        PSC_CUDA(cudaMemcpyAsync(B[k]->out, d + vbase[k], B[k]->n * 4, cudaMemcpyDefault, g->stream));
    }
    return call_end(g);
  };
  const int st = body();
  *launches = g->stats.kernel_launches;
  psc_graph_free(g);
  if (tr) {
    std::fprintf(stderr, "server batch at %.2f ms ticket %llu kind %d requests %u n %llu m %llu:",
                 std::chrono::duration<double, std::milli>(t_begin - S->t_epoch).count(),
                 (unsigned long long)ticket, kind, R, (unsigned long long)n, (unsigned long long)m);
    for (auto& mk : marks) std::fprintf(stderr, " %s %.2f", mk.first, mk.second);
    std::fprintf(stderr, " freed %.2f ms\n",
                 std::chrono::duration<double, std::milli>(Clock::now() - t_begin).count());
  }
  return st;
}

// Batch of the queue head's kind: requests in arrival order while they fit
// the budget left and the batch's share of the budget (budget / workers, so
// that a backlog is spread over all workers); a lone request always fits an
// idle server.  Caller holds the lock.  Returns false if nothing may start.
bool take_batch(psc_server_s* S, std::vector<Request*>& batch, int& kind, uint64_t& bytes) {
  if (S->queue.empty()) return false;
  const uint64_t budget = S->cfg.hbm_budget;
  const uint64_t share = std::max<uint64_t>(1, budget / S->cfg.workers);
  const uint64_t ecap = S->cfg.max_batch_edges ? S->cfg.max_batch_edges : ~0ull;
  kind = S->queue.front()->kind;
  bytes = 0;
  uint64_t edges = 0;
  for (auto it = S->queue.begin(); it != S->queue.end() && batch.size() < S->cfg.max_batch;) {
    Request* r = *it;
    if (r->kind != kind) {
      ++it;
      continue;
    }
    const bool fits = S->used + bytes + r->bytes <= budget && bytes + r->bytes <= share &&
                      edges + r->m <= ecap;
    // a request larger than the share goes alone when the budget allows
    if (!fits && !(batch.empty() && (S->running == 0 || S->used + r->bytes <= budget))) break;
    batch.push_back(r);
    bytes += r->bytes;
    edges += r->m;
    it = S->queue.erase(it);
  }
  return !batch.empty();
}

void worker_loop(psc_server_s* S) {
  cudaSetDevice(S->device);
  for (;;) {
    std::vector<Request*> batch;
    int kind = 0;
    uint64_t bytes = 0, ticket = 0;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      // on stop, the queue is still served before the workers leave
      S->work_cv.wait(lk, [&] { return take_batch(S, batch, kind, bytes) || S->stop; });
      if (batch.empty()) return;  // stopping with nothing to take
      ticket = S->next_ticket++;
      S->used += bytes;
      S->running++;
      S->stats.batches++;
      S->stats.peak_bytes = std::max(S->stats.peak_bytes, S->used);
      S->stats.max_running = std::max<uint64_t>(S->stats.max_running, S->running);
    }
    const auto t0 = Clock::now();
    for (auto* r : batch) {
      r->t_start = t0;
      r->batch_size = (uint32_t)batch.size();
    }
    uint64_t launches = 0;
    // malformed requests fail alone: the rest of the batch runs again
    // without them (at most once per malformed request)
    std::vector<Request*> run = batch, failed;
    int st = PSC_OK;
    while (!run.empty()) {
      std::vector<char> bad;
      uint64_t l = 0;
      st = run_batch(S, run, kind, ticket, &l, &bad);
      launches += l;
      if (st != PSC_ERR_INVALID || bad.empty()) break;
      std::vector<Request*> keep;
      for (size_t k = 0; k < run.size(); k++) {
        if (bad[k]) {
          run[k]->status = PSC_ERR_INVALID;
          failed.push_back(run[k]);
        } else {
          keep.push_back(run[k]);
        }
      }
      if (keep.size() == run.size()) break;  // flags without a flagged request
      run.swap(keep);
      st = PSC_OK;
      // the rest copies again, after the batches taken since (a ticket is
      // drawn only for a run that follows: every ticket drawn must be served)
      if (!run.empty()) ticket = take_ticket(S);
    }
    const auto t1 = Clock::now();
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->stats.kernel_launches += launches;
      S->used -= bytes;
      S->running--;
      S->stats.busy_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
      for (auto* r : run) {
        r->status = st;
        r->batch_size = (uint32_t)run.size();
      }
      for (auto* r : batch) {
        r->t_done = t1;
        r->done = true;
        S->stats.completed++;
        if (r->status != PSC_OK) S->stats.failed++;
      }
    }
    S->done_cv.notify_all();
    S->work_cv.notify_all();
  }
}

}  // namespace
}  // namespace psc

using namespace psc;

extern "C" void psc_server_config_default(psc_server_config_t* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->hbm_budget = 120ull << 30;
  c->workers = 4;
  c->max_batch = 4096;
  c->cc_beta = 0.2;
  psc_params_default(&c->scc);
  c->max_batch_edges = 1ull << 28;
}

extern "C" int psc_server_create(const psc_server_config_t* cfg, psc_server_t* out) {
  if (!out) return PSC_ERR_INVALID;
  *out = nullptr;
  psc_server_config_t c;
  psc_server_config_default(&c);
  if (cfg) c = *cfg;
  if (c.hbm_budget == 0 || c.workers == 0 || c.workers > 64 || c.max_batch == 0 ||
      !(c.cc_beta > 0) || !(c.scc.beta > 0))
    return PSC_ERR_INVALID;
  int dev = 0;
  PSC_CUDA(cudaGetDevice(&dev));
  int least = 0, greatest = 0;
  PSC_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  auto* S = new psc_server_s();
  S->cfg = c;
  S->device = dev;
  S->urgent_priority = greatest;
  for (uint32_t w = 0; w < 2 * c.workers; w++) S->workers.emplace_back(worker_loop, S);
  *out = S;
  return PSC_OK;
}

extern "C" int psc_server_submit(psc_server_t S, int kind, const uint64_t* off, const uint32_t* E,
                                 const uint64_t* in_off, const uint32_t* in_E, uint64_t n,
                                 uint64_t m, uint64_t seed, void* labels_out, uint64_t* id_out) {
  if (!S || !off || (m && !E) || !labels_out || !id_out || n == 0 || n >= 0xFFFFFFFFull)
    return PSC_ERR_INVALID;
  if (kind != PSC_REQ_SCC && kind != PSC_REQ_CC) return PSC_ERR_INVALID;
  if (off[0] != 0 || off[n] != m) return PSC_ERR_INVALID;
  if ((in_off && m && !in_E) || (!in_off && in_E)) return PSC_ERR_INVALID;
  if (in_off && (kind != PSC_REQ_SCC || in_off[0] != 0 || in_off[n] != m)) return PSC_ERR_INVALID;
  const uint64_t bytes = request_bytes(kind, n, m, in_off != nullptr);
  auto* r = new Request();
  r->kind = kind;
  r->n = n;
  r->m = m;
  r->off = off;
  r->E = E;
  r->in_off = in_off;
  r->in_E = in_E;
  r->seed = seed;
  r->out = labels_out;
  r->bytes = bytes;
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) {
      delete r;
      return PSC_ERR_INVALID;
    }
    if (bytes > S->cfg.hbm_budget) {
      S->stats.rejected++;
      delete r;
      return PSC_ERR_TOO_LARGE;
    }
    r->id = S->next_id++;
    S->requests[r->id] = r;
    S->queue.push_back(r);
    S->stats.submitted++;
    *id_out = r->id;
  }
  S->work_cv.notify_one();
  return PSC_OK;
}

extern "C" int psc_server_wait(psc_server_t S, uint64_t id, psc_request_info_t* info) {
  if (!S) return PSC_ERR_INVALID;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->requests.find(id);
  if (it == S->requests.end()) return PSC_ERR_INVALID;
  Request* r = it->second;
  S->done_cv.wait(lk, [&] { return r->done; });
  if (info) {
    info->status = r->status;
    info->batch_size = r->batch_size;
    info->queue_ms = std::chrono::duration<double, std::milli>(r->t_start - r->t_submit).count();
    info->latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  }
  const int st = r->status;
  S->requests.erase(it);
  delete r;
  return st;
}

extern "C" int psc_server_drain(psc_server_t S) {
  if (!S) return PSC_ERR_INVALID;
  std::unique_lock<std::mutex> lk(S->mu);
  S->done_cv.wait(lk, [&] {
    if (!S->queue.empty() || S->running) return false;
    for (auto& kv : S->requests)
      if (!kv.second->done) return false;
    return true;
  });
  return PSC_OK;
}

extern "C" int psc_server_stats(psc_server_t S, psc_server_stats_t* out) {
  if (!S || !out) return PSC_ERR_INVALID;
  std::lock_guard<std::mutex> lk(S->mu);
  *out = S->stats;
  out->queued = S->queue.size();
  out->bytes_in_use = S->used;
  return PSC_OK;
}

extern "C" int psc_server_destroy(psc_server_t S) {
  if (!S) return PSC_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->work_cv.notify_all();
  for (auto& t : S->workers) t.join();
  for (auto& kv : S->requests) delete kv.second;
  delete S;
  return PSC_OK;
}

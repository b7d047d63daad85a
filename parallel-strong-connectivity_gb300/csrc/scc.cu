// Strongly connected components on the device (SCC::scc, src/scc.hpp:277-476).
//
// Phases, each in the reference's order and with its label encoding
// (TOP bit 2^32 = done; trimmed vertex i of ZEROS -> (i+1)|TOP; pivot labels
// start at |ZEROS|+1):
//   trim         in/out-degree-zero filter by one scan; NON_ZEROS permuted by
//                the library's Feistel bijection (stands in for
//                parlay::random_shuffle)                    scc.hpp:288-305
//   first pivot  forward and backward reach from P[0]     scc.hpp:316-350
//   batches      prefix-doubling batches of live centres   scc.hpp:373-425
//   multi-search per direction, the closure {(v, pivot)} of reachability
//                inside each pivot's subproblem, held in a 64-bit
//                open-addressing table (atomicCAS, linear probing, grown by a
//                rehash kernel) and expanded from a frontier of new
//                (v, pivot) pairs, so every pair is expanded exactly once
//                                                           scc.hpp:144-275
//   partition    (v,l) in both tables -> max l|TOP, else max l  scc.hpp:437-464
//   finalise     (label & 0xFFFFFFFF) - 1                   scc.hpp:475-476
// The closure is unique, so the labels equal the reference's for the same
// pivot order no matter how the device schedules the work.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "engines.cuh"
#include "scan.cuh"

namespace psc {


struct TrimEmit {
  uint64_t* labels;
  uint32_t* nz;
  __device__ void operator()(uint64_t i, uint64_t excl, uint32_t v) const {
    if (v) {
      labels[i] = kTopBit + excl + 1;  // 1 + (i | TOP_BIT), scc.hpp:304-305
    } else {
      labels[i] = 0;
      nz[i - excl] = (uint32_t)i;
    }
  }
};

// Pivot order P[i] = nz[feistel(i)] (the reference's random_shuffle of
// NON_ZEROS, scc.hpp:303).  The permutation walks its cycle until it lands
// in [0, np): 2.5 network passes per element on average for 27 M elements on
// a 2^26 domain, but the slowest of a warp's 32 lanes takes ~8.  So a warp
// takes a chunk of kPermChunk elements, and a lane that lands takes the
// chunk's next element at once (one network pass per loop step): the warp
// waits only at the end of its chunk.
constexpr uint64_t kPermChunk = 32 * 32;

__global__ void k_perm_gather(const uint32_t* __restrict__ nz, uint64_t np, FeistelKey key,
                              uint32_t* P) {
  const unsigned lane = lane_id();
  const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t c0 = gw * kPermChunk; c0 < np; c0 += nw * kPermChunk) {
    const uint64_t c1 = c0 + kPermChunk < np ? c0 + kPermChunk : np;
    uint64_t next = c0 + 32;  // first element no lane has taken yet
    uint64_t i = c0 + lane, x = i;
    bool act = i < c1;
    while (__any_sync(kFull, act)) {
      bool landed = false;
      if (act) {
        x = feistel_net(key, x);
        landed = x < np;
        if (landed) P[i] = nz[x];
      }
      const uint32_t lm = __ballot_sync(kFull, landed);
      if (landed) {
        i = next + __popc(lm & ((1u << lane) - 1));
        x = i;
        act = i < c1;
      }
      next += __popc(lm);
    }
  }
}

// First-pivot labels (scc.hpp:340-349) in vertex order: a warp reads one word
// of each bitmap for its 32 vertices and writes the labels of reached vertices
// that trimming did not finish (labels without kTopBit).  It also writes the
// bitmap of finished vertices (trimmed, or reached both ways), one ballot per
// 32 vertices, for the compaction of the pivot order that follows.
__global__ void k_label_first(const uint32_t* __restrict__ vf, const uint32_t* __restrict__ vb,
                              uint64_t n, uint64_t* labels, uint64_t label, uint32_t* done) {
  const unsigned lane = lane_id();
  for (uint64_t base = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~31ull; base < n;
       base += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t v = base + lane;
    bool fin = false;
    if (v < n) {
      const uint32_t bit = 1u << lane;
      const bool f = __ldg(&vf[base >> 5]) & bit, b = __ldg(&vb[base >> 5]) & bit;
      fin = labels[v] & kTopBit;
      if ((f || b) && !fin) {
        labels[v] = (f && b) ? (label | kTopBit) : label;
        fin = f && b;
      }
    }
    const uint32_t word = __ballot_sync(kFull, fin);
    if (lane == 0) done[base >> 5] = word;
  }
}

// Partition (scc.hpp:437-464) of one batch in one launch: items below cap_s
// are slots of the smaller table, whose pairs also found in the larger table
// get their label with kTopBit (reached both ways); the rest are slots of the
// larger table.  Every write is an atomicMax, so the order does not matter.
__global__ void k_partition(const unsigned long long* __restrict__ Ts, uint64_t cap_s,
                            const unsigned long long* __restrict__ Tl, uint64_t cap_l,
                            unsigned long long* labels) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap_s + cap_l;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const bool small = i < cap_s;
    const uint64_t e = small ? Ts[i] : Tl[i - cap_s];
    if (e == kEmpty) continue;
    const uint32_t v = (uint32_t)(e >> 32);
    const uint64_t l = e & kValMask;
    const uint64_t val = small && table_contains(Tl, cap_l - 1, e) ? (l | kTopBit) : l;
    if (labels[v] < val) atomicMax(&labels[v], (unsigned long long)val);
  }
}

__global__ void k_finalise(uint64_t* labels, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    labels[i] = (labels[i] & kValMask) - 1;
}

static int scc_phases(psc_graph_s* g, uint64_t* labels, const psc_params_t* p);

void scc_clear_grow_events(psc_graph_s* g) {
  for (auto& pr : g->grow_events) {
    give_event(g, pr.first);
    give_event(g, pr.second);
  }
  g->grow_events.clear();
}

int scc_phase_times(psc_graph_s* g) {
  PSC_CUDA(cudaEventSynchronize(g->ph[3]));
  float a = 0, b = 0, c = 0;
  PSC_CUDA(cudaEventElapsedTime(&a, g->ph[0], g->ph[1]));
  PSC_CUDA(cudaEventElapsedTime(&b, g->ph[1], g->ph[2]));
  PSC_CUDA(cudaEventElapsedTime(&c, g->ph[2], g->ph[3]));
  double grow = 0;
  for (auto& pr : g->grow_events) {
    float x = 0;
    PSC_CUDA(cudaEventElapsedTime(&x, pr.first, pr.second));
    grow += x;
  }
  g->stats.phase_ms[0] = a;
  g->stats.phase_ms[1] = b;
  g->stats.phase_ms[2] = c - grow;
  g->stats.phase_ms[3] = grow;
  return PSC_OK;
}

int scc_run(psc_graph_s* g, const psc_params_t* p, uint64_t* labels) {
  g->block = p->block;
  const int st = scc_timed(g, [&](psc_graph_s* h) { return scc_phases(h, labels, p); });
  g->block = 0;
  return st;
}

int scc_partition(psc_graph_s* g, const MsResult res[2], uint64_t* labels) {
  const unsigned tb = 256;
  const MsResult& rf = res[0];
  const MsResult& rb = res[1];
  const bool f_small = rf.cap <= rb.cap;
  const unsigned long long* Ts = (const unsigned long long*)g->bufs[f_small ? B_TF : B_TB].p;
  const unsigned long long* Tl = (const unsigned long long*)g->bufs[f_small ? B_TB : B_TF].p;
  const uint64_t cap_s = f_small ? rf.cap : rb.cap, cap_l = f_small ? rb.cap : rf.cap;
  {
    ProfScope ps(g, F_PARTITION);
    ps.bytes = 8.0 * cap_s + 16.0 * (f_small ? rf.ne : rb.ne) + 8.0 * cap_l +
               8.0 * (f_small ? rb.ne : rf.ne);
    k_partition<<<grid_for(g, cap_s + cap_l, tb), tb, 0, g->stream>>>(
        Ts, cap_s, Tl, cap_l, (unsigned long long*)labels);
  }
  PSC_CUDA(cudaGetLastError());
  return PSC_OK;
}

// Batches whose candidate pivots fit the multi-search's VGC range (one pair
// per resident warp, num_sms * 32) start asynchronously (see the batch loop
// below): their upper bound chooses the same VGC sub-round as the pivot count
// would, and sizes their tables modestly.  Larger ones wait for the count.
#ifndef PSC_ASYNC_BATCHES
#define PSC_ASYNC_BATCHES 1
#endif

static int scc_phases(psc_graph_s* g, uint64_t* labels, const psc_params_t* p) {
  const uint64_t n = g->n;
  const unsigned tb = 256;
  uint32_t *P, *nz, *centers, *front, *vf, *vb;
  PSC_TRY(ensure_t(g, B_P, n + 1, &P));
  PSC_TRY(ensure_t(g, B_TMP32, n + 1, &nz));
  // trim
  uint64_t n_zeros = 0;
  // algorithmic bytes: two offsets of each direction read, an 8-byte label and
  // (for the live vertices) a 4-byte index written
  PSC_TRY(scan_emit_flags(g, n, ZeroFlag{g->off, g->in_off}, TrimEmit{labels, nz}, &n_zeros, F_TRIM,
                          28.0));
  const uint64_t np = n - n_zeros;
  if (np > 0) {
    FeistelKey key = feistel_key(np, p->seed);
    ProfScope ps(g, F_TRIM);
    ps.bytes = 8.0 * np;
    k_perm_gather<<<grid_for(g, np, tb), tb, 0, g->stream>>>(nz, np, key, P);
  }
  uint64_t label_offset = n_zeros + 1;
  PSC_CUDA(cudaEventRecord(g->ph[1], g->stream));
  if (np > 0) {
    // first pivot (scc.hpp:316-350)
    uint32_t src = 0;
    PSC_CUDA(cudaMemcpyAsync(&g->hctr->aux1, P, 4, cudaMemcpyDeviceToHost, g->stream));
    PSC_CUDA(cudaStreamSynchronize(g->stream));
    std::memcpy(&src, &g->hctr->aux1, 4);
    PSC_TRY(ensure_t(g, B_VIS_F, (n + 31) / 32 + 1, &vf));
    PSC_TRY(ensure_t(g, B_VIS_B, (n + 31) / 32 + 1, &vb));
    uint32_t r1 = 0, r2 = 0;
    PSC_TRY(reach_pair(g, src, p->local_reach != 0, p->tau, p->pull_div, vf, vb, &r1, &r2));
    g->stats.reach_rounds = r1 + r2;
    uint32_t* done;  // finished vertices after the first pivot (frontier slot, free by now)
    PSC_TRY(ensure_t(g, B_FB_A, (n + 31) / 32 + 1, &done));
    {
      ProfScope ps(g, F_LABEL_FIRST);
      // two bitmaps read and one written; label read per vertex, written per live vertex
      ps.bytes = 0.375 * n + 8.0 * n + 8.0 * np;
      k_label_first<<<grid_for(g, n, tb), tb, 0, g->stream>>>(vf, vb, n, labels, label_offset,
                                                            done);
    }
    PSC_TRY(ensure_t(g, B_CENTERS, np + 1, &centers));
    uint64_t nc = 0;
    PSC_TRY(scan_emit_flags(g, np, NotDoneBitAt{P, done}, CopyAt{P, centers, 0}, &nc, F_COMPACT, 8.0,
                      4.0));
    label_offset++;
    PSC_CUDA(cudaEventRecord(g->ph[2], g->stream));

    // prefix-doubling batches (scc.hpp:365-473)
    PSC_TRY(ensure_t(g, B_FRONT, np + 1, &front));
    const uint64_t n_remaining = nc;
    uint64_t step_size = 1, cur_offset = 0, finished = 0;
    uint64_t in_ne = 1, out_ne = 1;
    while (finished != n_remaining) {
      const uint64_t end = std::min(cur_offset + step_size, n_remaining);
      const uint64_t vs_size = end - cur_offset;
      finished += vs_size;
      step_size = (uint64_t)std::ceil((double)step_size * p->beta);
      if (step_size > n_remaining) step_size = n_remaining;
      if (step_size == 0) step_size = 1;
      // Small batches start without waiting for their pivot count: the
      // compaction's total is read on the device by the seeds and the first
      // sub-round, so the batch waits on the host once per sub-round only.
      const bool async = PSC_ASYNC_BATCHES && p->local_scc && vs_size <= (uint64_t)g->num_sms * 32;
      uint64_t nf = 0;
      const unsigned long long* nf_dev = nullptr;
      PSC_TRY(scan_emit_flags(g, vs_size, NotDoneAt{centers, labels, cur_offset},
                              CopyAt{centers, front, cur_offset}, async ? nullptr : &nf,
                              F_COMPACT, 12.0, 4.0, async ? &nf_dev : nullptr));
      cur_offset = end;
      if (!async && nf == 0) continue;
      MsResult res[2];
      const uint64_t prev[2] = {out_ne, in_ne};
      if (async) {
        MsAsync as;
        as.nf_dev = nf_dev;
        PSC_TRY(ms_pair(g, front, vs_size, label_offset, labels, p, prev, res, nullptr, 0, &as));
        nf = as.n_front;
        if (nf == 0) continue;
      } else {
        PSC_TRY(ms_pair(g, front, nf, label_offset, labels, p, prev, res));
      }
      g->stats.batches++;
      label_offset += nf;
      PSC_TRY(scc_partition(g, res, labels));
      out_ne = res[0].ne;
      in_ne = res[1].ne;
    }
  }
  if (np == 0) PSC_CUDA(cudaEventRecord(g->ph[2], g->stream));
  PSC_CUDA(cudaEventRecord(g->ph[3], g->stream));
  {
    ProfScope ps(g, F_FINALISE);
    ps.bytes = 16.0 * n;
    k_finalise<<<grid_for(g, n, tb), tb, 0, g->stream>>>(labels, n);
  }
  PSC_CUDA(cudaGetLastError());
  return PSC_OK;
}

}  // namespace psc

using namespace psc;

extern "C" int psc_scc(psc_graph_t g, const psc_params_t* p, uint64_t* labels_out) {
  if (!g || !labels_out) return PSC_ERR_INVALID;
  psc_params_t def;
  if (!p) {
    psc_params_default(&def);
    p = &def;
  }
  if (!(p->beta > 0)) return PSC_ERR_INVALID;
  PSC_TRY(call_begin(g));
  uint64_t* d;
  PSC_TRY(ensure_t(g, B_LABELS, g->n, &d));
  PSC_TRY(scc_run(g, p, d));
  PSC_CUDA(cudaMemcpyAsync(labels_out, d, g->n * 8, cudaMemcpyDeviceToHost, g->stream));
  return call_end(g);
}

extern "C" int psc_scc_device(psc_graph_t g, const psc_params_t* p, uint64_t* d_labels) {
  if (!g || !d_labels) return PSC_ERR_INVALID;
  psc_params_t def;
  if (!p) {
    psc_params_default(&def);
    p = &def;
  }
  if (!(p->beta > 0)) return PSC_ERR_INVALID;
  PSC_TRY(call_begin(g));
  PSC_TRY(scc_run(g, p, d_labels));
  return call_end(g);
}

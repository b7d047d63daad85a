// Batched SCC and connectivity over many independent graphs packed into one
// CSR (+ transpose) with a graph-offset table.
//
// Graph k owns the global vertex ids [vbase[k], vbase[k+1]) and its edges stay
// inside that range, so one device graph holds the whole batch and every
// kernel of the plain path runs unchanged over it: a frontier, a multi-search
// pair set or a table simply mixes items of many graphs, and each warp pulls
// whatever (graph, frontier chunk) work is next in the shared queue.
//
// Each graph still follows its own run of SCC::scc (src/scc.hpp:277-476)
// exactly, in lockstep with the others:
//   trim        one scan over the union; a graph's ZEROS keep their local
//               index (the union's index minus the zeros of earlier graphs,
//               applied at finalise through a marker bit)
//   permutation P_k = the Feistel bijection keyed by the graph's own seed on
//               its own NON_ZEROS segment
//   first pivot P_k[0] for every graph, one forward and one backward search
//               from all of them at once
//   batches     batch j of the union = the j-th prefix-doubling window of
//               every graph that still has one (window sizes per graph from
//               its own live-centre count and beta, src/scc.hpp:373-383)
//   labels      per graph: |ZEROS_k| + 1 for the first pivot, then
//               label_offset_k + index within the graph's part of the batch
// Labels never meet across graphs (edges never cross), so each graph's labels
// equal those of a plain solve of that graph alone with the same seed and
// parameters, and finalise leaves them as local vertex ids.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "engines.cuh"
#include "psc_hash.h"
#include "scan.cuh"

namespace psc {

// Marks a trimmed vertex's label until finalise (bit 62; labels of live
// vertices stay below 2^33, so the bit is free).
constexpr uint64_t kTrimMark = 1ull << 62;

// Largest frontier of a batch still expanded by VGC rounds.
constexpr uint64_t kBatchVgcMax = ~0ull;

// ---------------------------------------------------------------------------
// Graph-offset table
// ---------------------------------------------------------------------------

__global__ void k_fill_gid(const uint64_t* __restrict__ vbase, uint32_t G, uint64_t n, uint32_t* gid) {
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x)
    gid[v] = last_le(vbase, G + 1, v);
}

// Per-graph edge ranges of both directions: graph k's edges are
// E[eb[k] .. eb[k+1]) with eb[k] = off[vbase[k]] (and in_E with in_off).
__global__ void k_graph_edge_bases(const uint64_t* __restrict__ off,
                                   const uint64_t* __restrict__ in_off,
                                   const uint64_t* __restrict__ vbase, uint32_t G, uint64_t* eb,
                                   uint64_t* eb_in) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k <= G; k += gridDim.x * blockDim.x) {
    eb[k] = off[vbase[k]];
    eb_in[k] = in_off[vbase[k]];
  }
}

// Every edge stays inside its graph's id range: one coalesced pass over E in
// chunks of kCheckChunk edges per warp.  Lane 0 finds the graph of the
// chunk's first edge (the last k with eb[k] <= e, so empty graphs are
// skipped); each lane then steps k forward while its edge lies past eb[k+1]
// (edges are grouped by graph, so this is at most a few steps) and checks
// vbase[k] <= E[e] < vbase[k+1].
constexpr int kCheckK = 8;
constexpr uint64_t kCheckChunk = 32 * kCheckK;

__global__ void k_check_batch_edges(const uint32_t* __restrict__ E, uint64_t m,
                                    const uint64_t* __restrict__ eb,
                                    const uint64_t* __restrict__ vbase, uint32_t G,
                                    unsigned long long* bad) {
  const unsigned lane = lane_id();
  const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  bool found = false;
  for (uint64_t c0 = gw * kCheckChunk; c0 < m; c0 += nw * kCheckChunk) {
    uint32_t k0 = 0;
    if (lane == 0) {
      uint32_t lo = 0, hi = G - 1;  // last k in [0, G) with eb[k] <= c0
      while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (__ldg(&eb[mid]) <= c0)
          lo = mid;
        else
          hi = mid - 1;
      }
      k0 = lo;
    }
    uint32_t k = __shfl_sync(kFull, k0, 0);
    uint32_t v[kCheckK];
#pragma unroll
    for (int j = 0; j < kCheckK; j++) {
      const uint64_t e = c0 + (uint64_t)j * 32 + lane;
      v[j] = e < m ? __ldg(&E[e]) : 0u;
    }
#pragma unroll
    for (int j = 0; j < kCheckK; j++) {
      const uint64_t e = c0 + (uint64_t)j * 32 + lane;
      if (e < m) {
        while (k + 1 < G && __ldg(&eb[k + 1]) <= e) k++;
        found |= v[j] < __ldg(&vbase[k]) || v[j] >= __ldg(&vbase[k + 1]);
      }
    }
  }
  if (__any_sync(kFull, found) && lane == 0) atomicAdd(bad, 1ull);
}

// ---------------------------------------------------------------------------
// Batched SCC kernels
// ---------------------------------------------------------------------------

struct TrimEmitB {
  uint64_t* labels;
  uint32_t* nz;
  __device__ void operator()(uint64_t i, uint64_t excl, uint32_t v) const {
    if (v) {
      labels[i] = kTrimMark | kTopBit | (excl + 1);  // union index; made local at finalise
    } else {
      labels[i] = 0;
      nz[i - excl] = (uint32_t)i;
    }
  }
};

// out[k] = first index i of the nondecreasing nz[0..na) with nz[i] >= vbase[k],
// for k in [0, G]; nz holds vertex ids in increasing order.
__global__ void k_bases_by_value(const uint32_t* __restrict__ nz, uint64_t na,
                                 const uint64_t* __restrict__ vbase, uint32_t G, uint64_t* out) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k <= G; k += gridDim.x * blockDim.x) {
    const uint64_t x = vbase[k];
    uint64_t lo = 0, hi = na;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (nz[mid] < x)
        lo = mid + 1;
      else
        hi = mid;
    }
    out[k] = lo;
  }
}

// out[j] = first index i of a[0..na) whose graph gid[a[i]] >= graphs[j]
// (graphs null: graph j), for j in [0, cnt); out[cnt] = na.  The graphs of a
// are nondecreasing.
__global__ void k_bases_by_graph(const uint32_t* __restrict__ a, uint64_t na,
                                 const uint32_t* __restrict__ gid, const uint32_t* __restrict__ graphs,
                                 uint32_t cnt, uint64_t* out) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j <= cnt; j += gridDim.x * blockDim.x) {
    if (j == cnt) {
      out[j] = na;
      continue;
    }
    const uint32_t k = graphs ? graphs[j] : j;
    uint64_t lo = 0, hi = na;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (gid[a[mid]] < k)
        lo = mid + 1;
      else
        hi = mid;
    }
    out[j] = lo;
  }
}

// Per-graph pivot orders: P[j] = nz[base + feistel_k(j - base)] on graph k's
// segment [npbase[k], npbase[k+1]) of nz, with the lanes of a warp refilled as
// their walks land, as in k_perm_gather.
constexpr uint64_t kPermChunkB = 32 * 32;

__global__ void k_perm_gather_b(const uint32_t* __restrict__ nz, uint64_t np,
                                const uint32_t* __restrict__ gid, const uint64_t* __restrict__ npbase,
                                const FeistelKey* __restrict__ keys, uint32_t* P) {
  const unsigned lane = lane_id();
  const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t c0 = gw * kPermChunkB; c0 < np; c0 += nw * kPermChunkB) {
    const uint64_t c1 = c0 + kPermChunkB < np ? c0 + kPermChunkB : np;
    uint64_t next = c0 + 32;
    uint64_t j = c0 + lane, x = 0, base = 0;
    FeistelKey key{};
    bool act = j < c1;
    auto start = [&]() {  // element j: its graph's key and segment base
      const uint32_t k = gid[nz[j]];
      base = npbase[k];
      key = keys[k];
      x = j - base;
    };
    if (act) start();
    while (__any_sync(kFull, act)) {
      bool landed = false;
      if (act) {
        // a segment of at most one element maps to itself (feistel's k <= 1)
        x = key.k <= 1 ? 0 : feistel_net(key, x);
        landed = x < key.k;
        if (landed) P[j] = nz[base + x];
      }
      const uint32_t lm = __ballot_sync(kFull, landed);
      if (landed) {
        j = next + __popc(lm & ((1u << lane) - 1));
        act = j < c1;
        if (act) start();
      }
      next += __popc(lm);
    }
  }
}

__global__ void k_batch_sources(const uint32_t* __restrict__ P, const uint64_t* __restrict__ npbase,
                                const uint32_t* __restrict__ graphs, uint32_t cnt, uint32_t* srcs) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x)
    srcs[j] = P[npbase[graphs[j]]];
}

// First-pivot labels of every graph, in vertex order (see k_label_first):
// reached vertices that trimming did not finish take their graph's label;
// the bitmap of finished vertices is written alongside.
__global__ void k_label_first_b(const uint32_t* __restrict__ vf, const uint32_t* __restrict__ vb,
                                uint64_t n, const uint32_t* __restrict__ gid,
                                const uint64_t* __restrict__ lo, uint64_t* labels, uint32_t* done) {
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
        const uint64_t label = lo[gid[v]];
        labels[v] = (f && b) ? (label | kTopBit) : label;
        fin = f && b;
      }
    }
    const uint32_t word = __ballot_sync(kFull, fin);
    if (lane == 0) done[base >> 5] = word;
  }
}

// Live centres inside the batch's windows: item j of the concatenated windows
// lies in window a = last_le(wpre, j), at centres[wstart[a] + j - wpre[a]].
struct WinNotDone {
  const uint32_t* centres;
  const uint64_t* labels;
  const uint64_t* wstart;
  const uint64_t* wpre;
  uint32_t nw;
  __device__ uint32_t centre(uint64_t j) const {
    const uint32_t a = last_le(wpre, nw, j);
    return centres[wstart[a] + (j - wpre[a])];
  }
  __device__ uint32_t operator()(uint64_t j) const { return (labels[centre(j)] & kTopBit) ? 0u : 1u; }
};

struct WinCopy {
  WinNotDone w;
  uint32_t* front;
  __device__ void operator()(uint64_t j, uint64_t excl, uint32_t v) const {
    if (v) front[excl] = w.centre(j);
  }
};

// Pivot labels of a batch: item i of window a (front[fb[a] .. fb[a+1]))
// takes lo[graph] + (i - fb[a]), the graph's label_offset + its index.
__global__ void k_front_labels(uint64_t nf, const uint64_t* __restrict__ fb,
                               const uint32_t* __restrict__ wg, uint32_t nw,
                               const uint64_t* __restrict__ lo, uint32_t* flab) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nf;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t a = last_le(fb, nw + 1, i);
    flab[i] = (uint32_t)(lo[wg[a]] + (i - fb[a]));
  }
}

__global__ void k_lo_advance(const uint64_t* __restrict__ fb, const uint32_t* __restrict__ wg,
                             uint32_t nw, uint64_t* lo) {
  for (uint32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < nw; a += gridDim.x * blockDim.x)
    lo[wg[a]] += fb[a + 1] - fb[a];
}

__global__ void k_lo_first(const uint64_t* __restrict__ npbase, uint32_t G, uint64_t* lo) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < G; k += gridDim.x * blockDim.x)
    if (npbase[k + 1] > npbase[k]) lo[k] += 1;
}

__global__ void k_finalise_b(uint64_t* labels, uint64_t n, const uint32_t* __restrict__ gid,
                             const uint64_t* __restrict__ vbase, const uint64_t* __restrict__ npbase) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t l = labels[i];
    uint64_t r = (l & kValMask) - 1;
    if (l & kTrimMark) {
      const uint32_t k = gid[i];
      r -= vbase[k] - npbase[k];  // zeros of the earlier graphs
    }
    labels[i] = r;
  }
}

__global__ void k_localise_u32(uint32_t* labels, uint64_t n, const uint32_t* __restrict__ gid,
                               const uint64_t* __restrict__ vbase) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    labels[i] -= (uint32_t)vbase[gid[i]];
}

// ---------------------------------------------------------------------------
// Host driver
// ---------------------------------------------------------------------------

namespace {

// Per-graph device arrays carved from slot B_GRAPHS (u64 words).
struct BatchArrays {
  uint64_t* npbase;  // [G+1] NON_ZEROS segment bases in P
  uint64_t* lo;      // [G]   label_offset of each graph
  uint64_t* cbase;   // [G+1] centre segment bases
  uint64_t* fb;      // [G+1] batch front bases per window
  FeistelKey* keys;  // [G]
  uint32_t* glist;   // [G]   graphs with a first pivot
  uint32_t* srcs;    // [G]   their first pivots
};

size_t batch_words(uint32_t G) {
  const size_t G1 = (size_t)G + 1;
  return 4 * G1 + (sizeof(FeistelKey) / 8 + 1) * G1 + G1 + 8;
}

int batch_arrays(psc_graph_s* g, BatchArrays* a) {
  const uint32_t G = g->num_graphs;
  const size_t G1 = (size_t)G + 1;
  uint64_t* w;
  PSC_TRY(ensure_t(g, B_GRAPHS, batch_words(G), &w));
  a->npbase = w;
  a->lo = w + G1;
  a->cbase = w + 2 * G1;
  a->fb = w + 3 * G1;
  a->keys = (FeistelKey*)(w + 4 * G1);
  uint64_t* rest = w + 4 * G1 + (sizeof(FeistelKey) / 8 + 1) * G1;
  a->glist = (uint32_t*)rest;
  a->srcs = (uint32_t*)rest + G1;
  return PSC_OK;
}

// One window of a graph's prefix-doubling schedule.
struct Window {
  uint32_t graph;
  uint64_t start, len;  // into the centres array
};

// Windows of every batch: batch j holds the j-th window of each graph that
// has one (src/scc.hpp:373-383 per graph).
std::vector<std::vector<Window>> batch_schedule(const std::vector<uint64_t>& cbase, uint32_t G,
                                                double beta) {
  std::vector<std::vector<Window>> out;
  std::vector<uint64_t> step(G, 1), cur(G, 0);
  for (;;) {
    std::vector<Window> ws;
    for (uint32_t k = 0; k < G; k++) {
      const uint64_t nrem = cbase[k + 1] - cbase[k];
      if (cur[k] == nrem) continue;
      const uint64_t end = std::min(cur[k] + step[k], nrem);
      ws.push_back(Window{k, cbase[k] + cur[k], end - cur[k]});
      uint64_t st = (uint64_t)std::ceil((double)step[k] * beta);
      if (st > nrem) st = nrem;
      if (st == 0) st = 1;
      step[k] = st;
      cur[k] = end;
    }
    if (ws.empty()) break;
    out.push_back(std::move(ws));
  }
  return out;
}

}  // namespace

static int scc_batch_phases(psc_graph_s* g, uint64_t* labels, const psc_params_t* p,
                            const uint64_t* seeds) {
  const uint64_t n = g->n;
  const uint32_t G = g->num_graphs;
  const unsigned tb = 256;
  const uint32_t* gid = g->d_gid;
  uint32_t *P, *nz, *centres, *front, *vf, *vb, *flab;
  PSC_TRY(ensure_t(g, B_P, n + 1, &P));
  PSC_TRY(ensure_t(g, B_TMP32, n + 1, &nz));
  BatchArrays A;
  PSC_TRY(batch_arrays(g, &A));

  // trim over the union
  uint64_t n_zeros = 0;
  PSC_TRY(scan_emit_flags(g, n, ZeroFlag{g->off, g->in_off}, TrimEmitB{labels, nz}, &n_zeros, F_TRIM,
                          28.0));
  const uint64_t np = n - n_zeros;
  std::vector<uint64_t> npbase(G + 1), cbase(G + 1);
  {
    ProfScope ps(g, F_BATCH);
    k_bases_by_value<<<(G + 256) / 256, 256, 0, g->stream>>>(nz, np, g->d_vbase, G, A.npbase);
  }
  PSC_CUDA(cudaMemcpyAsync(npbase.data(), A.npbase, (G + 1) * 8, cudaMemcpyDeviceToHost, g->stream));
  PSC_CUDA(cudaStreamSynchronize(g->stream));
  npbase[G] = np;
  // per-graph permutation keys and first labels |ZEROS_k| + 1
  std::vector<FeistelKey> keys(G);
  std::vector<uint64_t> lo(G);
  std::vector<uint32_t> glist;
  for (uint32_t k = 0; k < G; k++) {
    const uint64_t npk = npbase[k + 1] - npbase[k];
    keys[k] = feistel_key(npk, seeds ? seeds[k] : p->seed);
    lo[k] = (g->vbase[k + 1] - g->vbase[k]) - npk + 1;
    if (npk) glist.push_back(k);
  }
  PSC_CUDA(cudaMemcpyAsync(A.keys, keys.data(), G * sizeof(FeistelKey), cudaMemcpyHostToDevice, g->stream));
  PSC_CUDA(cudaMemcpyAsync(A.lo, lo.data(), G * 8, cudaMemcpyHostToDevice, g->stream));
  if (!glist.empty())
    PSC_CUDA(cudaMemcpyAsync(A.glist, glist.data(), glist.size() * 4, cudaMemcpyHostToDevice, g->stream));
  if (np > 0) {
    ProfScope ps(g, F_TRIM);
    ps.bytes = 12.0 * np;
    k_perm_gather_b<<<grid_for(g, np, tb), tb, 0, g->stream>>>(nz, np, gid, A.npbase, A.keys, P);
  }
  PSC_CUDA(cudaEventRecord(g->ph[1], g->stream));
  if (np > 0) {
    // first pivots of all graphs, searched together
    const uint32_t ns = (uint32_t)glist.size();
    {
      ProfScope ps(g, F_BATCH);
      k_batch_sources<<<(ns + 255) / 256, 256, 0, g->stream>>>(P, A.npbase, A.glist, ns, A.srcs);
    }
    PSC_TRY(ensure_t(g, B_VIS_F, (n + 31) / 32 + 1, &vf));
    PSC_TRY(ensure_t(g, B_VIS_B, (n + 31) / 32 + 1, &vb));
    uint32_t r1 = 0, r2 = 0;
    // many small searches at once: VGC for every sparse round, so rounds
    // shrink by up to tau for the high-diameter members
    PSC_TRY(reach_pair_multi(g, A.srcs, ns, p->local_reach != 0, p->tau, p->pull_div, vf, vb, &r1,
                             &r2, kBatchVgcMax));
    g->stats.reach_rounds = r1 + r2;
    uint32_t* done;  // finished vertices after the first pivots (frontier slot, free by now)
    PSC_TRY(ensure_t(g, B_FB_A, (n + 31) / 32 + 1, &done));
    {
      ProfScope ps(g, F_LABEL_FIRST);
      ps.bytes = 0.375 * g->n + 8.0 * g->n + 12.0 * np;
      k_label_first_b<<<grid_for(g, g->n, tb), tb, 0, g->stream>>>(vf, vb, g->n, gid, A.lo, labels,
                                                                 done);
    }
    {
      ProfScope ps(g, F_BATCH);
      k_lo_first<<<(G + 255) / 256, 256, 0, g->stream>>>(A.npbase, G, A.lo);
    }
    PSC_TRY(ensure_t(g, B_CENTERS, np + 1, &centres));
    uint64_t nc = 0;
    PSC_TRY(scan_emit_flags(g, np, NotDoneBitAt{P, done}, CopyAt{P, centres, 0}, &nc, F_COMPACT, 8.0,
                      4.0));
    {
      ProfScope ps(g, F_BATCH);
      k_bases_by_graph<<<(G + 256) / 256, 256, 0, g->stream>>>(centres, nc, gid, nullptr, G, A.cbase);
    }
    PSC_CUDA(cudaMemcpyAsync(cbase.data(), A.cbase, (G + 1) * 8, cudaMemcpyDeviceToHost, g->stream));
    PSC_CUDA(cudaStreamSynchronize(g->stream));
    PSC_CUDA(cudaEventRecord(g->ph[2], g->stream));

    // the windows of every batch, uploaded once
    const auto sched = batch_schedule(cbase, G, p->beta);
    size_t words = 0;
    for (const auto& ws : sched) words += 3 * ws.size() + 1;
    uint64_t* sched_d;
    PSC_TRY(ensure_t(g, B_SCHED, words + 1, &sched_d));
    std::vector<uint64_t> hs(words);
    std::vector<size_t> at(sched.size());
    {
      size_t o = 0;
      for (size_t j = 0; j < sched.size(); j++) {
        const auto& ws = sched[j];
        const size_t c = ws.size();
        at[j] = o;
        uint32_t* wg = (uint32_t*)&hs[o];  // c u32 in ceil(c/2) words, padded to c words
        uint64_t* wstart = &hs[o + c];
        uint64_t* wpre = &hs[o + 2 * c];
        uint64_t acc = 0;
        for (size_t a = 0; a < c; a++) {
          wg[a] = ws[a].graph;
          wstart[a] = ws[a].start;
          wpre[a] = acc;
          acc += ws[a].len;
        }
        wpre[c] = acc;
        o += 3 * c + 1;
      }
    }
    if (words)
      PSC_CUDA(cudaMemcpyAsync(sched_d, hs.data(), words * 8, cudaMemcpyHostToDevice, g->stream));
    PSC_TRY(ensure_t(g, B_FRONT, np + 1, &front));
    PSC_TRY(ensure_t(g, B_FLAB, np + 1, &flab));
    uint64_t in_ne = 1, out_ne = 1;
    for (size_t j = 0; j < sched.size(); j++) {
      const uint32_t c = (uint32_t)sched[j].size();
      const uint32_t* wg = (const uint32_t*)(sched_d + at[j]);
      const uint64_t* wstart = sched_d + at[j] + c;
      const uint64_t* wpre = sched_d + at[j] + 2 * c;
      const uint64_t W = hs[at[j] + 3 * c];
      const WinNotDone wnd{centres, labels, wstart, wpre, c};
      uint64_t nf = 0;
      PSC_TRY(scan_emit_flags(g, W, wnd, WinCopy{wnd, front}, &nf, F_COMPACT, 12.0, 4.0));
      if (nf == 0) continue;
      g->stats.batches++;
      {
        ProfScope ps(g, F_BATCH);
        k_bases_by_graph<<<(c + 256) / 256, 256, 0, g->stream>>>(front, nf, gid, wg, c, A.fb);
        k_front_labels<<<grid_for(g, nf, tb), tb, 0, g->stream>>>(nf, A.fb, wg, c, A.lo, flab);
        k_lo_advance<<<(c + 255) / 256, 256, 0, g->stream>>>(A.fb, wg, c, A.lo);
      }
      MsResult res[2];
      const uint64_t prev[2] = {out_ne, in_ne};
      PSC_TRY(ms_pair(g, front, nf, 0, labels, p, prev, res, flab, kBatchVgcMax));
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
    k_finalise_b<<<grid_for(g, n, tb), tb, 0, g->stream>>>(labels, n, gid, g->d_vbase, A.npbase);
  }
  PSC_CUDA(cudaGetLastError());
  return PSC_OK;
}

int scc_batch_run(psc_graph_s* g, const psc_params_t* p, const uint64_t* seeds, uint64_t* labels) {
  g->block = p->block;
  const int st = scc_timed(g, [&](psc_graph_s* h) { return scc_batch_phases(h, labels, p, seeds); });
  g->block = 0;
  return st;
}

}  // namespace psc

using namespace psc;

namespace psc {

int batch_attach(psc_graph_s* g, const uint64_t* vbase, uint32_t num_graphs, bool check) {
  if (!g || !vbase || num_graphs == 0) return PSC_ERR_INVALID;
  if (vbase[0] != 0 || vbase[num_graphs] != g->n) return PSC_ERR_INVALID;
  for (uint32_t k = 0; k < num_graphs; k++)
    if (vbase[k + 1] < vbase[k]) return PSC_ERR_INVALID;
  PSC_CUDA(cudaSetDevice(g->device));
  if (g->d_vbase) PSC_CUDA(cudaFreeAsync(g->d_vbase, g->stream));
  if (g->d_gid) PSC_CUDA(cudaFreeAsync(g->d_gid, g->stream));
  g->d_vbase = nullptr;
  g->d_gid = nullptr;
  g->num_graphs = 0;
  g->vbase.clear();
  PSC_CUDA(cudaMallocAsync((void**)&g->d_vbase, ((size_t)num_graphs + 1) * 8, g->stream));
  PSC_CUDA(cudaMallocAsync((void**)&g->d_gid, g->n * 4, g->stream));
  PSC_CUDA(cudaMemcpyAsync(g->d_vbase, vbase, ((size_t)num_graphs + 1) * 8, cudaMemcpyHostToDevice,
                           g->stream));
  k_fill_gid<<<grid_for(g, g->n, 256), 256, 0, g->stream>>>(g->d_vbase, num_graphs, g->n, g->d_gid);
  PSC_CUDA(cudaGetLastError());
  if (check) {
    uint64_t* eb;
    PSC_TRY(ensure_t(g, B_GRAPHS, 2 * ((size_t)num_graphs + 1), &eb));
    PSC_CUDA(cudaMemsetAsync(&g->ctr->aux0, 0, 8, g->stream));
    k_graph_edge_bases<<<(num_graphs + 256) / 256, 256, 0, g->stream>>>(
        g->off, g->in_off, g->d_vbase, num_graphs, eb, eb + num_graphs + 1);
    const unsigned cg = grid_for(g, (g->m + kCheckChunk - 1) / kCheckChunk * 32, 256);
    k_check_batch_edges<<<cg, 256, 0, g->stream>>>(g->E, g->m, eb, g->d_vbase, num_graphs,
                                                  &g->ctr->aux0);
    if (g->in_E != g->E)
      k_check_batch_edges<<<cg, 256, 0, g->stream>>>(g->in_E, g->m, eb + num_graphs + 1,
                                                    g->d_vbase, num_graphs, &g->ctr->aux0);
    PSC_CUDA(cudaGetLastError());
    PSC_CUDA(cudaMemcpyAsync(&g->hctr->aux0, &g->ctr->aux0, 8, cudaMemcpyDeviceToHost, g->stream));
    PSC_CUDA(cudaStreamSynchronize(g->stream));
    if (g->hctr->aux0 != 0) {
      cudaFreeAsync(g->d_vbase, g->stream);
      cudaFreeAsync(g->d_gid, g->stream);
      g->d_vbase = nullptr;
      g->d_gid = nullptr;
      return PSC_ERR_INVALID;  // an edge crosses two graphs
    }
  }
  g->vbase.assign(vbase, vbase + num_graphs + 1);
  g->num_graphs = num_graphs;
  return PSC_OK;
}

}  // namespace psc

extern "C" int psc_batch_set(psc_graph_t g, const uint64_t* vbase, uint32_t num_graphs) {
  return batch_attach(g, vbase, num_graphs, true);
}

extern "C" uint32_t psc_batch_num_graphs(psc_graph_t g) { return g ? g->num_graphs : 0; }

extern "C" int psc_scc_batch_device(psc_graph_t g, const psc_params_t* p, const uint64_t* seeds,
                                    uint64_t* d_labels) {
  if (!g || !d_labels || g->num_graphs == 0) return PSC_ERR_INVALID;
  psc_params_t def;
  if (!p) {
    psc_params_default(&def);
    p = &def;
  }
  if (!(p->beta > 0)) return PSC_ERR_INVALID;
  PSC_TRY(call_begin(g));
  PSC_TRY(scc_batch_run(g, p, seeds, d_labels));
  return call_end(g);
}

extern "C" int psc_scc_batch(psc_graph_t g, const psc_params_t* p, const uint64_t* seeds,
                             uint64_t* labels_out) {
  if (!g || !labels_out || g->num_graphs == 0) return PSC_ERR_INVALID;
  psc_params_t def;
  if (!p) {
    psc_params_default(&def);
    p = &def;
  }
  if (!(p->beta > 0)) return PSC_ERR_INVALID;
  PSC_TRY(call_begin(g));
  uint64_t* d;
  PSC_TRY(ensure_t(g, B_LABELS, g->n, &d));
  PSC_TRY(scc_batch_run(g, p, seeds, d));
  PSC_CUDA(cudaMemcpyAsync(labels_out, d, g->n * 8, cudaMemcpyDeviceToHost, g->stream));
  return call_end(g);
}

namespace psc {

int cc_batch_run(psc_graph_s* g, double beta, uint32_t* d_labels) {
  PSC_TRY(cc_run(g, beta, d_labels, nullptr, nullptr));
  {
    ProfScope ps(g, F_BATCH);
    ps.bytes = 12.0 * g->n;
    k_localise_u32<<<grid_for(g, g->n, 256), 256, 0, g->stream>>>(d_labels, g->n, g->d_gid,
                                                                 g->d_vbase);
  }
  PSC_CUDA(cudaGetLastError());
  return PSC_OK;
}

}  // namespace psc

extern "C" int psc_cc_batch(psc_graph_t g, double beta, uint32_t* labels_out) {
  if (!g || !labels_out || !(beta > 0) || g->num_graphs == 0) return PSC_ERR_INVALID;
  PSC_TRY(call_begin(g));
  uint32_t* d;
  PSC_TRY(ensure_t(g, B_AUX0, g->n + 1, &d));
  PSC_TRY(cc_batch_run(g, beta, d));
  PSC_CUDA(cudaMemcpyAsync(labels_out, d, g->n * 4, cudaMemcpyDeviceToHost, g->stream));
  return call_end(g);
}

// Multi-search on the device (SCC::multi_search / multi_search_safe,
// src/scc.hpp:144-275), forward and backward in the same launches.
//
// Per direction ("side") the state is the closure table {(v, pivot)} — 64-bit
// keys v<<32 | pivot label in an open-addressing table with linear probing
// and atomicCAS inserts (the reference's resizable_table, keyed here by the
// hash of the whole pair) — and a frontier of pairs that are new to the table.
// A sub-round offers each frontier pair (u, l) to every out-neighbour w of u
// inside u's subproblem (labels[w] == labels[u]); new pairs form the next
// frontier, so each pair is expanded once.  The closure, and therefore the
// partition, is the reference's.
//
//   VGC (scc.hpp:177-219): while a side's frontier is small, one pair per
//     warp runs a local BFS for its pivot in a shared-memory queue (entries
//     carry the vertex's adjacency range, loaded alongside the claim), up to
//     tau vertices, spilling the rest as pairs;
//   expand: larger frontiers, 32 pairs per warp step with the balanced
//     expansion;
//   heavy: pairs of vertices with more than kHeavyDeg out-edges, expanded by
//     the whole grid.
// Claims are batched: a lane loads K target ids, then their labels (and in
// VGC their adjacency ranges), then issues the first table probes, so the
// memory round trips of K edges overlap.
//
// Table growth: the host keeps the load at most 1/2 between sub-rounds.  An
// insert that still gives up (kProbeLimit probes) re-queues its source pair;
// the host grows the table before the next sub-round and the pair is expanded
// again, finding the pairs it already placed.  This replaces the reference's
// restart of the whole search (scc.hpp:263-272) with the same fixed point.
#include <algorithm>
#include <cstdio>

#include "common.cuh"
#include "engines.cuh"

namespace psc {

constexpr int kMsBlock = 256;
constexpr int kMsVgcBlock = 128;
constexpr int kMsVgcQueue = 512;
constexpr int kMsK = 8;        // VGC: edges in flight per lane
constexpr int kMsExpandK = 4;  // expand: fewer registers, more warps
constexpr uint32_t kProbeLimit = 256;

struct MsSide {
  const uint64_t* off;
  const uint32_t* E;
  const uint64_t* Fin;  // frontier pairs
  uint64_t nin;
  unsigned long long* T;
  uint64_t mask;
  uint64_t* Fout;
  uint64_t* Fheavy;
  uint32_t* hflag;
  Counters* ctr;
  uint32_t vgc_budget;  // new pairs one VGC local search may insert
  // when set, the frontier size is read here instead of nin (the first
  // sub-round of a batch started without waiting for its pivot count)
  const unsigned long long* nin_dev;
};

constexpr int kMsHeavyK = 4;  // heavy pairs: edges in flight per lane
constexpr uint64_t kMsHeavyChunk = 32 * kMsHeavyK;
constexpr uint32_t kRequeued = 0x80000000u;  // hflag bit: the pair was re-queued

// Lists a pair whose vertex has more than kHeavyDeg out-edges for k_ms_heavy.
// Its edges are cut into chunks of kMsHeavyChunk; one 64-bit atomic on
// ctr->heavy = count << kPackShift | chunks gives the pair its slot and its
// first chunk (hflag, below the kRequeued bit), increasing with the slot.
__device__ __forceinline__ void ms_heavy_push(const MsSide& S, uint64_t key, uint64_t deg) {
  const unsigned long long old = atomicAdd(
      &S.ctr->heavy, (1ull << kPackShift) + (deg + kMsHeavyChunk - 1) / kMsHeavyChunk);
  const uint64_t hh = old >> kPackShift;
  S.Fheavy[hh] = key;
  S.hflag[hh] = (uint32_t)(old & kPackMask);
}

// Per-warp source data of one expansion step.
struct MsSrc {
  uint64_t sub[32];
  uint32_t lab[32];
  uint32_t fail;
};

// Seeds both sides of a batch: pair (front[i], label) into each side's table
// and frontier.
__global__ void k_ms_seed(const uint32_t* __restrict__ front, uint64_t nf, uint64_t label_offset,
                          const uint32_t* __restrict__ front_labels, unsigned long long* T0,
                          uint64_t mask0, uint64_t* F0, unsigned long long* T1, uint64_t mask1,
                          uint64_t* F1, const unsigned long long* nf_dev) {
  if (nf_dev) nf = *nf_dev;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nf;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t lab = front_labels ? front_labels[i] : (uint32_t)(label_offset + i);
    const uint64_t key = ((uint64_t)front[i] << 32) | (uint64_t)lab;
    uint32_t pr = 0;
    table_insert(T0, mask0, key, (uint32_t)(mask0 + 1 < 0xFFFFFFFFull ? mask0 + 1 : 0xFFFFFFFFu), &pr);
    table_insert(T1, mask1, key, (uint32_t)(mask1 + 1 < 0xFFFFFFFFull ? mask1 + 1 : 0xFFFFFFFFu), &pr);
    F0[i] = key;
    F1[i] = key;
  }
}

__global__ void k_rehash(const unsigned long long* __restrict__ T, uint64_t cap,
                         unsigned long long* T2, uint64_t mask2) {
  uint32_t pr = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t e = T[i];
    if (e != kEmpty) table_insert(T2, mask2, e, 0xFFFFFFFFu, &pr);
  }
}

// Linear probing from slot h (the first probe is already done by the caller).
__device__ __forceinline__ int table_insert_from(unsigned long long* T, uint64_t mask, uint64_t key,
                                                 uint64_t h, uint32_t limit, uint32_t* probes) {
  for (uint32_t i = 0; i < limit; i++) {
    h = (h + 1) & mask;
    uint64_t cur = __ldcg(&T[h]);
    if (cur == key) {
      *probes += i + 1;
      return 0;
    }
    if (cur == kEmpty) {
      uint64_t old = atomicCAS(&T[h], (unsigned long long)kEmpty, (unsigned long long)key);
      if (old == kEmpty) {
        *probes += i + 1;
        return 1;
      }
      if (old == key) {
        *probes += i + 1;
        return 0;
      }
    }
  }
  *probes += limit;
  return -1;
}

// Batched claim over the 32 lanes' adjacency ranges (K edges per lane in
// flight).  A candidate w of source lane s is offered pivot src.lab[s] if
// labels[w] == src.sub[s].  DIRECT: the first probe is an atomicCAS (one
// round trip, for latency-bound rounds); otherwise a load, then a CAS only on
// an empty slot.  PF: also load w's adjacency range.  A failed insert sets bit
// s of src.fail.  emit(tm, keys) gets the lane's K candidate pairs and the mask
// of those newly inserted (warp-collective).
template <int K, bool DIRECT, bool PF, class Emit>
__device__ __forceinline__ void ms_expand_claim(WarpExpandSmem& sm, MsSrc& src, uint64_t beg,
                                                uint32_t deg, const uint64_t* __restrict__ off,
                                                const uint32_t* __restrict__ E,
                                                const uint64_t* __restrict__ labels,
                                                unsigned long long* T, uint64_t mask,
                                                uint32_t& probes, Emit&& emit) {
  const unsigned lane = lane_id();
  uint32_t incl = deg;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(kFull, incl, o);
    if ((int)lane >= o) incl += t;
  }
  const uint32_t total = __shfl_sync(kFull, incl, 31);
  sm.excl[lane] = incl - deg;
  sm.beg[lane] = beg;
  __syncwarp();
  for (uint32_t base = 0; base < total; base += 32 * K) {
    uint32_t w[K];
    int sl[K];
    uint64_t key[K], old[K], h[K], vb[K], ve[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      const uint32_t gi = base + k * 32 + lane;
      w[k] = 0xFFFFFFFFu;
      sl[k] = 0;
      if (gi < total) {
        int lo = 0, hi = 31;
        while (lo < hi) {
          int mid = (lo + hi + 1) >> 1;
          if (sm.excl[mid] <= gi)
            lo = mid;
          else
            hi = mid - 1;
        }
        sl[k] = lo;
        w[k] = __ldg(&E[sm.beg[lo] + (gi - sm.excl[lo])]);
      }
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
      key[k] = kEmpty;
      vb[k] = ve[k] = 0;
      if (w[k] != 0xFFFFFFFFu) {
        const uint64_t lw = __ldg(&labels[w[k]]);
        if (PF) {
          vb[k] = __ldg(&off[w[k]]);
          ve[k] = __ldg(&off[w[k] + 1]);
        }
        if (lw == src.sub[sl[k]]) key[k] = ((uint64_t)w[k] << 32) | src.lab[sl[k]];
      }
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
      old[k] = kEmpty;
      h[k] = 0;
      if (key[k] != kEmpty) {
        h[k] = hash64(key[k]) & mask;
        if (DIRECT)
          old[k] = atomicCAS(&T[h[k]], (unsigned long long)kEmpty, (unsigned long long)key[k]);
        else
          old[k] = __ldcg(&T[h[k]]);
      }
    }
    uint32_t tm = 0;
#pragma unroll
    for (int k = 0; k < K; k++) {
      if (key[k] != kEmpty) {
        int r;
        probes++;
        if (DIRECT) {
          r = old[k] == kEmpty ? 1 : old[k] == key[k] ? 0
                                  : table_insert_from(T, mask, key[k], h[k], kProbeLimit - 1, &probes);
        } else if (old[k] == key[k]) {
          r = 0;
        } else if (old[k] == kEmpty) {
          const uint64_t o2 =
              atomicCAS(&T[h[k]], (unsigned long long)kEmpty, (unsigned long long)key[k]);
          r = o2 == kEmpty ? 1 : o2 == key[k] ? 0
                             : table_insert_from(T, mask, key[k], h[k], kProbeLimit - 1, &probes);
        } else {
          r = table_insert_from(T, mask, key[k], h[k], kProbeLimit - 1, &probes);
        }
        if (r == 1) tm |= 1u << k;
        if (r < 0) atomicOr(&src.fail, 1u << sl[k]);
      }
    }
    emit(tm, key);
  }
  __syncwarp();
}

__device__ __forceinline__ void flush_ms_counters(Counters* c0, Counters* c1,
                                                  unsigned long long s0, unsigned long long s1,
                                                  unsigned long long r0, unsigned long long r1,
                                                  unsigned long long p0, unsigned long long p1,
                                                  unsigned long long x0, unsigned long long x1,
                                                  unsigned long long i0, unsigned long long i1) {
  i0 = warp_sum(i0);
  i1 = warp_sum(i1);
  if (lane_id() == 0) {
    if (i0) atomicAdd(&c0->inserted, i0);
    if (i1) atomicAdd(&c1->inserted, i1);
  }
  s0 = warp_sum(s0);
  s1 = warp_sum(s1);
  r0 = warp_sum(r0);
  r1 = warp_sum(r1);
  p0 = warp_sum(p0);
  p1 = warp_sum(p1);
  x0 = warp_sum(x0);
  x1 = warp_sum(x1);
  if (lane_id() == 0) {
    if (s0 | r0 | p0 | x0) {
      atomicAdd(&c0->edges, s0);
      atomicAdd(&c0->probes, p0);
      atomicAdd(&c0->expanded, x0);
      if (r0) {
        atomicAdd(&c0->fail, r0);
        atomicAdd(&c0->aux1, r0);
      }
    }
    if (s1 | r1 | p1 | x1) {
      atomicAdd(&c1->edges, s1);
      atomicAdd(&c1->probes, p1);
      atomicAdd(&c1->expanded, x1);
      if (r1) {
        atomicAdd(&c1->fail, r1);
        atomicAdd(&c1->aux1, r1);
      }
    }
  }
}

// Expansion sub-round for up to two sides: 32 pairs per warp step.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK, (768 / BLOCK) > 0 ? (768 / BLOCK) : 1)
    k_ms_expand(MsSide s0, MsSide s1, const uint64_t* __restrict__ labels) {
  if (s0.nin_dev) s0.nin = *s0.nin_dev;
  if (s1.nin_dev) s1.nin = *s1.nin_dev;
  __shared__ WarpExpandSmem sm[BLOCK / 32];
  __shared__ MsSrc ssrc[BLOCK / 32];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  const uint64_t c0 = (s0.nin + 31) / 32, c1 = (s1.nin + 31) / 32;
  MsSrc& src = ssrc[wid];
  unsigned long long sc0 = 0, sc1 = 0, rq0 = 0, rq1 = 0, ex0 = 0, ex1 = 0, in0 = 0, in1 = 0;
  uint32_t pr0 = 0, pr1 = 0;
  for (uint64_t c = gw; c < c0 + c1; c += nw) {
    const int sd = c < c0 ? 0 : 1;
    const MsSide S = sd ? s1 : s0;
    const uint64_t i = (sd ? c - c0 : c) * 32 + lane;
    uint64_t beg = 0, key = 0, sub = 0;
    uint32_t deg = 0;
    if (i < S.nin) {
      key = S.Fin[i];
      const uint32_t u = (uint32_t)(key >> 32);
      beg = S.off[u];
      uint64_t d = S.off[u + 1] - beg;
      sub = labels[u];
      (sd ? ex1 : ex0)++;
      if (d > kHeavyDeg) {
        ms_heavy_push(S, key, d);
        d = 0;
      }
      deg = (uint32_t)d;
    }
    (sd ? sc1 : sc0) += deg;
    src.sub[lane] = sub;
    src.lab[lane] = (uint32_t)key;
    if (lane == 0) src.fail = 0;
    __syncwarp();
    uint32_t probes = 0;
    ms_expand_claim<kMsExpandK, false, false>(
        sm[wid], src, beg, deg, S.off, S.E, labels, S.T, S.mask, probes,
        [&](uint32_t tm, const uint64_t* keys) {
          (sd ? in1 : in0) += __popc(tm);
          warp_append_batch<kMsExpandK>(tm, keys, S.Fout, &S.ctr->next);
        });
    (sd ? pr1 : pr0) += probes;
    __syncwarp();
    const bool rq = (src.fail >> lane) & 1u;
    unsigned long long pos = warp_append(&S.ctr->next, rq);
    if (rq) {
      S.Fout[pos] = key;
      (sd ? rq1 : rq0)++;
    }
    __syncwarp();
  }
  flush_ms_counters(s0.ctr, s1.ctr, sc0, sc1, rq0, rq1, pr0, pr1, ex0, ex1, in0, in1);
}

struct MsQEnt {
  uint64_t beg;
  uint32_t v;
  uint32_t deg;
};

// Claims of one batch for pivot lab inside subproblem sub: each candidate's
// label and adjacency range are loaded together, then the first table probes
// (atomicCAS) of all K candidates are issued before any is resolved.  Returns
// the mask of new pairs; sets *failed if an insert gave up.
template <int K, bool ADJ = true>
__device__ __forceinline__ uint32_t ms_vgc_claim(const uint32_t* w, uint64_t* vb, uint64_t* ve,
                                                 uint64_t sub, uint32_t lab,
                                                 const uint64_t* __restrict__ off,
                                                 const uint64_t* __restrict__ labels,
                                                 unsigned long long* T, uint64_t mask,
                                                 uint32_t& probes, bool& failed) {
  uint64_t key[K], old[K], h[K];
#pragma unroll
  for (int k = 0; k < K; k++) {
    key[k] = kEmpty;
    vb[k] = ve[k] = 0;
    if (w[k] != 0xFFFFFFFFu) {
      const uint64_t lw = __ldg(&labels[w[k]]);
      if (ADJ) {
        vb[k] = __ldg(&off[w[k]]);
        ve[k] = __ldg(&off[w[k] + 1]);
      }
      if (lw == sub) key[k] = ((uint64_t)w[k] << 32) | lab;
    }
  }
#pragma unroll
  for (int k = 0; k < K; k++) {
    old[k] = kEmpty;
    h[k] = 0;
    if (key[k] != kEmpty) {
      h[k] = hash64(key[k]) & mask;
      old[k] = atomicCAS(&T[h[k]], (unsigned long long)kEmpty, (unsigned long long)key[k]);
    }
  }
  uint32_t tm = 0;
#pragma unroll
  for (int k = 0; k < K; k++)
    if (key[k] != kEmpty) {
      probes++;
      const int r = old[k] == kEmpty ? 1 : old[k] == key[k] ? 0
                    : table_insert_from(T, mask, key[k], h[k], kProbeLimit - 1, &probes);
      if (r == 1) tm |= 1u << k;
      failed |= r < 0;
    }
  return tm;
}

// Places this lane's new pairs (bit k of tm) into the warp's queue while it
// has room, then spills (w, lab) pairs: one warp scan, at most one atomic.
template <int K>
__device__ __forceinline__ void ms_vgc_place(uint32_t tm, const uint32_t* w, const uint64_t* vb,
                                             const uint64_t* ve, uint32_t lab, MsQEnt* Q,
                                             uint32_t& tail, uint32_t tq, uint64_t* Fout,
                                             unsigned long long* next_ctr) {
  const unsigned lane = lane_id();
  const uint32_t cnt = __popc(tm);
  uint32_t incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(kFull, incl, o);
    if ((int)lane >= o) incl += t;
  }
  const uint32_t total = __shfl_sync(kFull, incl, 31);
  if (total == 0) return;
  const uint32_t room = tq - tail;
  const uint32_t nloc = total < room ? total : room;
  unsigned long long sbase = 0;
  if (total > nloc && lane == 0) sbase = atomicAdd(next_ctr, (unsigned long long)(total - nloc));
  sbase = __shfl_sync(kFull, sbase, 0);
  uint32_t r = incl - cnt;
#pragma unroll
  for (int k = 0; k < K; k++)
    if (tm & (1u << k)) {
      if (r < nloc) {
        const uint64_t vd = ve[k] - vb[k];
        Q[tail + r] = MsQEnt{vb[k], w[k], (uint32_t)(vd < 0xFFFFFFFFull ? vd : 0xFFFFFFFFull)};
      } else {
        Fout[sbase + (r - nloc)] = ((uint64_t)w[k] << 32) | lab;
      }
      r++;
    }
  tail += nloc;
  __syncwarp();
}

// VGC sub-round for up to two sides: one frontier pair (u, l) per warp.  If
// 0 < deg(u) < tau the warp runs a local BFS for pivot l inside u's
// subproblem in a shared-memory queue of tq = min(tau, QCAP) vertices: each
// wave offers l along the edges of up to 32 queued vertices (one vertex per
// lane when their degrees are at most K, else the balanced expansion); a new
// pair stays in the queue while there is room, else spills to the next
// frontier.  Queued vertices with more than tq out-edges and the queue's
// remainder spill too.  A queued vertex whose expansion hit a failed insert is
// re-queued as a pair.
template <int BLOCK, int QCAP>
__global__ void __launch_bounds__(BLOCK)
    k_ms_vgc(MsSide s0, MsSide s1, const uint64_t* __restrict__ labels, uint32_t tau) {
  if (s0.nin_dev) s0.nin = *s0.nin_dev;
  if (s1.nin_dev) s1.nin = *s1.nin_dev;
  __shared__ WarpExpandSmem sm[BLOCK / 32];
  __shared__ MsQEnt sq[BLOCK / 32][QCAP];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  const uint32_t tq = tau < (uint32_t)QCAP ? tau : (uint32_t)QCAP;
  MsQEnt* Q = sq[wid];
  unsigned long long sc0 = 0, sc1 = 0, rq0 = 0, rq1 = 0, ex0 = 0, ex1 = 0, in0 = 0, in1 = 0;
  uint32_t pr0 = 0, pr1 = 0;
  if (lane == 0) sm[wid].fail = 0;
  __syncwarp();
  for (uint64_t i = gw; i < s0.nin + s1.nin; i += nw) {
    const int sd = i < s0.nin ? 0 : 1;
    const MsSide S = sd ? s1 : s0;
    const uint64_t key = S.Fin[sd ? i - s0.nin : i];
    const uint32_t u = (uint32_t)(key >> 32);
    const uint32_t lab = (uint32_t)key;
    const uint64_t sub = labels[u];
    const uint64_t ub = S.off[u], ue = S.off[u + 1];
    const uint64_t du = ue - ub;
    auto emit = [&](bool take, uint32_t w) {
      unsigned long long pos = warp_append(&S.ctr->next, take);
      if (take) S.Fout[pos] = ((uint64_t)w << 32) | lab;
    };
    if (lane == 0) (sd ? ex1 : ex0)++;
    uint32_t probes = 0;
    if (!(du > 0 && du < tq)) {
      if (du > kHeavyDeg) {
        if (lane == 0) ms_heavy_push(S, key, du);
        continue;
      }
      // a vertex with tau..kHeavyDeg out-edges: the warp walks them with
      // kMsK edges per lane in flight
      if (lane == 0) (sd ? sc1 : sc0) += du;
      bool failed = false;
      for (uint64_t b = ub; b < ue; b += 32 * kMsK) {
        uint32_t w[kMsK];
        uint64_t vb[kMsK], ve[kMsK], keys[kMsK];
#pragma unroll
        for (int k = 0; k < kMsK; k++) {
          const uint64_t e = b + k * 32 + lane;
          w[k] = e < ue ? __ldg(&S.E[e]) : 0xFFFFFFFFu;
        }
        bool fk = false;
        const uint32_t tm = ms_vgc_claim<kMsK, false>(w, vb, ve, sub, lab, S.off, labels, S.T,
                                                      S.mask, probes, fk);
        failed |= fk;
        (sd ? in1 : in0) += __popc(tm);
#pragma unroll
        for (int k = 0; k < kMsK; k++) keys[k] = ((uint64_t)w[k] << 32) | lab;
        warp_append_batch<kMsK>(tm, keys, S.Fout, &S.ctr->next);
      }
      (sd ? pr1 : pr0) += probes;
      const bool rq = __any_sync(kFull, failed) && lane == 0;
      emit(rq, u);
      if (rq) (sd ? rq1 : rq0)++;
      continue;
    }
    if (lane == 0) Q[0] = MsQEnt{ub, u, (uint32_t)du};
    __syncwarp();
    // the local search stops at tq queued vertices, or once it has inserted
    // its share of the table's free room (the first wave always runs)
    uint32_t head = 0, tail = 1, ins = 0;
    while (head < tail && tail < tq && (head == 0 || ins < S.vgc_budget)) {
      const uint32_t wave = min(32u, tail - head);
      uint64_t beg = 0;
      uint32_t deg = 0, x = 0;
      bool spill_self = false;
      if (lane < wave) {
        const MsQEnt q = Q[head + lane];
        x = q.v;
        beg = q.beg;
        deg = q.deg;
        if (deg > tq) {
          spill_self = true;
          deg = 0;
        }
        if (lane > 0 || head > 0) (sd ? ex1 : ex0)++;
      }
      head += wave;
      __syncwarp();
      if (__any_sync(kFull, spill_self)) emit(spill_self, x);
      (sd ? sc1 : sc0) += deg;
      bool failed = false;
      uint32_t incl = deg;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, o);
        if ((int)lane >= o) incl += t;
      }
      const uint32_t total = __shfl_sync(kFull, incl, 31);
      sm[wid].excl[lane] = incl - deg;
      sm[wid].beg[lane] = beg;
      __syncwarp();
      for (uint32_t base = 0; base < total; base += 32 * kMsK) {
        uint32_t w[kMsK];
        int sl[kMsK];
        uint64_t vb[kMsK], ve[kMsK];
#pragma unroll
        for (int k = 0; k < kMsK; k++) {
          const uint32_t gi = base + k * 32 + lane;
          w[k] = 0xFFFFFFFFu;
          sl[k] = 0;
          if (gi < total) {
            int lo = 0, hi = 31;
            while (lo < hi) {
              int mid = (lo + hi + 1) >> 1;
              if (sm[wid].excl[mid] <= gi)
                lo = mid;
              else
                hi = mid - 1;
            }
            sl[k] = lo;
            w[k] = __ldg(&S.E[sm[wid].beg[lo] + (gi - sm[wid].excl[lo])]);
          }
        }
        bool fk = false;
        const uint32_t tm = ms_vgc_claim<kMsK>(w, vb, ve, sub, lab, S.off, labels, S.T, S.mask,
                                               probes, fk);
        // a failure is charged to the source lane of the failed edge
        if (fk) {
#pragma unroll
          for (int k = 0; k < kMsK; k++)
            if (w[k] != 0xFFFFFFFFu) atomicOr(&sm[wid].fail, 1u << sl[k]);
        }
        (sd ? in1 : in0) += __popc(tm);
        ins += __reduce_add_sync(kFull, (unsigned)__popc(tm));
        ms_vgc_place<kMsK>(tm, w, vb, ve, lab, Q, tail, tq, S.Fout, &S.ctr->next);
      }
      __syncwarp();
      failed = (sm[wid].fail >> lane) & 1u;
      __syncwarp();
      if (lane == 0) sm[wid].fail = 0;
      __syncwarp();
      (sd ? pr1 : pr0) += probes;
      probes = 0;
      const bool rq = failed && lane < wave;
      if (__any_sync(kFull, rq)) {
        emit(rq, x);
        if (rq) (sd ? rq1 : rq0)++;
      }
    }
    // spill what is left in the queue with one reservation
    const uint32_t rem = tail - head;
    if (rem) {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(&S.ctr->next, (unsigned long long)rem);
      base = __shfl_sync(kFull, base, 0);
      for (uint32_t k = lane; k < rem; k += 32)
        S.Fout[base + k] = ((uint64_t)Q[head + k].v << 32) | lab;
    }
    __syncwarp();
  }
  flush_ms_counters(s0.ctr, s1.ctr, sc0, sc1, rq0, rq1, pr0, pr1, ex0, ex1, in0, in1);
}

// Heavy pairs of both sides: the chunks of a side's heavy list are cut into
// one contiguous range per warp; a warp finds the pair of its first chunk
// once, then offers kMsHeavyChunk edges per step (a heavy pair has more than
// 64 chunks, so the next pair is at most one step away).  A step with a
// failed insert re-queues its pair once (kRequeued), whichever warp failed
// first.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    k_ms_heavy(MsSide s0, MsSide s1, const uint64_t* __restrict__ labels) {
  constexpr int K = kMsHeavyK;
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
#pragma unroll 1
  for (int sd = 0; sd < 2; sd++) {
    const MsSide S = sd ? s1 : s0;
    if (!S.ctr) continue;
    const unsigned long long packed = S.ctr->heavy;
    const uint64_t nh = packed >> kPackShift, total = packed & kPackMask;
    const uint64_t per = (total + nw - 1) / nw;
    const uint64_t c_beg = gw * per, c_end = c_beg + per < total ? c_beg + per : total;
    if (nh == 0 || c_beg >= c_end) continue;
    // first chunks: hflag below the kRequeued bit (fixed while other warps set that bit)
    auto first_chunk = [&](uint64_t i) -> uint64_t { return S.hflag[i] & ~kRequeued; };
    uint64_t h = 0, hi = nh - 1;  // last pair whose first chunk is <= c_beg
    while (h < hi) {
      const uint64_t mid = (h + hi + 1) >> 1;
      if (first_chunk(mid) <= c_beg)
        h = mid;
      else
        hi = mid - 1;
    }
    uint64_t key = S.Fheavy[h], cs = first_chunk(h), cn = h + 1 < nh ? first_chunk(h + 1) : total;
    uint64_t sub = labels[key >> 32], beg = S.off[key >> 32], end = S.off[(key >> 32) + 1];
    unsigned long long scanned = 0, requeued = 0, ins = 0;
    uint32_t probes = 0;
    for (uint64_t c = c_beg; c < c_end; c++) {
      if (c >= cn) {
        h++;
        key = S.Fheavy[h];
        cs = cn;
        cn = h + 1 < nh ? first_chunk(h + 1) : total;
        sub = labels[key >> 32];
        beg = S.off[key >> 32];
        end = S.off[(key >> 32) + 1];
      }
      const uint64_t e0 = beg + (c - cs) * kMsHeavyChunk;
      const uint32_t lab = (uint32_t)key;
      uint32_t w[K];
#pragma unroll
      for (int k = 0; k < K; k++) {
        const uint64_t e = e0 + k * 32 + lane;
        w[k] = 0xFFFFFFFFu;
        if (e < end) {
          scanned++;
          w[k] = __ldg(&S.E[e]);
        }
      }
      uint64_t nk[K];
      uint32_t tm = 0;
      bool failed = false;
#pragma unroll
      for (int k = 0; k < K; k++) {
        nk[k] = 0;
        if (w[k] != 0xFFFFFFFFu && __ldg(&labels[w[k]]) == sub) {
          nk[k] = ((uint64_t)w[k] << 32) | lab;
          const int r = table_insert(S.T, S.mask, nk[k], kProbeLimit, &probes);
          if (r == 1) tm |= 1u << k;
          failed |= r < 0;
        }
      }
      ins += __popc(tm);
      warp_append_batch<K>(tm, nk, S.Fout, &S.ctr->next);
      bool rq = false;
      if (__any_sync(kFull, failed) && lane == 0)
        rq = !(atomicOr(&S.hflag[h], kRequeued) & kRequeued);
      const unsigned long long pos = warp_append(&S.ctr->next, rq);
      if (rq) {
        S.Fout[pos] = key;
        requeued++;
      }
    }
    scanned = warp_sum(scanned);
    requeued = warp_sum(requeued);
    ins = warp_sum(ins);
    const unsigned long long pr = warp_sum((unsigned long long)probes);
    if (lane == 0) {
      if (ins) atomicAdd(&S.ctr->inserted, ins);
      if (scanned) atomicAdd(&S.ctr->heavy_edges, scanned);
      if (pr) atomicAdd(&S.ctr->heavy_probes, pr);
      if (requeued) {
        atomicAdd(&S.ctr->fail, requeued);
        atomicAdd(&S.ctr->aux1, requeued);
      }
    }
  }
}

static uint64_t pow2_at_least(uint64_t x) {
  uint64_t c = 1;
  while (c < x) c <<= 1;
  return c;
}

// Rehash the table in slot tslot into a new table of capacity cap2.
static int ms_grow(psc_graph_s* g, int tslot, uint64_t cap, uint64_t cap2) {
  cudaEvent_t ea = take_event(g), eb = take_event(g);
  PSC_CUDA(cudaEventRecord(ea, g->stream));
  unsigned long long *T, *T2;
  T = (unsigned long long*)g->bufs[tslot].p;
  PSC_TRY(ensure_t(g, B_TS, cap2, &T2));
  PSC_CUDA(cudaMemsetAsync(T2, 0xFF, cap2 * 8, g->stream));
  {
    ProfScope ps(g, F_TABLE);
    ps.bytes = 8.0 * cap + 8.0 * cap2;
    k_rehash<<<grid_for(g, cap, 256), 256, 0, g->stream>>>(T, cap, T2, cap2 - 1);
  }
  PSC_CUDA(cudaGetLastError());
  swap_bufs(g, tslot, B_TS);
  g->stats.table_grows++;
  PSC_CUDA(cudaEventRecord(eb, g->stream));
  g->grow_events.emplace_back(ea, eb);
  return PSC_OK;
}

namespace {

struct MsState {
  bool backward;
  int t_slot, a_slot, b_slot, h_slot, f_slot, cset;
  uint64_t cap = 0, ne = 0, nf = 0;
  bool grow = false;
};

MsSide ms_args(psc_graph_s* g, const MsState& s) {
  MsSide r;
  r.off = s.backward ? g->in_off : g->off;
  r.E = s.backward ? g->in_E : g->E;
  r.Fin = (const uint64_t*)g->bufs[s.a_slot].p;
  r.nin = s.nf;
  r.T = (unsigned long long*)g->bufs[s.t_slot].p;
  r.mask = s.cap - 1;
  r.Fout = (uint64_t*)g->bufs[s.b_slot].p;
  r.Fheavy = (uint64_t*)g->bufs[s.h_slot].p;
  r.hflag = (uint32_t*)g->bufs[s.f_slot].p;
  r.ctr = g->ctr + s.cset;
  r.nin_dev = nullptr;
  // VGC local searches share the room left below half load, so one
  // sub-round cannot fill the table
  const uint64_t room = s.cap / 2 > s.ne ? s.cap / 2 - s.ne : 0;
  const uint64_t share = room / (s.nf ? s.nf : 1);
  r.vgc_budget = (uint32_t)(share < 0xFFFFFFFFull ? share : 0xFFFFFFFFull);
  return r;
}

}  // namespace

int ms_pair(psc_graph_s* g, const uint32_t* front, uint64_t n_front, uint64_t label_offset,
            const uint64_t* labels, const psc_params_t* p, const uint64_t prev_ne[2],
            MsResult out[2], const uint32_t* front_labels, uint64_t vgc_max, MsAsync* async) {
  // heavy-list fields: < 2^24 pairs (m / kHeavyDeg), first chunks < 2^31
  if (g->m >> 36) return PSC_ERR_TOO_LARGE;
  const uint32_t tau = p->tau ? p->tau : 512;
  const bool local = p->local_scc != 0;
  const uint64_t vgc_limit = vgc_max ? vgc_max : (uint64_t)g->num_sms * 32;
  MsState st[2];
  st[0] = MsState{false, B_TF, B_PA, B_PB, B_PH, B_AUX1, 0};
  st[1] = MsState{true, B_TB, B_PA2, B_PB2, B_PH2, B_HF2, 1};
  for (int k = 0; k < 2; k++) {
    MsState& s = st[k];
    const uint64_t want0 = (local && n_front <= vgc_limit) ? n_front * std::min<uint32_t>(tau, 64) : 0;
    s.cap = pow2_at_least(std::max<uint64_t>(
        {4096, 4 * n_front, 2 * prev_ne[k], std::min<uint64_t>(1ull << 27, 2 * (n_front + want0))}));
    void* q;
    PSC_TRY(ensure(g, s.t_slot, s.cap * 8 + 16, &q));
    PSC_CUDA(cudaMemsetAsync(q, 0xFF, s.cap * 8, g->stream));
    PSC_TRY(ensure(g, s.a_slot, s.cap * 8 + 16, &q));
    PSC_TRY(ensure(g, s.b_slot, s.cap * 8 + 16, &q));
    PSC_TRY(ensure(g, s.h_slot, s.cap * 8 + 16, &q));
    PSC_TRY(ensure(g, s.f_slot, s.cap * 4 + 16, &q));
    s.nf = s.ne = n_front;
  }
  {
    ProfScope ps(g, F_MS_SEED);
    ps.bytes = 40.0 * n_front;
    k_ms_seed<<<grid_for(g, n_front, 256), 256, 0, g->stream>>>(
        front, n_front, label_offset, front_labels, (unsigned long long*)g->bufs[st[0].t_slot].p,
        st[0].cap - 1, (uint64_t*)g->bufs[st[0].a_slot].p,
        (unsigned long long*)g->bufs[st[1].t_slot].p, st[1].cap - 1,
        (uint64_t*)g->bufs[st[1].a_slot].p, async ? async->nf_dev : nullptr);
  }
  // asynchronous start: the first sub-round runs on the device's pivot count
  // and the heavy walk follows it whenever some vertex could be heavy
  bool first_async = async && async->nf_dev;
  bool heavy_possible = false;
  if (first_async) {
    PSC_TRY(ensure_max_degrees(g));
    heavy_possible = g->max_deg[0] > kHeavyDeg || g->max_deg[1] > kHeavyDeg;
  }
  for (;;) {
    bool any = false;
    for (auto& s : st) {
      if (s.nf == 0) continue;
      any = true;
      g->stats.subrounds++;
      // room for the VGC local searches of this sub-round: up to
      // min(tq, 64) new pairs each, while the table stays below 2^27 slots
      const uint64_t want = (local && s.nf <= vgc_limit) ? s.nf * std::min<uint32_t>(tau, 64) : 0;
      const bool vgc_room = want && s.cap < (1ull << 27) && s.ne + want > s.cap / 2;
      if (s.grow || 2 * s.ne > s.cap || vgc_room) {
        // keep the load at most 1/2 (1/4 right after growing)
        uint64_t cap2 = pow2_at_least(std::max<uint64_t>(4 * s.ne, 2 * s.cap));
        if (vgc_room)
          cap2 = std::max(cap2, std::min<uint64_t>(1ull << 27, pow2_at_least(2 * (s.ne + want))));
        if (cap2 > (1ull << 40)) return PSC_ERR_TABLE_FULL;
        PSC_TRY(ms_grow(g, s.t_slot, s.cap, cap2));
        s.cap = cap2;
        void* q;
        PSC_TRY(ensure_keep(g, s.a_slot, s.cap * 8 + 16, s.nf * 8, &q));
        PSC_TRY(ensure(g, s.b_slot, s.cap * 8 + 16, &q));
        PSC_TRY(ensure(g, s.h_slot, s.cap * 8 + 16, &q));
        PSC_TRY(ensure(g, s.f_slot, s.cap * 4 + 16, &q));
      }
    }
    if (!any) break;
    PSC_TRY(zero_counters(g));
    if (first_async)  // the pivot count comes back with the counters (staging set 3)
      PSC_CUDA(cudaMemcpyAsync(&g->ctr[3].aux0, async->nf_dev, sizeof(unsigned long long),
                               cudaMemcpyDeviceToDevice, g->stream));
    MsSide vg[2] = {}, ex[2] = {}, hv[2] = {};
    int nv = 0, ne = 0, nh = 0;
    uint64_t v_items = 0, e_items = 0;
    bool is_vgc[2] = {false, false};
    for (int k = 0; k < 2; k++) {
      if (st[k].nf == 0) continue;
      MsSide a = ms_args(g, st[k]);
      if (first_async) a.nin_dev = async->nf_dev;
      is_vgc[k] = local && st[k].nf <= vgc_limit;
      if (is_vgc[k]) {
        vg[nv++] = a;
        v_items += st[k].nf;
      } else {
        ex[ne++] = a;
        e_items += st[k].nf;
      }
      hv[nh++] = a;
    }
    if (nv) {
      ProfScope ps(g, F_MS_VGC);
      // a resident grid, one pair per warp at a time
      if (!g->ms_vgc_blocks) {
        PSC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &g->ms_vgc_blocks, k_ms_vgc<kMsVgcBlock, kMsVgcQueue>, kMsVgcBlock, 0));
        if (g->ms_vgc_blocks < 1) g->ms_vgc_blocks = 1;
      }
      const uint64_t max_blocks = (uint64_t)g->num_sms * g->ms_vgc_blocks;
      const uint64_t blocks =
          std::min(max_blocks, (v_items + kMsVgcBlock / 32 - 1) / (kMsVgcBlock / 32));
      k_ms_vgc<kMsVgcBlock, kMsVgcQueue><<<(unsigned)std::max<uint64_t>(1, blocks), kMsVgcBlock, 0,
                                           g->stream>>>(vg[0], vg[1], labels, tau);
    }
    if (ne) {
      ProfScope ps(g, F_MS_EXPAND);
      switch (p->block) {
        case 128:
          k_ms_expand<128><<<grid_for(g, e_items, 128), 128, 0, g->stream>>>(ex[0], ex[1], labels);
          break;
        case 512:
          k_ms_expand<512><<<grid_for(g, e_items, 512), 512, 0, g->stream>>>(ex[0], ex[1], labels);
          break;
        default:
          k_ms_expand<kMsBlock><<<grid_for(g, e_items, kMsBlock), kMsBlock, 0, g->stream>>>(
              ex[0], ex[1], labels);
      }
    }
    PSC_CUDA(cudaGetLastError());
    if (first_async && heavy_possible) {  // returns at once when no pair was listed
      ProfScope ps(g, F_HEAVY);
      k_ms_heavy<kMsBlock><<<g->num_sms * 4, kMsBlock, 0, g->stream>>>(hv[0], hv[1], labels);
    }
    PSC_TRY(read_counters(g));
    if (first_async) {
      // the pivot count replaces its upper bound
      const uint64_t nf0 = g->hctr[3].aux0;
      async->n_front = nf0;
      for (auto& s : st) {
        s.ne = s.ne - s.nf + nf0;
        s.nf = nf0;
      }
      if (g->profiling && heavy_possible)
        for (int k = 0; k < 2; k++) {
          const Counters& c = g->hctr[st[k].cset];
          g->prof[F_HEAVY].bytes +=
              28.0 * (c.heavy >> kPackShift) + 12.0 * c.heavy_edges + 8.0 * c.heavy_probes;
        }
    }
    // Heavy pairs are rare: the grid-wide walk is launched only for a round
    // that queued some, then the counters are read again.
    if (!first_async &&
        ((st[0].nf && g->hctr[st[0].cset].heavy) || (st[1].nf && g->hctr[st[1].cset].heavy))) {
      {
        ProfScope ps(g, F_HEAVY);
        k_ms_heavy<kMsBlock><<<g->num_sms * 4, kMsBlock, 0, g->stream>>>(hv[0], hv[1], labels);
      }
      PSC_CUDA(cudaGetLastError());
      PSC_TRY(read_counters(g));
      if (g->profiling)
        for (int k = 0; k < 2; k++)
          if (st[k].nf) {
            const Counters& c = g->hctr[st[k].cset];
            g->prof[F_HEAVY].bytes +=
                28.0 * (c.heavy >> kPackShift) + 12.0 * c.heavy_edges + 8.0 * c.heavy_probes;
          }
    }
    if (trace_on()) {
      cudaEvent_t tr = take_event(g);
      PSC_CUDA(cudaEventRecord(tr, g->stream));
      PSC_CUDA(cudaEventSynchronize(tr));
      float ms = 0;  // since the start of the call
      cudaEventElapsedTime(&ms, g->t0, tr);
      give_event(g, tr);
      for (int k = 0; k < 2; k++)
        if (st[k].nf)
          std::fprintf(stderr, "ms side %d mode %s nf %llu next %llu edges %llu probes %llu "
                       "expanded %llu cap %llu ne %llu t %.3f ms\n",
                       k, is_vgc[k] ? "vgc" : "expand", (unsigned long long)st[k].nf,
                       g->hctr[st[k].cset].next, g->hctr[st[k].cset].edges,
                       g->hctr[st[k].cset].probes, g->hctr[st[k].cset].expanded,
                       (unsigned long long)st[k].cap, (unsigned long long)st[k].ne, ms);
    }
    for (int k = 0; k < 2; k++) {
      MsState& s = st[k];
      if (s.nf == 0) continue;
      const Counters& c = g->hctr[s.cset];
      if (g->profiling) {
        // 8 per frontier pair read + 16 per adjacency range + 4 per edge (ids)
        // + 8 per edge (label compare) + 8 per probe + 8 per appended pair
        g->prof[is_vgc[k] ? F_MS_VGC : F_MS_EXPAND].bytes +=
            8.0 * s.nf + 16.0 * c.expanded + 12.0 * c.edges + 8.0 * c.probes + 8.0 * c.next;
      }
      s.ne += c.inserted;
      s.grow = c.fail > 0;
      std::swap(g->bufs[s.a_slot], g->bufs[s.b_slot]);
      s.nf = c.next;
    }
    first_async = false;
  }
  if (async && !async->nf_dev) async->n_front = n_front;
  for (int k = 0; k < 2; k++) {
    out[k].cap = st[k].cap;
    out[k].ne = st[k].ne;
  }
  return PSC_OK;
}

}  // namespace psc

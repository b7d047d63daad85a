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

constexpr int kMsBlock = 256;
constexpr int kMsVgcQueue = 512;  // VGC queue entries per warp
constexpr uint32_t kProbeLimit = 256;

struct ZeroFlag {
  const uint64_t* off;
  const uint64_t* in_off;
  __device__ uint32_t operator()(uint64_t i) const {
    return (off[i + 1] == off[i] || in_off[i + 1] == in_off[i]) ? 1u : 0u;
  }
};

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

struct NotDoneAt {
  const uint32_t* src;
  const uint64_t* labels;
  uint64_t base;
  __device__ uint32_t operator()(uint64_t i) const {
    return (labels[src[base + i]] & kTopBit) ? 0u : 1u;
  }
};

struct CopyAt {
  const uint32_t* src;
  uint32_t* dst;
  uint64_t base;
  __device__ void operator()(uint64_t i, uint64_t excl, uint32_t v) const {
    if (v) dst[excl] = src[base + i];
  }
};

__global__ void k_perm_gather(const uint32_t* __restrict__ nz, uint64_t np, FeistelKey key,
                              uint32_t* P) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np;
       i += (uint64_t)gridDim.x * blockDim.x)
    P[i] = nz[feistel(key, i)];
}

__global__ void k_label_first(const uint32_t* __restrict__ P, uint64_t np,
                              const uint32_t* __restrict__ vf, const uint32_t* __restrict__ vb,
                              uint64_t* labels, uint64_t label) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t v = P[i];
    bool f = (vf[v >> 5] >> (v & 31)) & 1u, b = (vb[v >> 5] >> (v & 31)) & 1u;
    if (f && b)
      labels[v] = label | kTopBit;
    else if (f || b)
      labels[v] = label;
  }
}

__global__ void k_ms_seed(const uint32_t* __restrict__ front, uint64_t nf, uint64_t label_offset,
                          unsigned long long* T, uint64_t mask, uint64_t* F) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nf;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t key = ((uint64_t)front[i] << 32) | (uint64_t)(uint32_t)(label_offset + i);
    uint32_t pr = 0;
    table_insert(T, mask, key, (uint32_t)(mask + 1 < 0xFFFFFFFFull ? mask + 1 : 0xFFFFFFFFu), &pr);
    F[i] = key;
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

// One multi-search sub-round: every frontier pair (u, l) offers l to each
// out-neighbour w of u inside u's subproblem (labels[w] == labels[u]; the
// reference's check !(labels[w] & TOP) && labels[w] == labels[u], scc.hpp:191,225,
// since labels[u] carries no TOP bit); pairs new to the table form the next
// frontier.  An insert that gives up (table too full) re-queues its source
// pair, which is expanded again after the host has grown the table; pairs
// already present are then found and skipped, so no work is lost or doubled.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    k_ms_expand(const uint64_t* __restrict__ off, const uint32_t* __restrict__ E,
                const uint64_t* __restrict__ labels, const uint64_t* __restrict__ Fin, uint64_t nf,
                unsigned long long* T, uint64_t mask, uint64_t* Fout, uint64_t* Fheavy,
                uint32_t* hflag, Counters* ctr) {
  __shared__ WarpExpandSmem sm[BLOCK / 32];
  __shared__ uint64_t s_sub[BLOCK];
  __shared__ uint32_t s_lab[BLOCK];
  __shared__ uint32_t s_fail[BLOCK / 32];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const unsigned wbase = wid * 32;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  unsigned long long scanned = 0, requeued = 0;
  uint32_t probes = 0;
  for (uint64_t base = gw * 32; base < nf; base += nw * 32) {
    const uint64_t i = base + lane;
    uint64_t beg = 0, key = 0;
    uint32_t deg = 0;
    uint64_t sub = 0;
    uint32_t lab = 0;
    if (i < nf) {
      key = Fin[i];
      const uint32_t u = (uint32_t)(key >> 32);
      lab = (uint32_t)key;
      beg = off[u];
      uint64_t d = off[u + 1] - beg;
      sub = labels[u];
      if (d > kHeavyDeg) {
        const unsigned long long h = atomicAdd(&ctr->heavy, 1ull);
        Fheavy[h] = key;
        hflag[h] = 0;
        d = 0;
      }
      deg = (uint32_t)d;
    }
    scanned += deg;
    s_sub[wbase + lane] = sub;
    s_lab[wbase + lane] = lab;
    if (lane == 0) s_fail[wid] = 0;
    __syncwarp();
    warp_expand(sm[wid], beg, deg, [&](bool act, int s, uint64_t e) {
      bool take = false;
      uint64_t nk = 0;
      if (act) {
        const uint32_t w = __ldg(&E[e]);
        if (__ldg(&labels[w]) == s_sub[wbase + s]) {
          nk = ((uint64_t)w << 32) | s_lab[wbase + s];
          int r = table_insert(T, mask, nk, kProbeLimit, &probes);
          take = r == 1;
          if (r < 0) atomicOr(&s_fail[wid], 1u << s);
        }
      }
      unsigned long long pos = warp_append(&ctr->next, take);
      if (take) Fout[pos] = nk;
    });
    __syncwarp();
    const bool rq = (s_fail[wid] >> lane) & 1u;
    unsigned long long pos = warp_append(&ctr->next, rq);
    if (rq) {
      Fout[pos] = key;
      requeued++;
    }
    __syncwarp();
  }
  scanned = warp_sum(scanned);
  requeued = warp_sum(requeued);
  unsigned long long pr = warp_sum((unsigned long long)probes);
  if (lane == 0) {
    if (scanned) atomicAdd(&ctr->edges, scanned);
    if (pr) atomicAdd(&ctr->probes, pr);
    if (requeued) {
      atomicAdd(&ctr->fail, requeued);
      atomicAdd(&ctr->aux1, requeued);
    }
  }
}

// VGC multi-search sub-round (scc.hpp:177-219): one frontier pair (u, l) per
// warp.  If 0 < deg(u) < tau, the warp runs a local BFS for pivot l inside u's
// subproblem in a shared-memory queue of tq = min(tau, QCAP) vertices: a
// neighbour whose (w, l) insert succeeds stays in the queue while there is
// room, else (w, l) spills to the next frontier.  Queued vertices with more
// than tq out-edges and the queue's remainder spill too.  A queued vertex
// whose expansion hit a failed insert is re-queued globally.
template <int BLOCK, int QCAP>
__global__ void __launch_bounds__(BLOCK)
    k_ms_vgc(const uint64_t* __restrict__ off, const uint32_t* __restrict__ E,
             const uint64_t* __restrict__ labels, const uint64_t* __restrict__ Fin, uint64_t nf,
             unsigned long long* T, uint64_t mask, uint64_t* Fout, uint64_t* Fheavy, uint32_t* hflag,
             Counters* ctr, uint32_t tau) {
  __shared__ WarpExpandSmem sm[BLOCK / 32];
  __shared__ uint32_t sq[BLOCK / 32][QCAP];
  __shared__ uint32_t s_fail[BLOCK / 32];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  const uint32_t tq = tau < (uint32_t)QCAP ? tau : (uint32_t)QCAP;
  uint32_t* Q = sq[wid];
  unsigned long long scanned = 0, requeued = 0;
  uint32_t probes = 0;
  for (uint64_t i = gw; i < nf; i += nw) {
    const uint64_t key = Fin[i];
    const uint32_t u = (uint32_t)(key >> 32);
    const uint64_t lab = key & kValMask;
    const uint64_t sub = labels[u];
    const uint64_t ub = off[u], ue = off[u + 1];
    const uint64_t du = ue - ub;
    auto emit = [&](bool take, uint32_t w) {
      unsigned long long pos = warp_append(&ctr->next, take);
      if (take) Fout[pos] = ((uint64_t)w << 32) | lab;
    };
    if (!(du > 0 && du < tq)) {
      if (du > kHeavyDeg) {
        if (lane == 0) {
          const unsigned long long h = atomicAdd(&ctr->heavy, 1ull);
          Fheavy[h] = key;
          hflag[h] = 0;
        }
        continue;
      }
      if (lane == 0) scanned += du;
      bool failed = false;
      for (uint64_t b = ub; b < ue; b += 32) {
        const uint64_t e = b + lane;
        bool take = false;
        uint32_t w = 0;
        if (e < ue) {
          w = __ldg(&E[e]);
          if (__ldg(&labels[w]) == sub) {
            int r = table_insert(T, mask, ((uint64_t)w << 32) | lab, kProbeLimit, &probes);
            take = r == 1;
            failed |= r < 0;
          }
        }
        emit(take, w);
      }
      const bool rq = __any_sync(kFull, failed) && lane == 0;
      emit(rq, u);
      requeued += rq;
      continue;
    }
    if (lane == 0) Q[0] = u;
    __syncwarp();
    uint32_t head = 0, tail = 1;
    while (head < tail && tail < tq) {
      const uint32_t wave = min(32u, tail - head);
      uint64_t beg = 0;
      uint32_t deg = 0, x = 0;
      bool spill_self = false;
      if (lane < wave) {
        x = Q[head + lane];
        beg = off[x];
        uint64_t d = off[x + 1] - beg;
        if (d > tq) {
          spill_self = true;
          d = 0;
        }
        deg = (uint32_t)d;
      }
      head += wave;
      if (lane == 0) s_fail[wid] = 0;
      __syncwarp();
      emit(spill_self, x);
      scanned += deg;
      warp_expand(sm[wid], beg, deg, [&](bool act, int s, uint64_t e) {
        uint32_t w = 0;
        bool take = false;
        if (act) {
          w = __ldg(&E[e]);
          if (__ldg(&labels[w]) == sub) {
            int r = table_insert(T, mask, ((uint64_t)w << 32) | lab, kProbeLimit, &probes);
            take = r == 1;
            if (r < 0) atomicOr(&s_fail[wid], 1u << s);
          }
        }
        const unsigned m = __ballot_sync(kFull, take);
        const uint32_t rank = __popc(m & ((1u << lane) - 1u));
        const uint32_t room = tq - tail;
        const bool local = take && rank < room;
        if (local) Q[tail + rank] = w;
        const uint32_t nt = __popc(m);
        tail += nt < room ? nt : room;
        emit(take && !local, w);
      });
      __syncwarp();
      const bool rq = (s_fail[wid] >> lane) & 1u;
      emit(rq, x);
      requeued += rq;
      __syncwarp();
    }
    for (uint32_t b = head; b < tail; b += 32) {
      const uint32_t k = b + lane;
      const bool t = k < tail;
      emit(t, t ? Q[k] : 0u);
    }
    __syncwarp();
  }
  scanned = warp_sum(scanned);
  requeued = warp_sum(requeued);
  unsigned long long pr = warp_sum((unsigned long long)probes);
  if (lane == 0) {
    if (scanned) atomicAdd(&ctr->edges, scanned);
    if (pr) atomicAdd(&ctr->probes, pr);
    if (requeued) {
      atomicAdd(&ctr->fail, requeued);
      atomicAdd(&ctr->aux1, requeued);
    }
  }
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    k_ms_heavy(const uint64_t* __restrict__ off, const uint32_t* __restrict__ E,
               const uint64_t* __restrict__ labels, const uint64_t* __restrict__ Fheavy,
               uint32_t* hflag, Counters* ctr, unsigned long long* T, uint64_t mask,
               uint64_t* Fout) {
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t nh = *(volatile unsigned long long*)&ctr->heavy;
  const uint64_t stride = (uint64_t)gridDim.x * BLOCK;
  unsigned long long scanned = 0, requeued = 0;
  uint32_t probes = 0;
  for (uint64_t h = 0; h < nh; h++) {
    const uint64_t key = Fheavy[h];
    const uint32_t u = (uint32_t)(key >> 32);
    const uint32_t lab = (uint32_t)key;
    const uint64_t sub = labels[u];
    const uint64_t beg = off[u], end = off[u + 1];
    bool failed = false;
    for (uint64_t b = beg + (uint64_t)blockIdx.x * BLOCK + wid * 32; b < end; b += stride) {
      const uint64_t e = b + lane;
      bool take = false;
      uint64_t nk = 0;
      if (e < end) {
        scanned++;
        const uint32_t w = __ldg(&E[e]);
        if (__ldg(&labels[w]) == sub) {
          nk = ((uint64_t)w << 32) | lab;
          int r = table_insert(T, mask, nk, kProbeLimit, &probes);
          take = r == 1;
          failed |= r < 0;
        }
      }
      unsigned long long pos = warp_append(&ctr->next, take);
      if (take) Fout[pos] = nk;
    }
    // one re-queue per heavy pair, whichever warp saw the failure first
    bool rq = false;
    if (__any_sync(kFull, failed) && lane == 0) rq = atomicExch(&hflag[h], 1u) == 0;
    unsigned long long pos = warp_append(&ctr->next, rq);
    if (rq) {
      Fout[pos] = key;
      requeued++;
    }
  }
  scanned = warp_sum(scanned);
  requeued = warp_sum(requeued);
  unsigned long long pr = warp_sum((unsigned long long)probes);
  if (lane == 0) {
    if (scanned) atomicAdd(&ctr->edges, scanned);
    if (pr) atomicAdd(&ctr->probes, pr);
    if (requeued) {
      atomicAdd(&ctr->fail, requeued);
      atomicAdd(&ctr->aux1, requeued);
    }
  }
}

__global__ void k_partition_small(const unsigned long long* __restrict__ Ts, uint64_t cap_s,
                                  const unsigned long long* __restrict__ Tl, uint64_t mask_l,
                                  unsigned long long* labels) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap_s;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t e = Ts[i];
    if (e == kEmpty) continue;
    const uint32_t v = (uint32_t)(e >> 32);
    const uint64_t l = e & kValMask;
    const uint64_t val = table_contains(Tl, mask_l, e) ? (l | kTopBit) : l;
    if (labels[v] < val) atomicMax(&labels[v], (unsigned long long)val);
  }
}

__global__ void k_partition_large(const unsigned long long* __restrict__ Tl, uint64_t cap_l,
                                  unsigned long long* labels) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap_l;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t e = Tl[i];
    if (e == kEmpty) continue;
    const uint32_t v = (uint32_t)(e >> 32);
    const uint64_t l = e & kValMask;
    if (labels[v] < l) atomicMax(&labels[v], (unsigned long long)l);
  }
}

__global__ void k_finalise(uint64_t* labels, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    labels[i] = (labels[i] & kValMask) - 1;
}

static uint64_t pow2_at_least(uint64_t x) {
  uint64_t c = 1;
  while (c < x) c <<= 1;
  return c;
}

struct MsResult {
  uint64_t cap = 0;
  uint64_t ne = 0;
};

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

// Multi-search in one direction for the batch `front` (n_front pivots with
// labels label_offset + i).  Leaves the closure in table slot tslot.
static int ms_run(psc_graph_s* g, bool backward, const uint32_t* front, uint64_t n_front,
                  uint64_t label_offset, const uint64_t* labels, int tslot, uint64_t prev_ne,
                  const psc_params_t* p, MsResult* res) {
  const uint64_t* off = backward ? g->in_off : g->off;
  const uint32_t* E = backward ? g->in_E : g->E;
  const uint32_t tau = p->tau ? p->tau : 512;
  const bool local = p->local_scc != 0;
  const uint64_t vgc_limit = (uint64_t)g->num_sms * 64;
  uint64_t cap = pow2_at_least(std::max<uint64_t>({4096, 4 * n_front, 2 * prev_ne}));
  unsigned long long* T;
  uint64_t *PA, *PB, *PH;
  uint32_t* HF;
  PSC_TRY(ensure_t(g, tslot, cap, &T));
  PSC_CUDA(cudaMemsetAsync(T, 0xFF, cap * 8, g->stream));
  PSC_TRY(ensure_t(g, B_PA, cap, &PA));
  PSC_TRY(ensure_t(g, B_PB, cap, &PB));
  PSC_TRY(ensure_t(g, B_PH, cap, &PH));
  PSC_TRY(ensure_t(g, B_AUX1, cap, &HF));
  {
    ProfScope ps(g, F_MS_SEED);
    ps.bytes = 4.0 * n_front + 16.0 * n_front;
    k_ms_seed<<<grid_for(g, n_front, 256), 256, 0, g->stream>>>(front, n_front, label_offset, T,
                                                                 cap - 1, PA);
  }
  uint64_t nf = n_front, ne = n_front;
  bool grow = false;
  while (nf > 0) {
    g->stats.subrounds++;
    if (grow || 2 * ne > cap) {
      // keep the load at most 1/2 (1/4 right after growing)
      uint64_t cap2 = pow2_at_least(std::max<uint64_t>(4 * ne, 2 * cap));
      PSC_TRY(ms_grow(g, tslot, cap, cap2));
      cap = cap2;
      void* q;
      PSC_TRY(ensure_keep(g, B_PA, cap * 8 + 16, nf * 8, &q));
      PSC_TRY(ensure(g, B_PB, cap * 8 + 16, &q));
      PSC_TRY(ensure(g, B_PH, cap * 8 + 16, &q));
      PSC_TRY(ensure(g, B_AUX1, cap * 4 + 16, &q));
      if (cap > (1ull << 40)) return PSC_ERR_TABLE_FULL;
    }
    T = (unsigned long long*)g->bufs[tslot].p;
    PA = (uint64_t*)g->bufs[B_PA].p;
    PB = (uint64_t*)g->bufs[B_PB].p;
    PH = (uint64_t*)g->bufs[B_PH].p;
    HF = (uint32_t*)g->bufs[B_AUX1].p;
    PSC_TRY(zero_counters(g));
    if (local && nf <= vgc_limit) {
      ProfScope ps(g, F_MS_VGC);
      k_ms_vgc<kMsBlock, kMsVgcQueue><<<grid_for(g, nf * 32, kMsBlock), kMsBlock, 0, g->stream>>>(
          off, E, labels, PA, nf, T, cap - 1, PB, PH, HF, g->ctr, tau);
    } else {
      ProfScope ps(g, F_MS_EXPAND);
      k_ms_expand<kMsBlock><<<grid_for(g, nf, kMsBlock), kMsBlock, 0, g->stream>>>(
          off, E, labels, PA, nf, T, cap - 1, PB, PH, HF, g->ctr);
    }
    {
      ProfScope ps(g, F_HEAVY);
      k_ms_heavy<kMsBlock><<<g->num_sms * 4, kMsBlock, 0, g->stream>>>(off, E, labels, PH, HF, g->ctr,
                                                                       T, cap - 1, PB);
    }
    PSC_CUDA(cudaGetLastError());
    PSC_TRY(read_counters(g));
    const Counters& c = *g->hctr;
    if (g->profiling) {
      // 16|F| offsets + 4 per edge (ids) + 8 per edge (label compare) + 8 per probe
      // + 8 per appended pair + 8|F| reading the frontier
      g->prof[(local && nf <= vgc_limit) ? F_MS_VGC : F_MS_EXPAND].bytes +=
          24.0 * nf + 12.0 * c.edges + 8.0 * c.probes + 8.0 * c.next;
    }
    const uint64_t nnew = c.next;
    ne += nnew - c.aux1;
    grow = c.fail > 0;
    swap_bufs(g, B_PA, B_PB);
    nf = nnew;
  }
  res->cap = cap;
  res->ne = ne;
  return PSC_OK;
}

static int scc_phases(psc_graph_s* g, uint64_t* labels, const psc_params_t* p);

int scc_run(psc_graph_s* g, const psc_params_t* p, uint64_t* labels) {
  for (auto& pr : g->grow_events) {
    give_event(g, pr.first);
    give_event(g, pr.second);
  }
  g->grow_events.clear();
  PSC_CUDA(cudaEventRecord(g->ph[0], g->stream));
  PSC_TRY(scc_phases(g, labels, p));
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

static int scc_phases(psc_graph_s* g, uint64_t* labels, const psc_params_t* p) {
  const uint64_t n = g->n;
  const unsigned tb = 256;
  uint32_t *P, *nz, *centers, *front, *vf, *vb;
  PSC_TRY(ensure_t(g, B_P, n + 1, &P));
  PSC_TRY(ensure_t(g, B_TMP32, n + 1, &nz));
  // trim
  uint64_t n_zeros = 0;
  PSC_TRY(scan_emit(g, n, ZeroFlag{g->off, g->in_off}, TrimEmit{labels, nz}, &n_zeros, F_TRIM));
  const uint64_t np = n - n_zeros;
  if (np > 0) {
    FeistelKey key = feistel_key(np, p->seed);
    ProfScope ps(g, F_TRIM);
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
    {
      ProfScope ps(g, F_LABEL_FIRST);
      ps.bytes = 4.0 * np + 8.0 * np;
      k_label_first<<<grid_for(g, np, tb), tb, 0, g->stream>>>(P, np, vf, vb, labels, label_offset);
    }
    PSC_TRY(ensure_t(g, B_CENTERS, np + 1, &centers));
    uint64_t nc = 0;
    PSC_TRY(scan_emit(g, np, NotDoneAt{P, labels, 0}, CopyAt{P, centers, 0}, &nc));
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
      uint64_t nf = 0;
      PSC_TRY(scan_emit(g, vs_size, NotDoneAt{centers, labels, cur_offset},
                        CopyAt{centers, front, cur_offset}, &nf));
      cur_offset = end;
      if (nf == 0) continue;
      g->stats.batches++;
      MsResult rf, rb;
      PSC_TRY(ms_run(g, false, front, nf, label_offset, labels, B_TF, out_ne, p, &rf));
      PSC_TRY(ms_run(g, true, front, nf, label_offset, labels, B_TB, in_ne, p, &rb));
      label_offset += nf;
      const bool f_small = rf.cap <= rb.cap;
      const unsigned long long* Ts = (const unsigned long long*)g->bufs[f_small ? B_TF : B_TB].p;
      const unsigned long long* Tl = (const unsigned long long*)g->bufs[f_small ? B_TB : B_TF].p;
      const uint64_t cap_s = f_small ? rf.cap : rb.cap, cap_l = f_small ? rb.cap : rf.cap;
      {
        ProfScope ps(g, F_PARTITION);
        ps.bytes = 8.0 * cap_s + 16.0 * (f_small ? rf.ne : rb.ne);
        k_partition_small<<<grid_for(g, cap_s, tb), tb, 0, g->stream>>>(
            Ts, cap_s, Tl, cap_l - 1, (unsigned long long*)labels);
      }
      {
        ProfScope ps(g, F_PARTITION);
        ps.bytes = 8.0 * cap_l + 8.0 * (f_small ? rb.ne : rf.ne);
        k_partition_large<<<grid_for(g, cap_l, tb), tb, 0, g->stream>>>(Tl, cap_l,
                                                                        (unsigned long long*)labels);
      }
      PSC_CUDA(cudaGetLastError());
      out_ne = rf.ne;
      in_ne = rb.ne;
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

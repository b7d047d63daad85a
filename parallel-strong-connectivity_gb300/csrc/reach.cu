// Single-source reachability on the device (REACH, src/reach.hpp:21-243).
//
// A search "side" is one direction from one source.  The first pivot of SCC
// needs a forward and a backward side; both run in the same launches, so the
// two latency-bound searches overlap.  Each round, per side:
//   push: the frontier is a u32 queue; warps expand 32 frontier vertices at a
//         time with the balanced warp expansion, claim targets on the visited
//         bitmap and append winners with one warp-aggregated atomic (the
//         reference's hashbag insert + pack); vertices above kHeavyDeg
//         out-edges go to a heavy list that the whole grid expands next;
//   VGC:  (local search, reach.hpp:114-171) one frontier vertex per warp runs
//         a local BFS in a shared-memory queue of up to tau vertices before
//         spilling the rest to the next frontier — used while the frontier is
//         small, where rounds, not bandwidth, bound the search;
//   pull: the frontier is a bitmap; each warp owns 32 consecutive unvisited
//         vertices and scans their in-edges until a frontier bit is found,
//         then writes the visited / next-frontier words with one store
//         (the reference's dense_update, no atomics).  Dense rounds stage
//         each warp's next offsets and visited words in shared memory with
//         bulk asynchronous copies; once few reachable vertices remain, the
//         global-memory kernel skips vertices without in-edges (a bitmap per
//         direction, built once per handle), which no pull can reach.
// The push/pull switch follows the reference's rule (REACH::judge, reach.hpp:86-112):
// push while frontier vertices + their out-edges < m / pull_div (20).  After a
// push round the out-edge count is exact (gathered by the kernels); after a
// pull round it is exact for a frontier under 2^14 vertices and otherwise
// estimated from 50 sampled frontier vertices, as the reference's
// dense_sample does (reach.hpp:192-206).
//
// Expansion issues K edges per lane before using any of them, so the loads of
// E and the claims on the bitmap overlap instead of forming one dependent
// memory round trip per edge.
#include <cstdio>
#include <mutex>

#include "common.cuh"
#include "engines.cuh"

namespace psc {

constexpr int kReachBlock = 256;
constexpr int kVgcBlock = 128;  // VGC blocks: 4 warps
constexpr int kVgcQueue = 512;  // VGC queue entries per warp (8 KB of 16-byte entries)
// VGC: edges in flight per lane.  Sparse graphs (fewer than 8 edges per vertex
// on average) use 4: fewer registers, 6 instead of 5 resident blocks per SM,
// more local searches at once (kNN 10^7: 16.8 -> 16.3 ms, grid 4096^2:
// 17.6 -> 16.3 ms); denser ones and batches use 8 (a 1024-graph batch: 16.2
// instead of 19.1 ms).
constexpr int kVgcKWide = 8;
constexpr int kVgcKNarrow = 4;
constexpr int kPushK = 4;       // push: edges in flight per lane
constexpr int kHeavyK = 4;      // heavy vertices: edges in flight per lane
constexpr uint64_t kHeavyChunk = 32 * kHeavyK;  // edges of one heavy-list work unit

// One search side as the kernels see it.
struct ReachSide {
  const uint64_t* off;  // adjacency of the search direction
  const uint32_t* E;
  const uint32_t* qin;  // current frontier (queue)
  uint64_t nin;
  uint32_t* vis;        // visited bitmap
  uint32_t* qout;       // next frontier (queue)
  uint64_t* heavy;      // heavy list: vertex << 32 | first chunk (see heavy_push)
  Counters* ctr;
  // chained VGC rounds: when set, the frontier size is read here (the
  // previous round's ctr->next) instead of nin
  const unsigned long long* nin_dev;
};

// Lists a vertex with more than kHeavyDeg out-edges for k_reach_heavy.  Its
// edges are cut into chunks of kHeavyChunk; one 64-bit atomic on ctr->heavy =
// count << kPackShift | chunks gives the entry its slot and its first chunk,
// so entries in slot order have increasing first chunks.
__device__ __forceinline__ void heavy_push(const ReachSide& S, uint32_t u, uint64_t deg) {
  const unsigned long long old = atomicAdd(
      &S.ctr->heavy, (1ull << kPackShift) + (deg + kHeavyChunk - 1) / kHeavyChunk);
  S.heavy[old >> kPackShift] = ((uint64_t)u << 32) | (old & kPackMask);
}

__global__ void k_reach_init(uint32_t* vis, uint32_t* q, uint32_t src) {
  vis[src >> 5] = 1u << (src & 31);
  q[0] = src;
}

// Several sources at once (one per graph of a batch).
__global__ void k_reach_init_multi(uint32_t* vis, uint32_t* q, const uint32_t* __restrict__ srcs,
                                   uint64_t ns) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ns;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t v = srcs[i];
    atomicOr(&vis[v >> 5], 1u << (v & 31));
    q[i] = v;
  }
}

__device__ __forceinline__ int find_src(const WarpExpandSmem& sm, uint32_t gi) {
  int lo = 0, hi = 31;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (sm.excl[mid] <= gi)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Balanced expansion of the 32 lanes' ranges [beg, beg+deg) with K edges per
// lane in flight: K loads of E, then a read of each target's bitmap word, then
// atomicOr claims only for targets still unvisited.  emit(tm, v) gets the
// lane's K candidates and the mask of those it claimed (warp-collective).
template <int K, class Emit>
__device__ __forceinline__ void expand_claim(WarpExpandSmem& sm, uint64_t beg, uint32_t deg,
                                             const uint32_t* __restrict__ E, uint32_t* vis,
                                             Emit&& emit) {
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
    uint32_t v[K];
    uint32_t pre = 0, tm = 0;
#pragma unroll
    for (int k = 0; k < K; k++) {
      const uint32_t gi = base + k * 32 + lane;
      v[k] = 0xFFFFFFFFu;
      if (gi < total) {
        const int s = find_src(sm, gi);
        v[k] = __ldg(&E[sm.beg[s] + (gi - sm.excl[s])]);
      }
    }
#pragma unroll
    for (int k = 0; k < K; k++)
      if (v[k] != 0xFFFFFFFFu && !(__ldcg(&vis[v[k] >> 5]) & (1u << (v[k] & 31)))) pre |= 1u << k;
#pragma unroll
    for (int k = 0; k < K; k++)
      if (pre & (1u << k)) {
        const uint32_t b = 1u << (v[k] & 31);
        if (!(atomicOr(&vis[v[k] >> 5], b) & b)) tm |= 1u << k;
      }
    emit(tm, v);
  }
  __syncwarp();
}

__device__ __forceinline__ void flush_side_counters(Counters* c0, Counters* c1,
                                                    unsigned long long s0, unsigned long long s1,
                                                    unsigned long long n0, unsigned long long n1,
                                                    unsigned long long x0, unsigned long long x1) {
  s0 = warp_sum(s0);
  s1 = warp_sum(s1);
  n0 = warp_sum(n0);
  n1 = warp_sum(n1);
  x0 = warp_sum(x0);
  x1 = warp_sum(x1);
  if (lane_id() == 0) {
    if (s0 | n0 | x0) {
      atomicAdd(&c0->edges, s0);
      atomicAdd(&c0->next_edges, n0);
      atomicAdd(&c0->expanded, x0);
    }
    if (s1 | n1 | x1) {
      atomicAdd(&c1->edges, s1);
      atomicAdd(&c1->next_edges, n1);
      atomicAdd(&c1->expanded, x1);
    }
  }
}

// Push round for up to two sides: 32 frontier vertices per warp step.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_reach_push(ReachSide s0, ReachSide s1) {
  __shared__ WarpExpandSmem sm[BLOCK / 32];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  const uint64_t c0 = (s0.nin + 31) / 32, c1 = (s1.nin + 31) / 32;
  unsigned long long scanned0 = 0, scanned1 = 0, nedges0 = 0, nedges1 = 0, exp0 = 0, exp1 = 0;
  for (uint64_t c = gw; c < c0 + c1; c += nw) {
    const int sd = c < c0 ? 0 : 1;
    const ReachSide S = sd ? s1 : s0;
    const uint64_t i = (sd ? c - c0 : c) * 32 + lane;
    uint64_t beg = 0;
    uint32_t deg = 0;
    if (i < S.nin) {
      const uint32_t u = S.qin[i];
      beg = S.off[u];
      uint64_t d = S.off[u + 1] - beg;
      (sd ? exp1 : exp0)++;
      if (d > kHeavyDeg) {
        heavy_push(S, u, d);
        d = 0;
      }
      deg = (uint32_t)d;
    }
    (sd ? scanned1 : scanned0) += deg;
    expand_claim<kPushK>(sm[wid], beg, deg, S.E, S.vis, [&](uint32_t tm, const uint32_t* v) {
      warp_append_batch<kPushK>(tm, v, S.qout, &S.ctr->next);
#pragma unroll
      for (int k = 0; k < kPushK; k++)
        if (tm & (1u << k)) (sd ? nedges1 : nedges0) += S.off[v[k] + 1] - S.off[v[k]];
    });
  }
  flush_side_counters(s0.ctr, s1.ctr, scanned0, scanned1, nedges0, nedges1, exp0, exp1);
}

// Local-queue entry: a claimed vertex with its adjacency range.
struct QEnt {
  uint64_t beg;
  uint32_t v;
  uint32_t deg;
};

// Places this lane's claimed candidates (bit k of tm <=> w[k] claimed) into the
// warp's local queue while it has room, then spills the rest to the global
// frontier: one warp scan and at most one global atomic for the whole warp.
template <int K>
__device__ __forceinline__ void vgc_place(uint32_t tm, const uint32_t* w, const uint64_t* vb,
                                          const uint64_t* ve, QEnt* Q, uint32_t& tail, uint32_t tq,
                                          uint32_t* qout, unsigned long long* next_ctr,
                                          unsigned long long& nedges) {
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
  const uint32_t room = tail < tq ? tq - tail : 0;
  const uint32_t nloc = total < room ? total : room;
  unsigned long long sbase = 0;
  if (total > nloc && lane == 0) sbase = atomicAdd(next_ctr, (unsigned long long)(total - nloc));
  sbase = __shfl_sync(kFull, sbase, 0);
  uint32_t r = incl - cnt;
#pragma unroll
  for (int k = 0; k < K; k++)
    if (tm & (1u << k)) {
      const uint64_t vd = ve[k] - vb[k];
      if (r < nloc) {
        Q[tail + r] = QEnt{vb[k], w[k], (uint32_t)(vd < 0xFFFFFFFFull ? vd : 0xFFFFFFFFull)};
      } else {
        qout[sbase + (r - nloc)] = w[k];
        nedges += vd;
      }
      r++;
    }
  tail += nloc;
  __syncwarp();
}

// Claims of one batch: a claimed vertex enters the queue with its adjacency
// range, so the next wave needs no dependent load.  SPEC: the range is loaded
// alongside the claim (off the claim's latency chain, but wasted traffic when
// the claim fails), for latency-bound rounds; otherwise only after a claim
// succeeds, for rounds with more frontier than resident warps.
template <int K, bool SPEC>
__device__ __forceinline__ uint32_t vgc_claim(const uint32_t* w, uint64_t* vb, uint64_t* ve,
                                              const uint64_t* __restrict__ off, uint32_t* vis) {
  if (SPEC) {
#pragma unroll
    for (int k = 0; k < K; k++) {
      vb[k] = ve[k] = 0;
      if (w[k] != 0xFFFFFFFFu) {
        vb[k] = __ldg(&off[w[k]]);
        ve[k] = __ldg(&off[w[k] + 1]);
      }
    }
  }
  uint32_t tm = 0;
#pragma unroll
  for (int k = 0; k < K; k++)
    if (w[k] != 0xFFFFFFFFu) {
      const uint32_t b = 1u << (w[k] & 31);
      if (!(atomicOr(&vis[w[k] >> 5], b) & b)) tm |= 1u << k;
    }
  if (!SPEC) {
#pragma unroll
    for (int k = 0; k < K; k++) {
      vb[k] = ve[k] = 0;
      if (tm & (1u << k)) {
        vb[k] = __ldg(&off[w[k]]);
        ve[k] = __ldg(&off[w[k] + 1]);
      }
    }
  }
  return tm;
}

// A frontier vertex with tau..kHeavyDeg out-edges: the warp walks them with
// K edges per lane in flight.
template <int K>
__device__ __forceinline__ void vgc_direct(const ReachSide& S, uint64_t ub, uint64_t du,
                                           unsigned long long& nedges) {
  const unsigned lane = lane_id();
  const uint64_t ue = ub + du;
  for (uint64_t b = ub; b < ue; b += 32 * K) {
    uint32_t v[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      const uint64_t e = b + k * 32 + lane;
      v[k] = e < ue ? __ldg(&S.E[e]) : 0xFFFFFFFFu;
    }
    uint32_t tm = 0;
#pragma unroll
    for (int k = 0; k < K; k++)
      if (v[k] != 0xFFFFFFFFu && bit_set(S.vis, v[k])) tm |= 1u << k;
#pragma unroll
    for (int k = 0; k < K; k++)
      if (tm & (1u << k)) nedges += S.off[v[k] + 1] - S.off[v[k]];
    warp_append_batch<K>(tm, v, S.qout, &S.ctr->next);
  }
}

// VGC round for up to two sides.  Each warp takes a chunk of up to `chunk`
// frontier vertices (one when the frontier is small, up to 32 when it is much
// larger than the grid, so every warp has work).  Chunk vertices with
// 0 < deg < tau seed a local BFS in a shared-memory queue of tq =
// min(tau, QCAP) entries: each wave takes up to 32 queued vertices and claims
// their neighbours on the bitmap (balanced expansion, K edges per lane in
// flight), keeping claimed vertices in the queue while it has room and
// spilling the rest to the next frontier.  Queued vertices with more than tq
// out-edges, and whatever is left in the queue when it fills or after
// max_waves waves, are spilled too.
// Other chunk vertices are expanded directly (heavy ones by the whole grid).
template <int BLOCK, int QCAP, int K, bool SPEC>
__global__ void __launch_bounds__(BLOCK)
    k_reach_vgc(ReachSide s0, ReachSide s1, uint32_t tau, uint32_t chunk) {
  __shared__ WarpExpandSmem sm[BLOCK / 32];
  __shared__ QEnt sq[BLOCK / 32][QCAP];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  if (s0.nin_dev) s0.nin = *s0.nin_dev;
  if (s1.nin_dev) s1.nin = *s1.nin_dev;
  if (chunk == 0) {  // chained round: chunk size from the device frontier sizes
    const uint64_t per = (s0.nin + s1.nin + nw - 1) / nw;
    chunk = (uint32_t)(per < 1 ? 1 : per > 32 ? 32 : per);
  }
  const uint32_t tq = tau < (uint32_t)QCAP ? tau : (uint32_t)QCAP;
  // A round lasts as long as its longest local search.  Searches that stay
  // narrow (a few vertices per wave) stop after max_waves waves and spill
  // their queue, like a full one: on the kNN 10^7 graph waves hold 8 vertices
  // on average, and this cap (56 at tau = 512) cut the first-pivot phase by
  // 12 % at the cost of 7 % more rounds.
  const uint32_t max_waves = tq / 9 > 8 ? tq / 9 : 8;
  uint32_t C = chunk < tq ? chunk : tq;
  C = C < 1 ? 1 : C > 32 ? 32 : C;
  QEnt* Q = sq[wid];
  unsigned long long scanned0 = 0, scanned1 = 0, nedges0 = 0, nedges1 = 0, exp0 = 0, exp1 = 0;
  unsigned long long wv0 = 0, wv1 = 0;  // waves (warp-uniform)
  const uint64_t c0 = (s0.nin + C - 1) / C, c1 = (s1.nin + C - 1) / C;
  for (uint64_t c = gw; c < c0 + c1; c += nw) {
    const int sd = c < c0 ? 0 : 1;
    const ReachSide S = sd ? s1 : s0;
    unsigned long long& nedges = sd ? nedges1 : nedges0;
    const uint64_t first = (sd ? c - c0 : c) * C;
    const uint64_t left = S.nin - first;
    const uint32_t cnt = left < C ? (uint32_t)left : C;
    uint32_t u = 0;
    uint64_t ub = 0, du = 0;
    if (lane < cnt) {
      u = S.qin[first + lane];
      ub = S.off[u];
      du = S.off[u + 1] - ub;
      (sd ? exp1 : exp0)++;
      if (du > kHeavyDeg) heavy_push(S, u, du);
    }
    uint32_t big = __ballot_sync(kFull, lane < cnt && du >= tq && du <= kHeavyDeg);
    while (big) {
      const int l = __ffs(big) - 1;
      big &= big - 1;
      const uint64_t bb = __shfl_sync(kFull, ub, l), bd = __shfl_sync(kFull, du, l);
      if (lane == 0) (sd ? scanned1 : scanned0) += bd;
      vgc_direct<K>(S, bb, bd, nedges);
    }
    const bool seed = lane < cnt && du > 0 && du < tq;
    const uint32_t smask = __ballot_sync(kFull, seed);
    if (seed) Q[__popc(smask & ((1u << lane) - 1))] = QEnt{ub, u, (uint32_t)du};
    const uint32_t nseed = __popc(smask);
    __syncwarp();
    uint32_t head = 0, tail = nseed, nwave = 0;
    while (head < tail && (head == 0 || tail < tq) && nwave++ < max_waves) {
      const uint32_t wave = min(32u, tail - head);
      uint64_t beg = 0;
      uint32_t deg = 0, x = 0, xdeg = 0;
      bool spill_self = false;
      if (lane < wave) {
        const QEnt q = Q[head + lane];
        x = q.v;
        beg = q.beg;
        xdeg = q.deg;
        deg = q.deg;
        if (deg > tq) {
          spill_self = true;
          deg = 0;
        }
        if (head + lane >= nseed) (sd ? exp1 : exp0)++;
      }
      head += wave;
      (sd ? wv1 : wv0)++;
      __syncwarp();
      if (__any_sync(kFull, spill_self)) {
        unsigned long long pos = warp_append(&S.ctr->next, spill_self);
        if (spill_self) {
          S.qout[pos] = x;
          nedges += xdeg;
        }
      }
      (sd ? scanned1 : scanned0) += deg;
      // balanced expansion over the wave's edges, 32*K per batch
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
      for (uint32_t base = 0; base < total; base += 32 * K) {
        uint32_t w[K];
        uint64_t vb[K], ve[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
          const uint32_t gi = base + k * 32 + lane;
          w[k] = 0xFFFFFFFFu;
          if (gi < total) {
            const int src = find_src(sm[wid], gi);
            w[k] = __ldg(&S.E[sm[wid].beg[src] + (gi - sm[wid].excl[src])]);
          }
        }
        const uint32_t tm = vgc_claim<K, SPEC>(w, vb, ve, S.off, S.vis);
        vgc_place<K>(tm, w, vb, ve, Q, tail, tq, S.qout, &S.ctr->next, nedges);
      }
    }
    // spill what is left in the queue with one reservation
    const uint32_t rem = tail - head;
    if (rem) {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(&S.ctr->next, (unsigned long long)rem);
      base = __shfl_sync(kFull, base, 0);
      for (uint32_t k = lane; k < rem; k += 32) {
        const QEnt q = Q[head + k];
        S.qout[base + k] = q.v;
        nedges += q.deg;
      }
    }
    __syncwarp();
  }
  if (lane == 0) {
    if (wv0) atomicAdd(&s0.ctr->waves, wv0);
    if (wv1) atomicAdd(&s1.ctr->waves, wv1);
  }
  flush_side_counters(s0.ctr, s1.ctr, scanned0, scanned1, nedges0, nedges1, exp0, exp1);
}

// Heavy vertices of both sides: the chunks of a side's heavy list are cut
// into one contiguous range per warp; a warp finds the entry of its first
// chunk once, then claims kHeavyChunk edges per step (a heavy vertex has
// more than 64 chunks, so the next entry is at most one step away).
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_reach_heavy(ReachSide s0, ReachSide s1) {
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
#pragma unroll 1
  for (int sd = 0; sd < 2; sd++) {
    const ReachSide S = sd ? s1 : s0;
    if (!S.ctr) continue;
    const unsigned long long packed = S.ctr->heavy;
    const uint64_t nh = packed >> kPackShift, total = packed & kPackMask;
    const uint64_t per = (total + nw - 1) / nw;
    const uint64_t c_beg = gw * per, c_end = c_beg + per < total ? c_beg + per : total;
    if (nh == 0 || c_beg >= c_end) continue;
    uint64_t h = 0, hi = nh - 1;  // last entry whose first chunk is <= c_beg
    while (h < hi) {
      const uint64_t mid = (h + hi + 1) >> 1;
      if ((uint32_t)__ldg(&S.heavy[mid]) <= c_beg)
        h = mid;
      else
        hi = mid - 1;
    }
    uint64_t ent = __ldg(&S.heavy[h]);
    uint64_t cs = (uint32_t)ent, cn = h + 1 < nh ? (uint32_t)__ldg(&S.heavy[h + 1]) : total;
    uint64_t beg = S.off[ent >> 32], end = S.off[(ent >> 32) + 1];
    unsigned long long scanned = 0, next_edges = 0;
    for (uint64_t c = c_beg; c < c_end; c++) {
      if (c >= cn) {
        h++;
        ent = __ldg(&S.heavy[h]);
        cs = cn;
        cn = h + 1 < nh ? (uint32_t)__ldg(&S.heavy[h + 1]) : total;
        beg = S.off[ent >> 32];
        end = S.off[(ent >> 32) + 1];
      }
      const uint64_t e0 = beg + (c - cs) * kHeavyChunk;
      uint32_t v[kHeavyK], tm = 0;
#pragma unroll
      for (int k = 0; k < kHeavyK; k++) {
        const uint64_t e = e0 + k * 32 + lane;
        v[k] = 0;
        if (e < end) {
          scanned++;
          v[k] = __ldg(&S.E[e]);
        }
      }
#pragma unroll
      for (int k = 0; k < kHeavyK; k++)
        if (e0 + k * 32 + lane < end && bit_set(S.vis, v[k])) tm |= 1u << k;
      warp_append_batch<kHeavyK>(tm, v, S.qout, &S.ctr->next);
#pragma unroll
      for (int k = 0; k < kHeavyK; k++)
        if (tm & (1u << k)) next_edges += S.off[v[k] + 1] - S.off[v[k]];
    }
    scanned = warp_sum(scanned);
    next_edges = warp_sum(next_edges);
    if (lane == 0) {
      if (scanned) atomicAdd(&S.ctr->heavy_edges, scanned);
      if (next_edges) atomicAdd(&S.ctr->next_edges, next_edges);
    }
  }
}

// Pull round: B_* is the reverse direction of the search, A_off the search
// direction's offsets (for the next round's edge count).  A warp owns 32
// consecutive vertices; each unvisited one scans its in-edges for a frontier
// vertex, kPullP edges in flight, alone for its first kPullSolo in-edges; the
// longer in-lists left over are then scanned by the whole warp, one vertex at
// a time, 32 * kPullP edges per step, until a hit.
constexpr int kPullP = 4;
constexpr uint32_t kPullSolo = 64;
#ifndef PSC_PULL_W
#define PSC_PULL_W 4
#endif
constexpr int kPullW = PSC_PULL_W;  // bitmap words per warp step
#ifndef PSC_PULL_STAGED
#define PSC_PULL_STAGED 1
#endif
constexpr bool kPullStaged = PSC_PULL_STAGED != 0;  // tiles staged by bulk copies

__device__ __forceinline__ bool fb_test(const uint32_t* __restrict__ fb, uint32_t x) {
  return (__ldg(&fb[x >> 5]) >> (x & 31)) & 1u;
}

// Solo scan of one unvisited vertex's in-list [j, lim): kPullP in-edges at a
// time until a frontier in-neighbour is found.
__device__ __forceinline__ bool pull_scan(const uint32_t* __restrict__ B_E,
                                          const uint32_t* __restrict__ fb_in, uint64_t& j,
                                          uint64_t lim) {
  bool found = false;
  while (j < lim && !found) {
    uint32_t x[kPullP];
#pragma unroll
    for (int k = 0; k < kPullP; k++) x[k] = j + k < lim ? __ldg(&B_E[j + k]) : 0xFFFFFFFFu;
    bool hit[kPullP];
#pragma unroll
    for (int k = 0; k < kPullP; k++) hit[k] = x[k] != 0xFFFFFFFFu && fb_test(fb_in, x[k]);
    uint64_t step = lim - j < (uint64_t)kPullP ? lim - j : (uint64_t)kPullP;
#pragma unroll
    for (int k = kPullP - 1; k >= 0; k--)
      if (hit[k]) {
        found = true;
        step = k + 1;
      }
    j += step;
  }
  return found;
}

// The whole warp scans the in-lists left over from the solo phase, one
// vertex at a time, 32 * kPullP in-edges per step, until a hit.
__device__ __forceinline__ void pull_long(const uint32_t* __restrict__ B_E,
                                          const uint32_t* __restrict__ fb_in, uint32_t longm,
                                          uint64_t j, uint64_t e, bool& found,
                                          unsigned long long& scanned) {
  const unsigned lane = lane_id();
  while (longm) {
    const int l = __ffs(longm) - 1;
    longm &= longm - 1;
    const uint64_t lb = __shfl_sync(kFull, j, l), le = __shfl_sync(kFull, e, l);
    bool f = false;
    uint64_t jj = lb;
    for (; jj < le && !f; jj += 32 * kPullP) {
      bool hit = false;
#pragma unroll
      for (int k = 0; k < kPullP; k++) {
        const uint64_t q = jj + k * 32 + lane;
        if (q < le) hit |= fb_test(fb_in, __ldg(&B_E[q]));
      }
      f = __any_sync(kFull, hit);
    }
    if (lane == 0) scanned += (jj < le ? jj : le) - lb;
    if (lane == (unsigned)l) found = f;
  }
}

// One warp step of a pull round over W adjacent bitmap words (32 W vertices)
// starting at word w: lane's vertex of word k is unvisited when t[k], with
// in-list [b[k], e[k]).  The first in-edges of all W vertices are loaded
// together (dense rounds often hit at once), then each unvisited vertex
// scans alone, then the long in-lists left over are scanned by the whole
// warp; the words' new frontier bits are written with one store each.
template <int W>
__device__ __forceinline__ void pull_step(uint64_t w, uint64_t nwords, const uint32_t* vw,
                                          const bool* t, const uint64_t* b, const uint64_t* e,
                                          const uint32_t* __restrict__ B_E,
                                          const uint32_t* __restrict__ fb_in, uint32_t* vis,
                                          uint32_t* fb_out, unsigned long long& cnt,
                                          unsigned long long& scanned) {
  const unsigned lane = lane_id();
  bool f[W];
  uint64_t j[W], lim[W];
  uint32_t x[W];
#pragma unroll
  for (int k = 0; k < W; k++) {
    lim[k] = e[k] < b[k] + kPullSolo ? e[k] : b[k] + kPullSolo;
    j[k] = b[k];
    x[k] = t[k] && j[k] < lim[k] ? __ldg(&B_E[j[k]]) : 0xFFFFFFFFu;
  }
#pragma unroll
  for (int k = 0; k < W; k++) {
    f[k] = x[k] != 0xFFFFFFFFu && fb_test(fb_in, x[k]);
    if (t[k] && j[k] < lim[k]) j[k]++;
  }
#pragma unroll
  for (int k = 0; k < W; k++)
    if (t[k] && !f[k]) f[k] = pull_scan(B_E, fb_in, j[k], lim[k]);
#pragma unroll
  for (int k = 0; k < W; k++)
    if (t[k]) scanned += j[k] - b[k];
#pragma unroll
  for (int k = 0; k < W; k++)
    pull_long(B_E, fb_in, __ballot_sync(kFull, t[k] && !f[k] && j[k] < e[k]), j[k], e[k], f[k],
              scanned);
#pragma unroll
  for (int k = 0; k < W; k++) {
    const uint32_t mk = __ballot_sync(kFull, f[k]);
    if (lane == 0 && w + k < nwords) {
      fb_out[w + k] = mk;
      if (mk) vis[w + k] = vw[k] | mk;
      cnt += __popc(mk);
    }
  }
}

__device__ __forceinline__ void flush_pull_counters(Counters* ctr, unsigned long long cnt,
                                                    unsigned long long scanned,
                                                    unsigned long long unvisited) {
  scanned = warp_sum(scanned);
  unvisited = warp_sum(unvisited);
  if (lane_id() == 0) {
    if (cnt) atomicAdd(&ctr->next, cnt);
    if (scanned) atomicAdd(&ctr->edges, scanned);
    if (unvisited) atomicAdd(&ctr->unvisited, unvisited);
  }
}

// A warp's W words read from global memory: visited words and in-list ranges.
// dead (optional): bitmap of vertices without in-edges in this direction,
// which no pull can reach; they are skipped like visited ones (no in-list
// range read) but keep their visited bit clear, and still count as
// unvisited (the work of the reference's dense round).
template <int W>
__device__ __forceinline__ void pull_load_global(uint64_t w, uint64_t nwords, uint64_t n,
                                                 const uint64_t* __restrict__ B_off,
                                                 const uint32_t* __restrict__ dead,
                                                 const uint32_t* vis, uint32_t* vw, bool* t,
                                                 uint64_t* b, uint64_t* e,
                                                 unsigned long long& unvisited) {
  const unsigned lane = lane_id();
  uint32_t dw[W];
#pragma unroll
  for (int k = 0; k < W; k++) {
    vw[k] = w + k < nwords ? vis[w + k] : ~0u;
    dw[k] = dead && w + k < nwords ? __ldg(&dead[w + k]) : 0u;
  }
#pragma unroll
  for (int k = 0; k < W; k++) {
    const uint64_t v = (w + k) * 32 + lane;
    t[k] = v < n && !(((vw[k] | dw[k]) >> lane) & 1u);
    b[k] = e[k] = 0;
    if (t[k]) {
      b[k] = B_off[v];
      e[k] = B_off[v + 1];
    }
    unvisited += v < n && !((vw[k] >> lane) & 1u) ? 1 : 0;  // dead ones included
  }
}

// Pull round reading the visited words and in-list offsets from global
// memory: W words per warp step, so W dependent chains (visited word,
// in-list range, first in-edge, frontier bit) overlap.  The next round's
// out-edge count is left to k_pull_out_edges, off this chain.
template <int BLOCK, int W>
__global__ void __launch_bounds__(BLOCK)
    k_reach_pull(const uint64_t* __restrict__ B_off, const uint32_t* __restrict__ B_E,
                 const uint32_t* __restrict__ fb_in, uint32_t* vis, uint32_t* fb_out, uint64_t n,
                 Counters* ctr, const uint32_t* __restrict__ dead) {
  const unsigned wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  const uint64_t nwords = (n + 31) >> 5;
  unsigned long long cnt = 0, scanned = 0, unvisited = 0;
  for (uint64_t w = gw * W; w < nwords; w += nw * W) {
    uint32_t vw[W];
    bool t[W];
    uint64_t b[W], e[W];
    pull_load_global<W>(w, nwords, n, B_off, dead, vis, vw, t, b, e, unvisited);
    pull_step<W>(w, nwords, vw, t, b, e, B_E, fb_in, vis, fb_out, cnt, scanned);
  }
  flush_pull_counters(ctr, cnt, scanned, unvisited);
}

// ---------------------------------------------------------------------------
// Bulk asynchronous copies into shared memory (cp.async.bulk, the 1-D form of
// the tensor memory accelerator's copies) completing on an mbarrier.  Every
// wait is bounded: past kStageSpin polls it gives up and the kernel reports
// the failure through its counters instead of waiting on.
// ---------------------------------------------------------------------------
constexpr uint32_t kStageSpin = 1u << 20;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < kStageSpin; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Pull round with staged steps: each warp works through its steps of W words
// (32 W vertices) in grid-stride order and keeps its own two shared-memory
// buffers; lane 0 copies the visited words and in-list offsets of the step
// after next into the buffer just worked on (bulk asynchronous copies on the
// warp's own mbarrier), so the loads left on the warp's dependent chain are
// the first in-edge and the frontier bit, and no warp waits for another.  A
// step is staged when its copy stays inside the arrays (offsets
// [v0, v0 + 32 W + 2) with v0 + 32 W + 1 <= n); the last steps are read from
// global memory like k_reach_pull.  A copy that does not arrive within the
// bounded wait sets ctr->aux1 and the warp stops (the host reports it).
template <int BLOCK, int W>
__global__ void __launch_bounds__(BLOCK, 1024 / BLOCK)
    k_reach_pull_staged(const uint64_t* __restrict__ B_off, const uint32_t* __restrict__ B_E,
                        const uint32_t* __restrict__ fb_in, uint32_t* vis, uint32_t* fb_out,
                        uint64_t n, Counters* ctr) {
  constexpr uint32_t NW = BLOCK / 32;
  constexpr uint32_t SV = 32 * W;  // vertices per step
  constexpr uint32_t OFF_BYTES = (SV + 2) * 8;
  constexpr uint32_t VIS_BYTES = W * 4;
  static_assert(OFF_BYTES % 16 == 0 && VIS_BYTES % 16 == 0, "bulk copies of 16-byte multiples");
  __shared__ __align__(128) uint64_t soff[NW][2][SV + 2];
  __shared__ __align__(16) uint32_t svis[NW][2][W];
  __shared__ __align__(8) uint64_t bar[NW][2];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t nwords = (n + 31) >> 5;
  const uint64_t nsteps = (nwords + W - 1) / W;
  const uint64_t s0 = (uint64_t)blockIdx.x * NW + wid, sstep = (uint64_t)gridDim.x * NW;
  auto staged = [&](uint64_t st) { return st * SV + SV + 1 <= n; };
  auto issue = [&](uint64_t st, int b) {  // lane 0
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(&bar[wid][b], OFF_BYTES + VIS_BYTES);
    bulk_copy_g2s(soff[wid][b], B_off + st * SV, OFF_BYTES, &bar[wid][b]);
    bulk_copy_g2s(svis[wid][b], vis + st * W, VIS_BYTES, &bar[wid][b]);
  };
  if (lane == 0) {
    mbar_init(&bar[wid][0], 1);
    mbar_init(&bar[wid][1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  // bit b: the phase parity to wait for / a copy in flight, of buffer b
  uint32_t parity = 0, pending = 0;
  for (int b = 0; b < 2; b++) {
    const uint64_t st = s0 + b * sstep;
    if (st < nsteps && staged(st)) {
      if (lane == 0) issue(st, b);
      pending |= 1u << b;
    }
  }
  unsigned long long cnt = 0, scanned = 0, unvisited = 0;
  bool failed = false;
  int buf = 0;
  for (uint64_t st = s0; st < nsteps; st += sstep, buf ^= 1) {
    const uint64_t w = st * W;
    uint32_t vw[W];
    bool t[W];
    uint64_t b[W], e[W];
    if ((pending >> buf) & 1u) {
      const bool ok = mbar_wait_bounded(&bar[wid][buf], (parity >> buf) & 1u);
      if (__any_sync(kFull, !ok)) {  // giving up is decided warp-wide
        failed = true;
        break;
      }
      parity ^= 1u << buf;
      pending &= ~(1u << buf);
#pragma unroll
      for (int k = 0; k < W; k++) {
        const uint32_t li = k * 32 + lane;
        vw[k] = svis[wid][buf][k];
        t[k] = !((vw[k] >> lane) & 1u);
        b[k] = e[k] = 0;
        if (t[k]) {
          b[k] = soff[wid][buf][li];
          e[k] = soff[wid][buf][li + 1];
        }
        unvisited += t[k] ? 1 : 0;
      }
      // every lane has its values: the buffer may take the step after next
      __syncwarp();
      const uint64_t nt = st + 2 * sstep;
      if (nt < nsteps && staged(nt)) {
        if (lane == 0) issue(nt, buf);
        pending |= 1u << buf;
      }
    } else {
      pull_load_global<W>(w, nwords, n, B_off, nullptr, vis, vw, t, b, e, unvisited);
    }
    pull_step<W>(w, nwords, vw, t, b, e, B_E, fb_in, vis, fb_out, cnt, scanned);
  }
  if (failed) {
    // the copies still in flight land before the block's shared memory goes
    if (pending & 1u) mbar_wait_bounded(&bar[wid][0], parity & 1u);
    if (pending & 2u) mbar_wait_bounded(&bar[wid][1], (parity >> 1) & 1u);
    if (lane == 0) atomicOr(&ctr->aux1, 1ull);
  }
  flush_pull_counters(ctr, cnt, scanned, unvisited);
}

// A pull round's grid: the resident blocks of the kernel (a grid-stride loop
// covers the rest), fewer when the bitmap has fewer warp steps than that.
template <int BLOCK, bool STAGED = false>
static unsigned pull_grid(int num_sms, uint64_t nwords) {
  static int per_sm = [] {
    int b = 0;
    cudaError_t e =
        STAGED ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                     &b, k_reach_pull_staged<BLOCK, kPullW>, BLOCK, 0)
               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_reach_pull<BLOCK, kPullW>,
                                                               BLOCK, 0);
    if (e != cudaSuccess || b < 1) {
      cudaGetLastError();
      b = 1;
    }
    return b;
  }();
  const uint64_t steps = (nwords + kPullW - 1) / kPullW;
  const uint64_t want = (steps + BLOCK / 32 - 1) / (BLOCK / 32);
  const uint64_t cap = (uint64_t)num_sms * per_sm;
  return (unsigned)std::max<uint64_t>(1, std::min(want, cap));
}

constexpr uint64_t kPullStagedTile = 32ull * kPullW;  // vertices of a staged warp step

constexpr uint64_t kPullExactBelow = 1u << 14;
constexpr uint32_t kSampleProbes = 32 * 64;
constexpr uint32_t kSampleHits = 50;

__global__ void k_pull_out_edges(const uint32_t* __restrict__ fb, const uint64_t* __restrict__ A_off,
                                 uint64_t n, uint32_t seed, Counters* ctr) {
  const unsigned lane = lane_id();
  const uint64_t nf = *(volatile unsigned long long*)&ctr->next;
  if (nf < kPullExactBelow) {
    const uint64_t nwords = (n + 31) >> 5;
    unsigned long long sum = 0;
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nwords;
         w += (uint64_t)gridDim.x * blockDim.x) {
      uint32_t word = fb[w];
      while (word) {
        const uint64_t v = w * 32 + (__ffs(word) - 1);
        word &= word - 1;
        sum += A_off[v + 1] - A_off[v];
      }
    }
    sum = warp_sum(sum);
    if (lane == 0 && sum) atomicAdd(&ctr->next_edges, sum);
    return;
  }
  if (blockIdx.x != 0 || threadIdx.x >= 32) return;
  unsigned long long sum = 0;
  uint32_t hits = 0;
  for (uint32_t base = 1; base <= kSampleProbes && hits < kSampleHits; base += 32) {
    const uint32_t idx = (uint32_t)(hash32(seed + base + lane) % n);
    const bool hit = fb_test(fb, idx);
    const uint32_t m = __ballot_sync(kFull, hit);
    const uint32_t rank = __popc(m & ((1u << lane) - 1));
    if (hit && hits + rank < kSampleHits) sum += A_off[idx + 1] - A_off[idx];
    hits += __popc(m);
  }
  sum = warp_sum(sum);
  if (hits > kSampleHits) hits = kSampleHits;
  if (lane == 0) ctr->next_edges = hits ? nf * (sum / hits) : 0;
}

__global__ void k_queue_to_bitmap(const uint32_t* __restrict__ q, uint64_t nq, uint32_t* fb) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nq;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t v = q[i];
    atomicOr(&fb[v >> 5], 1u << (v & 31));
  }
}

// Unordered compaction of a bitmap into a queue (counter: ctr->aux0).
__global__ void k_bitmap_to_queue(const uint32_t* __restrict__ fb, uint64_t nwords, uint32_t* q,
                                  Counters* ctr) {
  const unsigned lane = lane_id();
  const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t base = gw * 32; base < nwords; base += nw * 32) {
    const uint64_t w = base + lane;
    uint32_t word = w < nwords ? fb[w] : 0u;
    uint32_t c = __popc(word);
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(kFull, incl, o);
      if ((int)lane >= o) incl += t;
    }
    uint32_t total = __shfl_sync(kFull, incl, 31);
    unsigned long long pos = 0;
    if (lane == 0 && total) pos = atomicAdd(&ctr->aux0, (unsigned long long)total);
    pos = __shfl_sync(kFull, pos, 0) + (incl - c);
    while (word) {
      int b = __ffs(word) - 1;
      word &= word - 1;
      q[pos++] = (uint32_t)(w * 32 + b);
    }
  }
}

__global__ void k_bitmap_to_bytes(const uint32_t* __restrict__ vis, uint64_t n, uint8_t* out) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = (vis[i >> 5] >> (i & 31)) & 1u;
}

// ---------------------------------------------------------------------------
// Host round loop over one or two sides.
// ---------------------------------------------------------------------------
namespace {

// The VGC kernel of a graph (see kVgcKNarrow): its resident blocks per SM
// (cached on the handle) and its launch.
static bool vgc_narrow(const psc_graph_s* g) { return g->m < 8 * g->n; }

static int vgc_occupancy(psc_graph_s* g) {
  if (!g->vgc_blocks) {
    PSC_CUDA(vgc_narrow(g) ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                                 &g->vgc_blocks, k_reach_vgc<kVgcBlock, kVgcQueue, kVgcKNarrow, true>,
                                 kVgcBlock, 0)
                           : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                                 &g->vgc_blocks, k_reach_vgc<kVgcBlock, kVgcQueue, kVgcKWide, true>,
                                 kVgcBlock, 0));
    if (g->vgc_blocks < 1) g->vgc_blocks = 1;
  }
  return PSC_OK;
}

// spec: speculative range loads (vgc_claim), for rounds whose frontier gives
// each resident warp at most kVgcSpecChunk vertices (latency-bound rounds)
#ifndef PSC_VGC_SPEC_CHUNK
#define PSC_VGC_SPEC_CHUNK 8
#endif
constexpr uint64_t kVgcSpecChunk = PSC_VGC_SPEC_CHUNK;
static void launch_vgc(psc_graph_s* g, unsigned blocks, const ReachSide& a, const ReachSide& b,
                       uint32_t tau, uint32_t chunk, bool spec) {
  cudaStream_t st = g->stream;
  if (vgc_narrow(g)) {
    if (spec)
      k_reach_vgc<kVgcBlock, kVgcQueue, kVgcKNarrow, true><<<blocks, kVgcBlock, 0, st>>>(a, b, tau, chunk);
    else
      k_reach_vgc<kVgcBlock, kVgcQueue, kVgcKNarrow, false><<<blocks, kVgcBlock, 0, st>>>(a, b, tau, chunk);
  } else {
    if (spec)
      k_reach_vgc<kVgcBlock, kVgcQueue, kVgcKWide, true><<<blocks, kVgcBlock, 0, st>>>(a, b, tau, chunk);
    else
      k_reach_vgc<kVgcBlock, kVgcQueue, kVgcKWide, false><<<blocks, kVgcBlock, 0, st>>>(a, b, tau, chunk);
  }
}

// Largest out-degree (out[0]) and in-degree (out[1]) of the graph.
__global__ void k_max_degrees(const uint64_t* __restrict__ off, const uint64_t* __restrict__ in_off,
                              uint64_t n, unsigned long long* out) {
  unsigned long long a = 0, b = 0;
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned long long x = off[v + 1] - off[v], y = in_off[v + 1] - in_off[v];
    a = x > a ? x : a;
    b = y > b ? y : b;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(kFull, a, o), y = __shfl_xor_sync(kFull, b, o);
    a = x > a ? x : a;
    b = y > b ? y : b;
  }
  if (lane_id() == 0) {
    if (a) atomicMax(&out[0], a);
    if (b) atomicMax(&out[1], b);
  }
}

// Once per handle (the graph does not change): max_deg for the heavy-vertex
// check of chained rounds.
int max_degrees_once(psc_graph_s* g) {
  if (g->deg_known) return PSC_OK;
  unsigned long long* d = &g->ctr[2].aux0;  // aux0, aux1 of the staging set
  PSC_CUDA(cudaMemsetAsync(d, 0, 2 * sizeof(unsigned long long), g->stream));
  k_max_degrees<<<grid_for(g, g->n, 256), 256, 0, g->stream>>>(g->off, g->in_off, g->n, d);
  PSC_CUDA(cudaGetLastError());
  PSC_TRY(read_counters(g));
  g->max_deg[0] = g->hctr[2].aux0;
  g->max_deg[1] = g->hctr[2].aux1;
  g->deg_known = true;
  return PSC_OK;
}

// Bitmap words of vertices whose range in off is empty (one warp per word),
// and their count.
__global__ void k_dead_bits(const uint64_t* __restrict__ off, uint64_t n, uint32_t* bits,
                            unsigned long long* count) {
  const uint64_t nwords = (n + 31) >> 5;
  unsigned long long c = 0;
  for (uint64_t base = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~31ull;
       base < nwords * 32; base += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t v = base + lane_id();
    const uint32_t word = __ballot_sync(kFull, v < n && off[v + 1] == off[v]);
    if (lane_id() == 0) {
      bits[base >> 5] = word;
      c += __popc(word);
    }
  }
  if (lane_id() == 0 && c) atomicAdd(count, c);
}

// Once per handle: the vertices a forward pull can never reach (no in-edge)
// and those a backward pull can never reach (no out-edge).
static int dead_bits_once(psc_graph_s* g) {
  if (g->dead_known) return PSC_OK;
  const uint64_t nwords = (g->n + 31) / 32;
  uint32_t* d;
  PSC_TRY(ensure_t(g, B_DEAD, 2 * (nwords + 1), &d));
  unsigned long long* c = &g->ctr[2].aux0;  // aux0, aux1 of the staging set
  PSC_CUDA(cudaMemsetAsync(c, 0, 2 * sizeof(unsigned long long), g->stream));
  k_dead_bits<<<grid_for(g, nwords * 32, 256), 256, 0, g->stream>>>(g->in_off, g->n, d, c);
  k_dead_bits<<<grid_for(g, nwords * 32, 256), 256, 0, g->stream>>>(g->off, g->n, d + nwords + 1,
                                                                     c + 1);
  PSC_CUDA(cudaGetLastError());
  PSC_TRY(read_counters(g));
  g->dead_count[0] = g->hctr[2].aux0;
  g->dead_count[1] = g->hctr[2].aux1;
  g->dead_known = true;
  return PSC_OK;
}

struct Side {
  bool backward = false;
  uint32_t* vis = nullptr;
  int slot_qa = 0, slot_qb = 0, slot_fa = 0, slot_fb = 0, slot_heavy = 0;
  int cset = 0;  // counter block
  uint64_t nf = 0, nf_edges = 0, prev_nf = 0;
  bool pull = false;
  uint32_t rounds = 0;
  // unvisited vertices that some pull could still reach, after the last
  // pull round (an upper bound; UINT64_MAX before the first)
  uint64_t live = UINT64_MAX;
};

// Chained VGC rounds (see reach_sides): rounds per chain, and the counter set
// of side k in round j of a chain.
constexpr int kVgcChain = 8;
static_assert(kVgcChain % 2 == 0, "a chain leaves the frontier in the side's first queue");
constexpr int chain_set(int j, int k) { return 4 + 2 * j + k; }
static_assert(chain_set(kVgcChain - 1, 1) < kCounterSets, "chain counter sets");

enum Mode { M_NONE, M_VGC, M_PUSH, M_PULL };

ReachSide side_args(psc_graph_s* g, const Side& s) {
  ReachSide r;
  r.off = s.backward ? g->in_off : g->off;
  r.E = s.backward ? g->in_E : g->E;
  r.qin = (const uint32_t*)g->bufs[s.slot_qa].p;
  r.nin = s.nf;
  r.vis = s.vis;
  r.qout = (uint32_t*)g->bufs[s.slot_qb].p;
  r.heavy = (uint64_t*)g->bufs[s.slot_heavy].p;
  r.ctr = g->ctr + s.cset;
  r.nin_dev = nullptr;
  return r;
}

Side make_side(bool backward, uint32_t* vis, int second) {
  Side s;
  s.backward = backward;
  s.vis = vis;
  s.slot_qa = second ? B_QA2 : B_QA;
  s.slot_qb = second ? B_QB2 : B_QB;
  s.slot_fa = second ? B_FB_A2 : B_FB_A;
  s.slot_fb = second ? B_FB_B2 : B_FB_B;
  s.slot_heavy = second ? B_HEAVY2 : B_HEAVY;
  s.cset = second ? 1 : 0;
  return s;
}

}  // namespace

int ensure_max_degrees(psc_graph_s* g) { return max_degrees_once(g); }

// Runs the searches of `ns` sides (1 or 2) to completion.  Side k starts from
// srcs[k], or, when d_srcs is given, every side starts from the n_dsrc device
// sources d_srcs.
static int reach_sides(psc_graph_s* g, Side* sides, int ns, const uint32_t* srcs, bool local,
                       uint32_t tau, uint32_t pull_div, const uint32_t* d_srcs = nullptr,
                       uint64_t n_dsrc = 0, uint64_t vgc_max = 0) {
  const uint64_t n = g->n, nwords = (n + 31) / 32;
  // heavy-list fields: < 2^24 entries (m / kHeavyDeg), < 2^32 chunks
  if (g->m >> 36) return PSC_ERR_TOO_LARGE;
  // VGC rounds while the frontier is below one vertex per resident warp
  // (unless the caller sets the limit)
  const uint64_t vgc_limit = vgc_max ? vgc_max : (uint64_t)g->num_sms * 64;
  if (pull_div == 0) pull_div = 20;
  const uint64_t threshold = g->m / pull_div;
  for (int k = 0; k < ns; k++) {
    Side& s = sides[k];
    void* p;
    PSC_TRY(ensure(g, s.slot_qa, (n + 1) * 4, &p));
    PSC_TRY(ensure(g, s.slot_qb, (n + 1) * 4, &p));
    PSC_TRY(ensure(g, s.slot_fa, (nwords + 1) * 4, &p));
    PSC_TRY(ensure(g, s.slot_fb, (nwords + 1) * 4, &p));
    PSC_TRY(ensure(g, s.slot_heavy, (n + 1) * 8, &p));
    PSC_CUDA(cudaMemsetAsync(s.vis, 0, nwords * 4, g->stream));
    if (d_srcs) {
      if (n_dsrc)
        k_reach_init_multi<<<grid_for(g, n_dsrc, 256), 256, 0, g->stream>>>(
            s.vis, (uint32_t*)g->bufs[s.slot_qa].p, d_srcs, n_dsrc);
      s.nf = n_dsrc;
    } else {
      k_reach_init<<<1, 1, 0, g->stream>>>(s.vis, (uint32_t*)g->bufs[s.slot_qa].p, srcs[k]);
      s.nf = 1;
    }
    s.nf_edges = 0;
    s.prev_nf = 0;
    s.pull = false;
    s.rounds = 0;
  }
  const bool tr = trace_on();
  for (uint64_t iter = 0;; iter++) {
    if (iter > n + 2) return PSC_ERR_ITER_LIMIT;
    // Chained VGC rounds: while every active side has a steady frontier well
    // inside VGC range (at least two rounds done, grown at most 1.5x in the
    // last one, far from the pull threshold), kVgcChain rounds are launched
    // back to back, each reading its frontier size from the previous round's
    // counters on the device, and the counters are read back once for the
    // whole chain instead of once per round.  Every round is a VGC round as
    // the switch would have chosen it; a round of a side that ran dry does
    // nothing.
    if (local) {
      int act[2], na = 0;
      bool steady = true;
      for (int k = 0; k < ns; k++) {
        const Side& s = sides[k];
        if (s.nf == 0) continue;
        act[na++] = k;
        steady = steady && !s.pull && s.rounds >= 2 && s.nf <= vgc_limit &&
                 2 * s.nf <= 3 * s.prev_nf && 3 * (s.nf + s.nf_edges) < threshold;
      }
      if (na > 0 && steady) {
        PSC_TRY(max_degrees_once(g));
        bool heavy_possible = false;  // some active direction has a vertex above kHeavyDeg
        for (int a = 0; a < na; a++)
          heavy_possible |= g->max_deg[sides[act[a]].backward ? 1 : 0] > kHeavyDeg;
        PSC_TRY(vgc_occupancy(g));
        const unsigned blocks = (unsigned)((uint64_t)g->num_sms * g->vgc_blocks);
        // speculative range loads while the frontier gives each warp at
        // most kVgcSpecChunk vertices (steady frontiers stay near their
        // start size)
        uint64_t chain_nf = 0;
        for (int a = 0; a < na; a++) chain_nf += sides[act[a]].nf;
        const bool spec = chain_nf <= (uint64_t)blocks * (kVgcBlock / 32) * kVgcSpecChunk;
        PSC_TRY(zero_counters(g));
        for (int j = 0; j < kVgcChain; j++) {
          ReachSide vg[2] = {};
          for (int a = 0; a < na; a++) {
            const Side& s = sides[act[a]];
            ReachSide r = side_args(g, s);
            uint32_t* qa = (uint32_t*)g->bufs[s.slot_qa].p;
            uint32_t* qb = (uint32_t*)g->bufs[s.slot_qb].p;
            r.qin = (j & 1) ? qb : qa;
            r.qout = (j & 1) ? qa : qb;
            r.ctr = g->ctr + chain_set(j, a);
            r.nin_dev = j ? &g->ctr[chain_set(j - 1, a)].next : nullptr;
            vg[a] = r;
          }
          {
            ProfScope ps(g, F_REACH_VGC);
            launch_vgc(g, blocks, vg[0], vg[1], tau, 0u, spec);
          }
          if (heavy_possible) {
            // heavy vertices queued by this round (the kernel returns at once
            // when there are none)
            ProfScope ps(g, F_HEAVY);
            k_reach_heavy<kReachBlock><<<g->num_sms * 4, kReachBlock, 0, g->stream>>>(vg[0], vg[1]);
          }
        }
        PSC_CUDA(cudaGetLastError());
        PSC_TRY(read_counters(g));
        float t_ms = 0;
        if (tr) {
          cudaEvent_t e = take_event(g);
          PSC_CUDA(cudaEventRecord(e, g->stream));
          PSC_CUDA(cudaEventSynchronize(e));
          cudaEventElapsedTime(&t_ms, g->t0, e);
          give_event(g, e);
        }
        for (int a = 0; a < na; a++) {
          Side& s = sides[act[a]];
          uint64_t nin = s.nf;
          for (int j = 0; j < kVgcChain && nin; j++) {
            const Counters& c = g->hctr[chain_set(j, a)];
            s.rounds++;
            if (g->profiling) {
              g->prof[F_REACH_VGC].bytes += 16.0 * c.expanded + 5.0 * c.edges + 5.0 * c.next;
              g->prof[F_HEAVY].bytes += 24.0 * (c.heavy >> kPackShift) + 5.0 * c.heavy_edges;
            }
            if (tr)
              std::fprintf(stderr, "reach side %d round %u mode vgc-chain nf %llu next %llu edges %llu "
                           "expanded %llu waves %llu t %.3f ms\n",
                           act[a], s.rounds, (unsigned long long)nin, c.next, c.edges, c.expanded,
                           c.waves, t_ms);
            s.prev_nf = nin;
            nin = c.next;
          }
          const Counters& last = g->hctr[chain_set(kVgcChain - 1, a)];
          s.nf = last.next;  // zero when the side ran dry inside the chain
          s.nf_edges = last.next_edges;
        }
        continue;
      }
    }
    Mode mode[2] = {M_NONE, M_NONE};
    bool any = false;
    for (int k = 0; k < ns; k++) {
      Side& s = sides[k];
      if (s.nf == 0) continue;
      any = true;
      s.rounds++;
      const bool want_pull = (s.nf + s.nf_edges) >= threshold;
      uint32_t* qa = (uint32_t*)g->bufs[s.slot_qa].p;
      uint32_t* fa = (uint32_t*)g->bufs[s.slot_fa].p;
      if (want_pull && !s.pull) {
        PSC_TRY(dead_bits_once(g));
        ProfScope ps(g, F_REACH_PULL);
        PSC_CUDA(cudaMemsetAsync(fa, 0, nwords * 4, g->stream));
        k_queue_to_bitmap<<<grid_for(g, s.nf, 256), 256, 0, g->stream>>>(qa, s.nf, fa);
        s.pull = true;
      } else if (!want_pull && s.pull) {
        ProfScope ps(g, F_REACH_PUSH);
        PSC_CUDA(cudaMemsetAsync(&g->ctr[s.cset].aux0, 0, 8, g->stream));
        k_bitmap_to_queue<<<grid_for(g, nwords, 256), 256, 0, g->stream>>>(fa, nwords, qa,
                                                                         g->ctr + s.cset);
        s.pull = false;
      }
      mode[k] = s.pull ? M_PULL : (local && s.nf <= vgc_limit) ? M_VGC : M_PUSH;
    }
    if (!any) break;
    PSC_TRY(zero_counters(g));
    ReachSide vg[2] = {}, pu[2] = {}, hv[2] = {};
    int nv = 0, np = 0, nh = 0;
    uint64_t v_items = 0, p_items = 0;
    for (int k = 0; k < ns; k++) {
      if (mode[k] == M_VGC) {
        vg[nv++] = side_args(g, sides[k]);
        v_items += sides[k].nf;
      } else if (mode[k] == M_PUSH) {
        pu[np++] = side_args(g, sides[k]);
        p_items += sides[k].nf;
      }
      if (mode[k] == M_VGC || mode[k] == M_PUSH) hv[nh++] = side_args(g, sides[k]);
    }
    if (nv) {
      ProfScope ps(g, F_REACH_VGC);
      // a resident grid; one frontier vertex per warp while the frontier
      // fits it, else chunks of up to 32 so that every warp stays busy
      PSC_TRY(vgc_occupancy(g));
      const uint64_t max_blocks = (uint64_t)g->num_sms * g->vgc_blocks;
      const uint64_t max_warps = max_blocks * (kVgcBlock / 32);
      const uint64_t chunk = std::min<uint64_t>(32, (v_items + max_warps - 1) / max_warps);
      const uint64_t chunks = (v_items + chunk - 1) / chunk;
      const uint64_t blocks = std::min(max_blocks, (chunks + kVgcBlock / 32 - 1) / (kVgcBlock / 32));
      launch_vgc(g, (unsigned)std::max<uint64_t>(1, blocks), vg[0], vg[1], tau, (uint32_t)chunk,
                 chunk <= kVgcSpecChunk);
    }
    if (np) {
      ProfScope ps(g, F_REACH_PUSH);
      switch (g->block) {
        case 128:
          k_reach_push<128><<<grid_for(g, p_items, 128), 128, 0, g->stream>>>(pu[0], pu[1]);
          break;
        case 512:
          k_reach_push<512><<<grid_for(g, p_items, 512), 512, 0, g->stream>>>(pu[0], pu[1]);
          break;
        default:
          k_reach_push<kReachBlock><<<grid_for(g, p_items, kReachBlock), kReachBlock, 0,
                                      g->stream>>>(pu[0], pu[1]);
      }
    }
    for (int k = 0; k < ns; k++) {
      if (mode[k] != M_PULL) continue;
      Side& s = sides[k];
      ProfScope ps(g, F_REACH_PULL);
      const uint64_t* B_off = s.backward ? g->off : g->in_off;
      const uint32_t* B_E = s.backward ? g->E : g->in_E;
      const uint64_t* A_off = s.backward ? g->in_off : g->off;
      const uint32_t* fa = (const uint32_t*)g->bufs[s.slot_fa].p;
      uint32_t* fbo = (uint32_t*)g->bufs[s.slot_fb].p;
      const uint32_t* dead = (const uint32_t*)g->bufs[B_DEAD].p + (s.backward ? nwords + 1 : 0);
      // Few vertices left that a pull could reach (on R-MAT 2^26 the second
      // pull round finds 1-2 M of the 41 M unvisited, the rest have no
      // in-edge): the global-memory kernel with the dead bitmap reads only
      // their ranges, where the staged one copies every range.
      const bool sparse = s.live != UINT64_MAX && 8 * s.live < n;
      switch (g->block) {
        case 128:
          k_reach_pull<128, kPullW><<<pull_grid<128>(g->num_sms, nwords), 128, 0, g->stream>>>(
              B_off, B_E, fa, s.vis, fbo, n, g->ctr + s.cset, dead);
          break;
        case 512:
          k_reach_pull<512, kPullW><<<pull_grid<512>(g->num_sms, nwords), 512, 0, g->stream>>>(
              B_off, B_E, fa, s.vis, fbo, n, g->ctr + s.cset, dead);
          break;
        default:
          // staged tiles when at least one tile fits inside the arrays and
          // they are 16-byte aligned (bulk copies)
          if (kPullStaged && !sparse && n >= kPullStagedTile + 1 && ((uintptr_t)B_off & 15) == 0 &&
              ((uintptr_t)s.vis & 15) == 0) {
            k_reach_pull_staged<kReachBlock, kPullW>
                <<<pull_grid<kReachBlock, true>(g->num_sms, nwords), kReachBlock, 0, g->stream>>>(
                    B_off, B_E, fa, s.vis, fbo, n, g->ctr + s.cset);
          } else {
            k_reach_pull<kReachBlock, kPullW>
                <<<pull_grid<kReachBlock>(g->num_sms, nwords), kReachBlock, 0, g->stream>>>(
                    B_off, B_E, fa, s.vis, fbo, n, g->ctr + s.cset, dead);
          }
      }
      k_pull_out_edges<<<grid_for(g, nwords, 256), 256, 0, g->stream>>>(
          fbo, A_off, n, hash32((uint32_t)s.rounds), g->ctr + s.cset);
    }
    PSC_CUDA(cudaGetLastError());
    cudaEvent_t tr_b = nullptr;
    if (tr) {
      tr_b = take_event(g);
      PSC_CUDA(cudaEventRecord(tr_b, g->stream));
    }
    PSC_TRY(read_counters(g));
    // Heavy vertices are rare: the grid-wide walk is launched only for a
    // round that queued some, then the counters are read again.
    bool heavy = false;
    for (int k = 0; k < nh; k++) heavy |= g->hctr[hv[k].ctr - g->ctr].heavy != 0;
    if (heavy) {
      {
        ProfScope ps(g, F_HEAVY);
        k_reach_heavy<kReachBlock><<<g->num_sms * 4, kReachBlock, 0, g->stream>>>(hv[0], hv[1]);
      }
      PSC_CUDA(cudaGetLastError());
      PSC_TRY(read_counters(g));
      if (g->profiling)
        for (int k = 0; k < nh; k++) {
          const Counters& c = g->hctr[hv[k].ctr - g->ctr];
          g->prof[F_HEAVY].bytes += 24.0 * (c.heavy >> kPackShift) + 5.0 * c.heavy_edges;
        }
    }
    if (tr) {
      float us = 0;  // ms since the start of the call
      cudaEventElapsedTime(&us, g->t0, tr_b);
      give_event(g, tr_b);
      for (int k = 0; k < ns; k++)
        if (mode[k] != M_NONE)
          std::fprintf(stderr, "reach side %d round %u mode %s nf %llu next %llu edges %llu "
                       "expanded %llu unvisited %llu waves %llu t %.3f ms\n",
                       k, sides[k].rounds, mode[k] == M_VGC ? "vgc" : mode[k] == M_PUSH ? "push" : "pull",
                       (unsigned long long)sides[k].nf, g->hctr[sides[k].cset].next,
                       g->hctr[sides[k].cset].edges, g->hctr[sides[k].cset].expanded,
                       g->hctr[sides[k].cset].unvisited, g->hctr[sides[k].cset].waves, us);
    }
    for (int k = 0; k < ns; k++) {
      Side& s = sides[k];
      if (mode[k] == M_NONE) continue;
      const Counters& c = g->hctr[s.cset];
      if (mode[k] == M_PULL && c.aux1) return PSC_ERR_ITER_LIMIT;  // a staged copy never came
      if (g->profiling) {
        // algorithmic bytes: 16 per adjacency range read, 4 + 1 per edge
        // (target id, visited flag), 5 per new frontier vertex; pull: 16 per
        // unvisited vertex, 5 per scanned in-edge, bitmap words 1/4 byte per vertex
        const int fam = mode[k] == M_VGC ? F_REACH_VGC : mode[k] == M_PUSH ? F_REACH_PUSH
                                                                           : F_REACH_PULL;
        g->prof[fam].bytes += mode[k] == M_PULL
                                  ? 16.0 * c.unvisited + 5.0 * c.edges + 0.25 * n + 1.0 * c.next
                                  : 16.0 * c.expanded + 5.0 * c.edges + 5.0 * c.next;
      }
      if (mode[k] == M_PULL) {
        // unvisited minus the dead ones (all unvisited but sources) minus found
        const uint64_t dead_n = g->dead_count[s.backward ? 1 : 0];
        const uint64_t u = c.unvisited > dead_n ? c.unvisited - dead_n : 0;
        s.live = u > c.next ? u - c.next : 0;
      }
      if (mode[k] == M_PULL)
        std::swap(g->bufs[s.slot_fa], g->bufs[s.slot_fb]);
      else
        std::swap(g->bufs[s.slot_qa], g->bufs[s.slot_qb]);
      s.prev_nf = s.nf;
      s.nf = c.next;
      s.nf_edges = c.next_edges;
    }
  }
  return PSC_OK;
}

int reach_run(psc_graph_s* g, uint32_t src, bool backward, bool local, uint32_t tau,
              uint32_t pull_div, uint32_t* vis, uint32_t* rounds_out) {
  Side s = make_side(backward, vis, 0);
  PSC_TRY(reach_sides(g, &s, 1, &src, local, tau ? tau : 512, pull_div));
  if (rounds_out) *rounds_out = s.rounds;
  return PSC_OK;
}

int reach_pair(psc_graph_s* g, uint32_t src, bool local, uint32_t tau, uint32_t pull_div,
               uint32_t* vis_f, uint32_t* vis_b, uint32_t* rounds_f, uint32_t* rounds_b) {
  Side s[2] = {make_side(false, vis_f, 0), make_side(true, vis_b, 1)};
  const uint32_t srcs[2] = {src, src};
  PSC_TRY(reach_sides(g, s, 2, srcs, local, tau ? tau : 512, pull_div));
  if (rounds_f) *rounds_f = s[0].rounds;
  if (rounds_b) *rounds_b = s[1].rounds;
  return PSC_OK;
}

int reach_pair_multi(psc_graph_s* g, const uint32_t* d_srcs, uint64_t n_srcs, bool local,
                     uint32_t tau, uint32_t pull_div, uint32_t* vis_f, uint32_t* vis_b,
                     uint32_t* rounds_f, uint32_t* rounds_b, uint64_t vgc_max) {
  Side s[2] = {make_side(false, vis_f, 0), make_side(true, vis_b, 1)};
  PSC_TRY(reach_sides(g, s, 2, nullptr, local, tau ? tau : 512, pull_div, d_srcs, n_srcs, vgc_max));
  if (rounds_f) *rounds_f = s[0].rounds;
  if (rounds_b) *rounds_b = s[1].rounds;
  return PSC_OK;
}

}  // namespace psc

using namespace psc;

extern "C" int psc_reach(psc_graph_t g, uint32_t src, int dir, int local, uint32_t tau,
                         uint8_t* dst_out, uint32_t* rounds) {
  if (!g || !dst_out || src >= g->n || (dir != 0 && dir != 1)) return PSC_ERR_INVALID;
  PSC_TRY(call_begin(g));
  uint32_t* vis;
  uint8_t* bytes;
  PSC_TRY(ensure_t(g, B_VIS_F, (g->n + 31) / 32 + 1, &vis));
  PSC_TRY(ensure_t(g, B_AUX0, g->n, &bytes));
  uint32_t r = 0;
  PSC_TRY(reach_run(g, src, dir == 1, local != 0, tau ? tau : 512, 0, vis, &r));
  k_bitmap_to_bytes<<<grid_for(g, g->n, 256), 256, 0, g->stream>>>(vis, g->n, bytes);
  PSC_CUDA(cudaMemcpyAsync(dst_out, bytes, g->n, cudaMemcpyDeviceToHost, g->stream));
  g->stats.reach_rounds = r;
  if (rounds) *rounds = r;
  return call_end(g);
}

// ---------------------------------------------------------------------------
// psc_reach_noalloc: the same reach kernels with their scratch in one
// file-scope device array instead of allocated buffers.
// ---------------------------------------------------------------------------
namespace psc {

constexpr uint64_t kNaMaxN = PSC_NOALLOC_MAX_VERTICES;
constexpr uint64_t kNaWords = kNaMaxN / 32;
// Region sizes are multiples of 64 u32 (256 bytes) so every region, and the
// Counters block at the end, starts 256-byte aligned.
constexpr size_t kNaBitmap = kNaWords + 64;
constexpr size_t kNaQueue = kNaMaxN + 64;
constexpr size_t kNaVis = 0;
constexpr size_t kNaFa = kNaVis + kNaBitmap;
constexpr size_t kNaFb = kNaFa + kNaBitmap;
constexpr size_t kNaQa = kNaFb + kNaBitmap;
constexpr size_t kNaQb = kNaQa + kNaQueue;
constexpr size_t kNaHeavy = kNaQb + kNaQueue;  // u64 entries: two u32 per vertex
constexpr size_t kNaCtr = kNaHeavy + 2 * kNaQueue;
constexpr size_t kNaTotal = kNaCtr + 64;
static_assert(sizeof(Counters) <= 64 * sizeof(uint32_t), "counters fit their region");
static_assert(kNaCtr % 64 == 0, "256-byte aligned counters");

static __device__ __align__(256) uint32_t g_noalloc_scratch[kNaTotal];

struct NoAllocDevice {
  uint32_t* scratch = nullptr;
  int num_sms = 0;
  bool ready = false;
};
constexpr int kNaMaxDevices = 64;
static NoAllocDevice g_na_dev[kNaMaxDevices];
static std::mutex g_na_mu;

// Once per device, with that device current: the array's device address.
static int noalloc_setup(int dev, NoAllocDevice* out) {
  if (dev < 0 || dev >= kNaMaxDevices) return PSC_ERR_INVALID;
  std::lock_guard<std::mutex> lock(g_na_mu);
  NoAllocDevice& d = g_na_dev[dev];
  if (!d.ready) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_status(e);
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_status(e);
    d.scratch = (uint32_t*)p;
    d.num_sms = sms;
    d.ready = true;
  }
  *out = d;
  return PSC_OK;
}

static unsigned na_grid(int sms, uint64_t items, unsigned block) {
  uint64_t want = (items + block - 1) / block;
  uint64_t cap = (uint64_t)sms * 16;
  if (want < 1) want = 1;
  if (want > cap) want = cap;
  return (unsigned)want;
}

}  // namespace psc

extern "C" int psc_reach_noalloc(const uint64_t* d_off, const uint32_t* d_E,
                                 const uint64_t* d_in_off, const uint32_t* d_in_E, uint64_t n,
                                 uint64_t m, uint32_t src, int dir, uint8_t* d_dst, void* stream,
                                 uint32_t* rounds) {
  if (n > kNaMaxN || (m >> 36)) return PSC_ERR_TOO_LARGE;
  if (!d_off || (m && !d_E) || !d_dst || n == 0 || src >= n || (dir != 0 && dir != 1))
    return PSC_ERR_INVALID;
  if ((d_in_off == nullptr) != (d_in_E == nullptr)) return PSC_ERR_INVALID;
  if (!d_in_off) {  // symmetric: the transpose is the graph itself
    d_in_off = d_off;
    d_in_E = d_E;
  }
  int dev = 0;
  PSC_CUDA(cudaGetDevice(&dev));
  NoAllocDevice nd;
  PSC_TRY(noalloc_setup(dev, &nd));
  cudaStream_t s = (cudaStream_t)stream;
  const bool backward = dir == 1;
  const uint64_t* A_off = backward ? d_in_off : d_off;
  const uint32_t* A_E = backward ? d_in_E : d_E;
  const uint64_t* B_off = backward ? d_off : d_in_off;
  const uint32_t* B_E = backward ? d_E : d_in_E;
  const uint64_t nwords = (n + 31) / 32;
  uint32_t* vis = nd.scratch + kNaVis;
  uint32_t* fa = nd.scratch + kNaFa;
  uint32_t* fb = nd.scratch + kNaFb;
  uint32_t* qa = nd.scratch + kNaQa;
  uint32_t* qb = nd.scratch + kNaQb;
  uint64_t* heavy = (uint64_t*)(nd.scratch + kNaHeavy);
  Counters* ctr = (Counters*)(nd.scratch + kNaCtr);
  Counters hc;  // host copy of the counters (stack memory)

  // the caller's arrays are checked before any kernel indexes by them (the
  // check of psc_graph_upload; the flag is a word of the counters region)
  PSC_CUDA(cudaMemsetAsync(ctr, 0, sizeof(Counters), s));
  const unsigned vgrid = na_grid(nd.num_sms, std::max<uint64_t>(n, m), 256);
  k_validate_csr<><<<vgrid, 256, 0, s>>>(d_off, n, d_E, m, &ctr->aux0);
  if (d_in_off != d_off)
    k_validate_csr<><<<vgrid, 256, 0, s>>>(d_in_off, n, d_in_E, m, &ctr->aux0);
  PSC_CUDA(cudaGetLastError());
  PSC_CUDA(cudaMemcpyAsync(&hc, ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
  PSC_CUDA(cudaStreamSynchronize(s));
  if (hc.aux0) return PSC_ERR_INVALID;
  // the array keeps the previous call's contents: clear the visited bitmap
  PSC_CUDA(cudaMemsetAsync(vis, 0, nwords * 4, s));
  k_reach_init<<<1, 1, 0, s>>>(vis, qa, src);
  const uint64_t threshold = m / 20;
  uint64_t nf = 1, nf_edges = 0;
  bool pull = false;
  uint32_t r = 0;
  while (nf > 0) {
    r++;
    if (r > n + 2) return PSC_ERR_ITER_LIMIT;
    const bool want_pull = (nf + nf_edges) >= threshold;
    if (want_pull && !pull) {
      PSC_CUDA(cudaMemsetAsync(fa, 0, nwords * 4, s));
      k_queue_to_bitmap<<<na_grid(nd.num_sms, nf, 256), 256, 0, s>>>(qa, nf, fa);
      pull = true;
    } else if (!want_pull && pull) {
      PSC_CUDA(cudaMemsetAsync(ctr, 0, sizeof(Counters), s));
      k_bitmap_to_queue<<<na_grid(nd.num_sms, nwords, 256), 256, 0, s>>>(fa, nwords, qa, ctr);
      pull = false;
    }
    PSC_CUDA(cudaMemsetAsync(ctr, 0, sizeof(Counters), s));
    if (!pull) {
      ReachSide side{A_off, A_E, qa, nf, vis, qb, heavy, ctr};
      ReachSide none{};
      k_reach_push<kReachBlock><<<na_grid(nd.num_sms, nf, kReachBlock), kReachBlock, 0, s>>>(side,
                                                                                          none);
      PSC_CUDA(cudaGetLastError());
      PSC_CUDA(cudaMemcpyAsync(&hc, ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
      PSC_CUDA(cudaStreamSynchronize(s));
      // vertices above the heavy threshold were listed: the whole grid
      // expands them before the round ends
      if (hc.heavy)
        k_reach_heavy<kReachBlock><<<nd.num_sms * 4, kReachBlock, 0, s>>>(side, none);
      std::swap(qa, qb);
      if (!hc.heavy) {
        nf = hc.next;
        nf_edges = hc.next_edges;
        continue;
      }
    } else {
      k_reach_pull<kReachBlock, kPullW>
          <<<pull_grid<kReachBlock>(nd.num_sms, nwords), kReachBlock, 0, s>>>(
              B_off, B_E, fa, vis, fb, n, ctr, nullptr);
      k_pull_out_edges<<<na_grid(nd.num_sms, nwords, 256), 256, 0, s>>>(fb, A_off, n,
                                                                        hash32(r), ctr);
      std::swap(fa, fb);
    }
    PSC_CUDA(cudaGetLastError());
    PSC_CUDA(cudaMemcpyAsync(&hc, ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    PSC_CUDA(cudaStreamSynchronize(s));
    nf = hc.next;
    nf_edges = hc.next_edges;
  }
  k_bitmap_to_bytes<<<na_grid(nd.num_sms, n, 256), 256, 0, s>>>(vis, n, d_dst);
  PSC_CUDA(cudaGetLastError());
  PSC_CUDA(cudaStreamSynchronize(s));
  if (rounds) *rounds = r;
  return PSC_OK;
}

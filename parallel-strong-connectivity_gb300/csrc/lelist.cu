// BFS distances and LE-lists on the device.
//
// BFS (BFS::bfs, src/bfs.hpp:200-238): level-synchronous; each level is a
// push round (frontier queue, balanced warp expansion, atomicCAS on dist) or
// a pull round (every unreached vertex scans its in-edges for a frontier bit),
// switched by the reference's rule (bfs.hpp:88-117).
//
// LE-lists (LE_LIST::le_list, src/LeList.hpp:219-328) for the priority order
// centers[0..n): a BFS from centers[0] gives every reached v the entry
// (v, 0, dist); then prefix-doubling batches of priorities run a multi-source
// BFS over (priority, vertex) pairs (a pair set in an open-addressing table of
// 64-bit keys).  Level s of a batch offers (p, w) for every edge (u, w) of a
// frontier pair (p, u) when s < dist[w] (dist of earlier batches), records a
// new pair as the entry (w, p, s) and lowers next_dist[w] to s.  The table is
// grown before every level so that every possible insert fits: the levels
// stay exact.  Finally the entries are bucketed by target, sorted by priority
// inside each bucket, and an entry is kept only if its distance is below every
// earlier priority's (LeList.hpp:278-313); priorities map back to vertices.
// The result is the reference's list, and seq_le_list's (LeList.hpp:76-115).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "engines.cuh"
#include "scan.cuh"

namespace psc {

constexpr int kLeBlock = 256;
constexpr int kLeK = 4;       // edges in flight per lane: BFS push, heavy pairs
constexpr int kLeKLight = 8;  // the same for the warp expansion of light pairs

// ---------------------------------------------------------------------------
// BFS
// ---------------------------------------------------------------------------
__global__ void k_fill_u32(uint32_t* a, uint64_t n, uint32_t v) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    a[i] = v;
}

__global__ void k_bfs_init(uint32_t* dist, uint32_t* q, uint32_t src) {
  dist[src] = 0;
  q[0] = src;
}

template <int BLOCK, int K>
__global__ void __launch_bounds__(BLOCK)
    k_bfs_push(const uint64_t* __restrict__ off, const uint32_t* __restrict__ E,
               const uint32_t* __restrict__ qin, uint64_t nin, uint32_t* dist, uint32_t level,
               uint32_t* qout, Counters* ctr) {
  __shared__ WarpExpandSmem sm[BLOCK / 32];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  unsigned long long scanned = 0, next_edges = 0;
  for (uint64_t base = gw * 32; base < nin; base += nw * 32) {
    const uint64_t i = base + lane;
    uint64_t beg = 0, rem = 0;
    if (i < nin) {
      const uint32_t u = qin[i];
      beg = off[u];
      rem = off[u + 1] - beg;
    }
    scanned += rem;
    while (__any_sync(kFull, rem > 0)) {
      const uint32_t deg = (uint32_t)(rem < (1ull << 26) ? rem : (1ull << 26));
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
      for (uint32_t b = 0; b < total; b += 32 * K) {
        uint32_t v[K], tm = 0, pre = 0;
#pragma unroll
        for (int k = 0; k < K; k++) {
          const uint32_t gi = b + k * 32 + lane;
          v[k] = kNone;
          if (gi < total) {
            int lo = 0, hi = 31;
            while (lo < hi) {
              const int mid = (lo + hi + 1) >> 1;
              if (sm[wid].excl[mid] <= gi)
                lo = mid;
              else
                hi = mid - 1;
            }
            v[k] = __ldg(&E[sm[wid].beg[lo] + (gi - sm[wid].excl[lo])]);
          }
        }
#pragma unroll
        for (int k = 0; k < K; k++)
          if (v[k] != kNone && __ldcg(&dist[v[k]]) == kNone) pre |= 1u << k;
#pragma unroll
        for (int k = 0; k < K; k++)
          if ((pre & (1u << k)) && atomicCAS(&dist[v[k]], kNone, level) == kNone) tm |= 1u << k;
        warp_append_batch<K>(tm, v, qout, &ctr->next);
#pragma unroll
        for (int k = 0; k < K; k++)
          if (tm & (1u << k)) next_edges += off[v[k] + 1] - off[v[k]];
      }
      __syncwarp();
      beg += deg;
      rem -= deg;
    }
  }
  scanned = warp_sum(scanned);
  next_edges = warp_sum(next_edges);
  if (lane == 0) {
    if (scanned) atomicAdd(&ctr->edges, scanned);
    if (next_edges) atomicAdd(&ctr->next_edges, next_edges);
  }
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    k_bfs_pull(const uint64_t* __restrict__ B_off, const uint32_t* __restrict__ B_E,
               const uint64_t* __restrict__ A_off, const uint32_t* __restrict__ fb_in,
               uint32_t* dist, uint32_t level, uint32_t* fb_out, uint64_t n, Counters* ctr) {
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  const uint64_t nwords = (n + 31) >> 5;
  unsigned long long cnt = 0, scanned = 0, next_edges = 0;
  for (uint64_t w = gw; w < nwords; w += nw) {
    const uint64_t v = w * 32 + lane;
    bool found = false;
    if (v < n && dist[v] == kNone) {
      const uint64_t b = B_off[v], e = B_off[v + 1];
      uint64_t j = b;
      for (; j < e; j++) {
        const uint32_t x = __ldg(&B_E[j]);
        if ((__ldg(&fb_in[x >> 5]) >> (x & 31)) & 1u) {
          found = true;
          break;
        }
      }
      scanned += (found ? j + 1 : j) - b;
      if (found) {
        dist[v] = level;
        next_edges += A_off[v + 1] - A_off[v];
      }
    }
    const uint32_t mask = __ballot_sync(kFull, found);
    if (lane == 0) {
      fb_out[w] = mask;
      cnt += __popc(mask);
    }
  }
  scanned = warp_sum(scanned);
  next_edges = warp_sum(next_edges);
  if (lane == 0) {
    if (cnt) atomicAdd(&ctr->next, cnt);
    if (scanned) atomicAdd(&ctr->edges, scanned);
    if (next_edges) atomicAdd(&ctr->next_edges, next_edges);
  }
}

__global__ void k_bfs_q2b(const uint32_t* __restrict__ q, uint64_t nq, uint32_t* fb) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nq;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t v = q[i];
    atomicOr(&fb[v >> 5], 1u << (v & 31));
  }
}

__global__ void k_bfs_b2q(const uint32_t* __restrict__ fb, uint64_t nwords, uint32_t* q,
                          Counters* ctr) {
  const unsigned lane = lane_id();
  const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t base = gw * 32; base < nwords; base += nw * 32) {
    const uint64_t w = base + lane;
    uint32_t word = w < nwords ? fb[w] : 0u;
    const uint32_t c = __popc(word);
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(kFull, incl, o);
      if ((int)lane >= o) incl += t;
    }
    const uint32_t total = __shfl_sync(kFull, incl, 31);
    unsigned long long pos = 0;
    if (lane == 0 && total) pos = atomicAdd(&ctr->aux0, (unsigned long long)total);
    pos = __shfl_sync(kFull, pos, 0) + (incl - c);
    while (word) {
      const int b = __ffs(word) - 1;
      word &= word - 1;
      q[pos++] = (uint32_t)(w * 32 + b);
    }
  }
}

// dist: device u32[n], filled here (UINT32_MAX = unreached).
int bfs_run(psc_graph_s* g, uint32_t src, uint32_t* dist, uint32_t* rounds_out) {
  const uint64_t n = g->n, nwords = (n + 31) / 32;
  uint32_t *qa, *qb, *fa, *fb;
  PSC_TRY(ensure_t(g, B_QA, n + 1, &qa));
  PSC_TRY(ensure_t(g, B_QB, n + 1, &qb));
  PSC_TRY(ensure_t(g, B_FB_A, nwords + 1, &fa));
  PSC_TRY(ensure_t(g, B_FB_B, nwords + 1, &fb));
  k_fill_u32<<<grid_for(g, n, 256), 256, 0, g->stream>>>(dist, n, kNone);
  k_bfs_init<<<1, 1, 0, g->stream>>>(dist, qa, src);
  const uint64_t threshold = g->m / 20;
  uint64_t nf = 1, nf_edges = 0;
  bool pull = false;
  uint32_t level = 0;
  while (nf > 0) {
    level++;
    if (level > n + 1) return PSC_ERR_ITER_LIMIT;
    const bool want_pull = (nf + nf_edges) >= threshold;
    if (want_pull && !pull) {
      PSC_CUDA(cudaMemsetAsync(fa, 0, nwords * 4, g->stream));
      k_bfs_q2b<<<grid_for(g, nf, 256), 256, 0, g->stream>>>(qa, nf, fa);
      pull = true;
    } else if (!want_pull && pull) {
      PSC_TRY(zero_counters(g));
      k_bfs_b2q<<<grid_for(g, nwords, 256), 256, 0, g->stream>>>(fa, nwords, qa, g->ctr);
      pull = false;
    }
    PSC_TRY(zero_counters(g));
    if (!pull) {
      ProfScope ps(g, F_LE);
      k_bfs_push<kLeBlock, kLeK><<<grid_for(g, nf, kLeBlock), kLeBlock, 0, g->stream>>>(
          g->off, g->E, qa, nf, dist, level, qb, g->ctr);
      std::swap(qa, qb);
      swap_bufs(g, B_QA, B_QB);
    } else {
      ProfScope ps(g, F_LE);
      k_bfs_pull<kLeBlock><<<grid_for(g, nwords * 32, kLeBlock), kLeBlock, 0, g->stream>>>(
          g->in_off, g->in_E, g->off, fa, dist, level, fb, n, g->ctr);
      std::swap(fa, fb);
      swap_bufs(g, B_FB_A, B_FB_B);
    }
    PSC_CUDA(cudaGetLastError());
    PSC_TRY(read_counters(g));
    if (g->profiling) {
      // push: 16 per frontier vertex, 8 per edge (id, distance), 8 per new
      // vertex; pull: both bitmaps, 16 per unvisited vertex, 8 per scanned
      // in-edge, 4 per new vertex
      const Counters& c = g->hctr[0];
      g->prof[F_LE].bytes += pull ? 0.25 * n + 16.0 * c.unvisited + 8.0 * c.edges + 4.0 * c.next
                                  : 16.0 * nf + 8.0 * c.edges + 8.0 * c.next;
    }
    nf = g->hctr[0].next;
    nf_edges = g->hctr[0].next_edges;
  }
  if (rounds_out) *rounds_out = level;
  return PSC_OK;
}

// ---------------------------------------------------------------------------
// LE-lists
// ---------------------------------------------------------------------------
// List entries: key = target << 32 | priority, value = distance.

// First round: every reached v gives (v, 0, dist[v]).
__global__ void k_le_first(const uint32_t* __restrict__ dist, uint64_t n, uint64_t* Lk,
                           uint32_t* Ld, Counters* ctr) {
  const unsigned lane = lane_id();
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n;
       base += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t v = base + lane;
    const bool t = v < n && dist[v] != kNone;
    const unsigned long long pos = warp_append(&ctr->aux1, t);
    if (t) {
      Lk[pos] = v << 32;
      Ld[pos] = dist[v];
    }
  }
}

// Batch seeds (LeList.hpp:137-147): pair (i, centers[i]) for i in
// [start, start + count); entry (centers[i], i, 0); next_dist = 0.
__global__ void k_le_seed(const uint32_t* __restrict__ centers, uint64_t start, uint64_t count,
                          unsigned long long* T, uint64_t mask, uint64_t* F, uint32_t* next_dist,
                          uint64_t* Lk, uint32_t* Ld, uint64_t lbase) {
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < count;
       j += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = start + j;
    const uint32_t c = centers[i];
    const uint64_t key = (i << 32) | c;
    uint32_t pr = 0;
    table_insert(T, mask, key, 0xFFFFFFFFu, &pr);
    F[j] = key;
    next_dist[c] = 0;
    Lk[lbase + j] = ((uint64_t)c << 32) | i;
    Ld[lbase + j] = 0;
  }
}

// Pairs whose vertex has more than `hthr` edges are expanded by k_le_heavy,
// balanced over the whole grid, instead of by one warp.  They are listed with
// one 64-bit atomic on ctr->heavy = count << kLeHeavyShift | edge offset, so
// list order and edge offsets agree: Hs is increasing and entry h owns the
// virtual edges [Hs[h], Hs[h + 1]).
constexpr uint64_t kLeHeavy = 256;
constexpr int kLeHeavyShift = 40;
constexpr uint32_t kLeProbes = 256;  // probe limit of a sized-by-estimate level
constexpr uint64_t kLeHeavyMask = (1ull << kLeHeavyShift) - 1;

// Offers the warp's K candidate pairs key[k] = (p, w[k]) (kEmpty: none):
// new pairs go to the next frontier and become list entries (w, p, level),
// and lower next_dist[w]; an insert that gives up after `limit` probes is
// counted in `fails`, and the level is then run again on a larger table.
// Once a lane of the warp has failed, the warp stops probing and counts its
// further offers as failures (the rerun makes them all again).  Called by all
// 32 lanes.
template <int K>
__device__ __forceinline__ void le_offer(const uint64_t* __restrict__ off, const uint32_t (&w)[K],
                                         const uint64_t (&key)[K], uint32_t level,
                                         unsigned long long* T, uint64_t mask, uint32_t limit,
                                         uint64_t* Fout, uint32_t* next_dist, uint64_t* Lk,
                                         uint32_t* Ld, Counters* ctr, uint32_t& probes,
                                         uint32_t& fails, unsigned long long& next_edges) {
  const unsigned lane = lane_id();
  uint32_t tm = 0;
  const bool full = __any_sync(kFull, fails != 0);
#pragma unroll
  for (int k = 0; k < K; k++)
    if (key[k] != kEmpty && full) {
      fails++;
    } else if (key[k] != kEmpty) {
      const int r = table_insert(T, mask, key[k], limit, &probes);
      if (r == 1) {
        tm |= 1u << k;
        atomicMin(&next_dist[w[k]], level);
      } else if (r < 0) {
        fails++;
      }
    }
  const uint32_t cnt = __popc(tm);
  uint32_t pinc = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(kFull, pinc, o);
    if ((int)lane >= o) pinc += t;
  }
  const uint32_t tot = __shfl_sync(kFull, pinc, 31);
  if (!tot) return;
  unsigned long long fb = 0, lb = 0;
  if (lane == 31) {
    fb = atomicAdd(&ctr->next, (unsigned long long)tot);
    lb = atomicAdd(&ctr->aux1, (unsigned long long)tot);
  }
  fb = __shfl_sync(kFull, fb, 31) + (pinc - cnt);
  lb = __shfl_sync(kFull, lb, 31) + (pinc - cnt);
#pragma unroll
  for (int k = 0; k < K; k++)
    if (tm & (1u << k)) {
      Fout[fb++] = key[k];
      Lk[lb] = ((uint64_t)w[k] << 32) | (key[k] >> 32);
      Ld[lb++] = level;
      next_edges += off[w[k] + 1] - off[w[k]];
    }
}

// One level of a batch: frontier pairs (p, u); every edge (u, w) with
// level < dist[w] offers (p, w).  A warp expands 32 pairs together; pairs
// with more than hthr edges are listed for k_le_heavy.
template <int BLOCK, int K>
__global__ void __launch_bounds__(BLOCK)
    k_le_expand(const uint64_t* __restrict__ off, const uint32_t* __restrict__ E,
                const uint32_t* __restrict__ dist, const uint64_t* __restrict__ Fin, uint64_t nf,
                uint32_t level, unsigned long long* T, uint64_t mask, uint32_t limit,
                uint64_t* Fout, uint32_t* next_dist, uint64_t* Lk, uint32_t* Ld, uint64_t hthr,
                uint64_t* Hk, uint64_t* Hs, Counters* ctr) {
  __shared__ WarpExpandSmem sm[BLOCK / 32];
  __shared__ uint32_t s_p[BLOCK];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  unsigned long long scanned = 0, next_edges = 0;
  uint32_t probes = 0, fails = 0;
  for (uint64_t base = gw * 32; base < nf; base += nw * 32) {
    const uint64_t i = base + lane;
    uint64_t beg = 0, rem = 0;
    uint32_t p = 0;
    if (i < nf) {
      const uint64_t key = Fin[i];
      const uint32_t u = (uint32_t)key;
      p = (uint32_t)(key >> 32);
      beg = off[u];
      rem = off[u + 1] - beg;
      if (rem > hthr) {
        const unsigned long long old =
            atomicAdd(&ctr->heavy, (1ull << kLeHeavyShift) + (unsigned long long)rem);
        const uint64_t h = old >> kLeHeavyShift;
        Hk[h] = key;
        Hs[h] = old & kLeHeavyMask;
        rem = 0;
      }
    }
    scanned += rem;
    s_p[wid * 32 + lane] = p;
    while (__any_sync(kFull, rem > 0)) {
      const uint32_t deg = (uint32_t)(rem < (1ull << 26) ? rem : (1ull << 26));
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
      for (uint32_t b = 0; b < total; b += 32 * K) {
        uint32_t w[K], src[K];
        uint64_t key[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
          const uint32_t gi = b + k * 32 + lane;
          w[k] = kNone;
          src[k] = 0;
          if (gi < total) {
            int lo = 0, hi = 31;
            while (lo < hi) {
              const int mid = (lo + hi + 1) >> 1;
              if (sm[wid].excl[mid] <= gi)
                lo = mid;
              else
                hi = mid - 1;
            }
            src[k] = lo;
            w[k] = __ldg(&E[sm[wid].beg[lo] + (gi - sm[wid].excl[lo])]);
          }
        }
#pragma unroll
        for (int k = 0; k < K; k++) {
          key[k] = kEmpty;
          if (w[k] != kNone && level < __ldg(&dist[w[k]]))
            key[k] = ((uint64_t)s_p[wid * 32 + src[k]] << 32) | w[k];
        }
        le_offer<K>(off, w, key, level, T, mask, limit, Fout, next_dist, Lk, Ld, ctr, probes,
                    fails, next_edges);
      }
      __syncwarp();
      beg += deg;
      rem -= deg;
    }
  }
  scanned = warp_sum(scanned);
  next_edges = warp_sum(next_edges);
  const unsigned long long pr = warp_sum((unsigned long long)probes);
  const unsigned long long nfail = warp_sum((unsigned long long)fails);
  if (lane == 0) {
    if (scanned) atomicAdd(&ctr->edges, scanned);
    if (next_edges) atomicAdd(&ctr->next_edges, next_edges);
    if (pr) atomicAdd(&ctr->probes, pr);
    if (nfail) atomicAdd(&ctr->fail, nfail);
  }
}

// The heavy pairs of a level: their edge lists, concatenated, are cut into
// one contiguous slice per warp of a resident grid.  A warp finds the entry at
// the start of its slice once, then walks 32 * K edges per step with the
// entry's data held warp-uniform; an entry has more than 32 * K edges, so a
// step spans at most two entries.
template <int BLOCK, int K>
__global__ void __launch_bounds__(BLOCK)
    k_le_heavy(const uint64_t* __restrict__ off, const uint32_t* __restrict__ E,
               const uint32_t* __restrict__ dist, const uint64_t* __restrict__ Hk,
               const uint64_t* __restrict__ Hs, uint32_t level, unsigned long long* T,
               uint64_t mask, uint32_t limit, uint64_t* Fout, uint32_t* next_dist, uint64_t* Lk,
               uint32_t* Ld, Counters* ctr) {
  constexpr uint64_t kStep = 32 * K;
  const unsigned long long packed = ctr->heavy;
  const uint64_t nh = packed >> kLeHeavyShift, total = packed & kLeHeavyMask;
  if (nh == 0) return;
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  const uint64_t slice = ((total + nw - 1) / nw + kStep - 1) / kStep * kStep;
  const uint64_t x_beg = gw * slice;
  if (x_beg >= total) return;
  const uint64_t x_end = x_beg + slice < total ? x_beg + slice : total;
  uint64_t h = 0, hi = nh - 1;  // last entry with Hs <= x_beg
  while (h < hi) {
    const uint64_t mid = (h + hi + 1) >> 1;
    if (__ldg(&Hs[mid]) <= x_beg)
      h = mid;
    else
      hi = mid - 1;
  }
  // entry h: virtual edges [hs, hn), pair key pk, edge list from eb
  uint64_t hs = __ldg(&Hs[h]), hn = h + 1 < nh ? __ldg(&Hs[h + 1]) : total;
  uint64_t pk = __ldg(&Hk[h]), eb = off[(uint32_t)pk];
  unsigned long long scanned = 0, next_edges = 0;
  uint32_t probes = 0, fails = 0;
  for (uint64_t x0 = x_beg; x0 < x_end; x0 += kStep) {
    const bool nxt = x0 + kStep >= hn && h + 1 < nh;
    uint64_t pk2 = 0, eb2 = 0, hn2 = 0;
    if (nxt) {
      pk2 = __ldg(&Hk[h + 1]);
      eb2 = off[(uint32_t)pk2];
      hn2 = h + 2 < nh ? __ldg(&Hs[h + 2]) : total;
    }
    uint32_t w[K];
    uint64_t key[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      const uint64_t x = x0 + k * 32 + lane;
      w[k] = kNone;
      key[k] = kEmpty;
      if (x < x_end) {
        const bool second = x >= hn;
        const uint32_t v = __ldg(&E[second ? eb2 + (x - hn) : eb + (x - hs)]);
        scanned++;
        if (level < __ldg(&dist[v])) {
          w[k] = v;
          key[k] = ((second ? pk2 : pk) & 0xFFFFFFFF00000000ull) | v;
        }
      }
    }
    le_offer<K>(off, w, key, level, T, mask, limit, Fout, next_dist, Lk, Ld, ctr, probes, fails,
                next_edges);
    if (nxt) {
      h++;
      hs = hn;
      hn = hn2;
      pk = pk2;
      eb = eb2;
    }
  }
  scanned = warp_sum(scanned);
  next_edges = warp_sum(next_edges);
  const unsigned long long pr = warp_sum((unsigned long long)probes);
  const unsigned long long nfail = warp_sum((unsigned long long)fails);
  if (lane == 0) {
    if (scanned) atomicAdd(&ctr->edges, scanned);
    if (next_edges) atomicAdd(&ctr->next_edges, next_edges);
    if (pr) atomicAdd(&ctr->probes, pr);
    if (nfail) atomicAdd(&ctr->fail, nfail);
  }
}

__global__ void k_le_rehash(const unsigned long long* __restrict__ T, uint64_t cap,
                            unsigned long long* T2, uint64_t mask2) {
  uint32_t pr = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t e = T[i];
    if (e != kEmpty) table_insert(T2, mask2, e, 0xFFFFFFFFu, &pr);
  }
}

// Bucket the entries by target: counts, then scatter (keys become
// priority << 32 | dist inside each target's bucket).
__global__ void k_le_count(const uint64_t* __restrict__ Lk, uint64_t L, uint32_t* cnt) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < L;
       i += (uint64_t)gridDim.x * blockDim.x)
    atomicAdd(&cnt[Lk[i] >> 32], 1u);
}

struct CountValue {
  const uint32_t* cnt;
  __device__ uint32_t operator()(uint64_t i) const { return cnt[i]; }
};

struct BucketOffsets {
  uint64_t* boff;
  uint32_t* cursor;
  __device__ void operator()(uint64_t i, uint64_t excl, uint32_t) const {
    boff[i] = excl;
    cursor[i] = 0;
  }
};

__global__ void k_le_scatter(const uint64_t* __restrict__ Lk, const uint32_t* __restrict__ Ld,
                             uint64_t L, const uint64_t* __restrict__ boff, uint32_t* cursor,
                             uint64_t* B) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < L;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t t = (uint32_t)(Lk[i] >> 32);
    const uint32_t p = (uint32_t)Lk[i];
    const uint32_t k = atomicAdd(&cursor[t], 1u);
    B[boff[t] + k] = ((uint64_t)p << 32) | Ld[i];
  }
}

// Sorts every bucket [boff[v], boff[v+1]) of u64 values ascending.  Buckets
// of at most kSegThread entries (nearly all of them: a vertex's list candidates
// number a few) are sorted by one thread each with a compare-exchange network
// in registers, and the longer ones are listed; a block then sorts each listed
// bucket: one warp up to 32 entries (odd-even transposition in registers), a
// bitonic network in shared memory up to kSegSmem entries, and the same
// network over a global scratch row beyond that.
constexpr int kSegBlock = 256;
constexpr int kSegSmem = 2048;
constexpr int kSegThread = 16;

template <int S>
__device__ __forceinline__ void sort_net_u64(uint64_t* B, uint64_t b, uint32_t len) {
  uint64_t a[S];
#pragma unroll
  for (int i = 0; i < S; i++) a[i] = i < (int)len ? B[b + i] : ~0ull;
#pragma unroll
  for (int i = 1; i < S; i++)
#pragma unroll
    for (int j = i; j > 0; j--) {
      const uint64_t x = a[j - 1], y = a[j];
      a[j - 1] = x < y ? x : y;
      a[j] = x < y ? y : x;
    }
#pragma unroll
  for (int i = 0; i < S; i++)
    if (i < (int)len) B[b + i] = a[i];
}

// Small buckets sorted in place; longer ones appended to big[] (count in
// ctr->heavy); the longest length goes to ctr->aux0.
__global__ void k_seg_sort_small(const uint64_t* __restrict__ boff, uint64_t nseg, uint64_t* B,
                                 uint32_t* big, Counters* ctr) {
  unsigned long long mx = 0;
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nseg;
       v += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = boff[v], len = boff[v + 1] - b;
    mx = len > mx ? len : mx;
    if (len < 2) continue;
    if (len <= 4)
      sort_net_u64<4>(B, b, (uint32_t)len);
    else if (len <= kSegThread)
      sort_net_u64<kSegThread>(B, b, (uint32_t)len);
    else
      big[atomicAdd(&ctr->heavy, 1ull)] = (uint32_t)v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(kFull, mx, o);
    mx = t > mx ? t : mx;
  }
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(&ctr->aux0, mx);
}

__device__ void bitonic_u64(uint64_t* a, uint32_t len, uint32_t pad) {
  for (uint32_t i = len + threadIdx.x; i < pad; i += blockDim.x) a[i] = ~0ull;
  __syncthreads();
  for (uint32_t k = 2; k <= pad; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < pad; i += blockDim.x) {
        const uint32_t p = i ^ j;
        if (p > i) {
          const uint64_t x = a[i], y = a[p];
          const bool up = (i & k) == 0;
          if ((x > y) == up) {
            a[i] = y;
            a[p] = x;
          }
        }
      }
      __syncthreads();
    }
  }
}

__global__ void __launch_bounds__(kSegBlock)
    k_seg_sort_u64(const uint32_t* __restrict__ big, uint64_t nbig,
                   const uint64_t* __restrict__ boff, uint64_t* B, uint64_t* scratch,
                   uint64_t scratch_len) {
  __shared__ uint64_t buf[kSegSmem];
  for (uint64_t k = blockIdx.x; k < nbig; k += gridDim.x) {
    const uint32_t v = big[k];
    const uint64_t b = boff[v], len = boff[v + 1] - b;
    if (len <= 32) {
      if (threadIdx.x < 32) {
        const int t = (int)threadIdx.x;
        uint64_t x = t < (int)len ? B[b + t] : ~0ull;
        for (int r = 0; r < 32; r++) {
          const int partner = ((t & 1) == (r & 1)) ? t + 1 : t - 1;
          const uint64_t y = __shfl_sync(kFull, x, partner & 31);
          if (partner >= 0 && partner < 32) x = t < partner ? min(x, y) : max(x, y);
        }
        if (t < (int)len) B[b + t] = x;
      }
      __syncthreads();
      continue;
    }
    uint32_t pad = 64;
    while (pad < len) pad <<= 1;
    if (pad <= kSegSmem) {
      for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) buf[i] = B[b + i];
      bitonic_u64(buf, (uint32_t)len, pad);
      for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) B[b + i] = buf[i];
      __syncthreads();
    } else if (pad <= scratch_len) {
      uint64_t* a = scratch + (uint64_t)blockIdx.x * scratch_len;
      for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) a[i] = B[b + i];
      __syncthreads();
      bitonic_u64(a, (uint32_t)len, pad);
      for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) B[b + i] = a[i];
      __syncthreads();
    }
  }
}

// Keep an entry if its distance is below every earlier priority's in its
// bucket (LeList.hpp:293-311); marks keep[i] in {0, 1}.
__global__ void k_le_filter(const uint64_t* __restrict__ boff, uint64_t nseg,
                            const uint64_t* __restrict__ B, uint8_t* keep) {
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nseg;
       v += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t best = 0xFFFFFFFFu;
    for (uint64_t i = boff[v]; i < boff[v + 1]; i++) {
      const uint32_t d = (uint32_t)B[i];
      const bool k = d < best;
      keep[i] = k;
      if (k) best = d;
    }
  }
}

__global__ void k_le_target(const uint64_t* __restrict__ boff, uint64_t nseg, uint32_t* tgt) {
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nseg;
       v += (uint64_t)gridDim.x * blockDim.x)
    for (uint64_t i = boff[v]; i < boff[v + 1]; i++) tgt[i] = (uint32_t)v;
}

struct KeepValue {
  const uint8_t* keep;
  __device__ uint32_t operator()(uint64_t i) const { return keep[i]; }
};

struct TripleEmit {
  const uint64_t* B;
  const uint32_t* tgt;
  const uint32_t* centers;
  uint32_t* out;
  __device__ void operator()(uint64_t i, uint64_t excl, uint32_t v) const {
    if (!v) return;
    out[3 * excl] = tgt[i];
    out[3 * excl + 1] = centers[B[i] >> 32];
    out[3 * excl + 2] = (uint32_t)B[i];
  }
};

struct SeedDeg {
  const uint64_t* off;
  const uint32_t* c;
  uint64_t s;
  __device__ uint32_t operator()(uint64_t i) const {
    const uint64_t d = off[c[s + i] + 1] - off[c[s + i]];
    return (uint32_t)(d < 0xFFFFFFFFull ? d : 0xFFFFFFFFull);
  }
};

struct NoEmit {
  __device__ void operator()(uint64_t, uint64_t, uint32_t) const {}
};

static uint64_t p2(uint64_t x) {
  uint64_t c = 1;
  while (c < x) c <<= 1;
  return c;
}

// Grows the entry buffers (Lk u64, Ld u32) to hold `need` entries, keeping
// the first `len`.
static int le_list_reserve(psc_graph_s* g, uint64_t need, uint64_t len, uint64_t* cap) {
  if (need <= *cap) return PSC_OK;
  uint64_t c = std::max<uint64_t>(need, *cap + *cap / 2);
  void* p;
  PSC_TRY(ensure_keep(g, B_PH, c * 8 + 16, len * 8, &p));
  PSC_TRY(ensure_keep(g, B_AUX3, c * 4 + 16, len * 4, &p));
  *cap = c;
  return PSC_OK;
}

// LE-list of the graph for priorities centers (device u32[n]); the result
// (triples) stays in slot B_AUX0; *len = its entry count.
int lelist_run(psc_graph_s* g, const uint32_t* centers, double beta, uint64_t* len_out) {
  const uint64_t n = g->n;
  const unsigned tb = 256;
  uint32_t *dist, *next_dist, *cnt;
  PSC_TRY(ensure_t(g, B_VIS_F, n + 1, &dist));
  PSC_TRY(ensure_t(g, B_VIS_B, n + 1, &next_dist));
  // first round: BFS from centers[0] (LeList.hpp:232-253)
  uint32_t c0 = 0;
  PSC_CUDA(cudaMemcpyAsync(&g->hctr[3].aux0, centers, 4, cudaMemcpyDeviceToHost, g->stream));
  PSC_CUDA(cudaStreamSynchronize(g->stream));
  std::memcpy(&c0, &g->hctr[3].aux0, 4);
  uint32_t r = 0;
  PSC_TRY(bfs_run(g, c0, dist, &r));
  g->stats.reach_rounds = r;
  uint64_t lcap = 0, L = 0;
  PSC_TRY(le_list_reserve(g, std::max<uint64_t>(4 * n, 1024), 0, &lcap));
  PSC_TRY(zero_counters(g));
  {
    ProfScope ps(g, F_LE);
    k_le_first<<<grid_for(g, n, tb), tb, 0, g->stream>>>(dist, n, (uint64_t*)g->bufs[B_PH].p,
                                                        (uint32_t*)g->bufs[B_AUX3].p, g->ctr);
  }
  PSC_CUDA(cudaMemcpyAsync(next_dist, dist, n * 4, cudaMemcpyDeviceToDevice, g->stream));
  PSC_TRY(read_counters(g));
  L = g->hctr[0].aux1;
  // prefix-doubling batches (LeList.hpp:255-276)
  uint64_t step = 1, finished = 1;
  uint64_t prev_ne = n >> 1;
  // inserts per scanned edge at each level of the previous batch
  std::vector<double> ratio, ratio_next;
  while (finished < n) {
    step = (uint64_t)std::ceil((double)step * beta);
    if (step < 1) step = 1;
    const uint64_t end = std::min<uint64_t>(finished + step, n);
    const uint64_t start = finished, nf0 = end - start;
    g->stats.batches++;
    uint64_t cap = p2(std::max<uint64_t>({4096, 4 * nf0, 2 * std::min<uint64_t>(prev_ne, 4 * n)}));
    unsigned long long* T;
    uint64_t *FA, *FB;
    PSC_TRY(ensure_t(g, B_TF, cap, &T));
    PSC_CUDA(cudaMemsetAsync(T, 0xFF, cap * 8, g->stream));
    PSC_TRY(ensure_t(g, B_PA, cap, &FA));
    PSC_TRY(ensure_t(g, B_PB, cap, &FB));
    PSC_TRY(le_list_reserve(g, L + nf0, L, &lcap));
    {
      ProfScope ps(g, F_LE);
      k_le_seed<<<grid_for(g, nf0, tb), tb, 0, g->stream>>>(
          centers, start, nf0, T, cap - 1, FA, next_dist, (uint64_t*)g->bufs[B_PH].p,
          (uint32_t*)g->bufs[B_AUX3].p, L);
    }
    L += nf0;
    uint64_t nf = nf0, ne = nf0;
    // out-edges of the seeds bound the first level's inserts
    uint64_t bound = 0;
    PSC_TRY(scan_emit(g, nf0, SeedDeg{g->off, centers, start}, NoEmit{}, &bound, F_LE));
    // Rehashes the pair set into a table of cap2 slots; the frontiers keep
    // their first keep_a (current) and keep_b (next) pairs.
    auto grow = [&](uint64_t cap2, uint64_t keep_a, uint64_t keep_b) -> int {
      unsigned long long* T2;
      PSC_TRY(ensure_t(g, B_TS, cap2, &T2));
      PSC_CUDA(cudaMemsetAsync(T2, 0xFF, cap2 * 8, g->stream));
      k_le_rehash<<<grid_for(g, cap, 256), 256, 0, g->stream>>>(T, cap, T2, cap2 - 1);
      swap_bufs(g, B_TF, B_TS);
      cap = cap2;
      T = T2;
      g->stats.table_grows++;
      void* q;
      PSC_TRY(ensure_keep(g, B_PA, cap * 8 + 16, keep_a * 8, &q));
      PSC_TRY(ensure_keep(g, B_PB, cap * 8 + 16, keep_b * 8, &q));
      FA = (uint64_t*)g->bufs[B_PA].p;
      FB = (uint64_t*)g->bufs[B_PB].p;
      return PSC_OK;
    };
    ratio_next.clear();
    uint32_t level = 0;
    while (nf > 0) {
      level++;
      g->stats.subrounds++;
      // A level inserts at most `bound` pairs (one per scanned edge), far
      // fewer in practice.  The table is sized for twice the previous batch's
      // inserts per edge at this level, at load <= 1/2; inserts give up after
      // kLeProbes probes, and a level that had failures runs again on a table
      // sized for `bound` (offers are idempotent: pairs already inserted are
      // not emitted twice), without a probe limit.
      uint64_t est = bound;
      if (level <= ratio.size())
        est = std::min<uint64_t>(bound, (uint64_t)std::ceil(2.0 * ratio[level - 1] * bound) + 4096);
      bool exact = est == bound;
      if (2 * (ne + est) > cap) PSC_TRY(grow(p2(2 * (ne + est) + 1024), nf, 0));
      PSC_TRY(le_list_reserve(g, L + bound, L, &lcap));
      // heavy list: at most bound / (hthr + 1) <= 2^23 entries (count field)
      // over at most bound < 2^40 edges (offset field)
      if (bound >> kLeHeavyShift) return PSC_ERR_CAPACITY;
      const uint64_t hthr = std::max<uint64_t>(kLeHeavy, bound >> 23);
      const bool any_heavy = bound > hthr;
      uint64_t *Hk = nullptr, *Hs = nullptr;
      if (any_heavy) {
        const uint64_t hcap = std::min<uint64_t>(nf, bound / (hthr + 1)) + 1;
        PSC_TRY(ensure_t(g, B_PA2, hcap, &Hk));
        PSC_TRY(ensure_t(g, B_PB2, hcap, &Hs));
      }
      if (any_heavy && !g->le_heavy_blocks) {
        PSC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &g->le_heavy_blocks, k_le_heavy<kLeBlock, kLeK>, kLeBlock, 0));
        if (g->le_heavy_blocks < 1) g->le_heavy_blocks = 1;
      }
      PSC_TRY(zero_counters(g));
      uint32_t attempts = 0;
      for (;;) {
        attempts++;
        {
          ProfScope ps(g, F_LE);
          uint64_t* Lk = (uint64_t*)g->bufs[B_PH].p + L;
          uint32_t* Ld = (uint32_t*)g->bufs[B_AUX3].p + L;
          const uint32_t limit = exact ? 0xFFFFFFFFu : kLeProbes;
          k_le_expand<kLeBlock, kLeKLight><<<grid_for(g, nf, kLeBlock), kLeBlock, 0, g->stream>>>(
              g->off, g->E, dist, FA, nf, level, T, cap - 1, limit, FB, next_dist, Lk, Ld,
              any_heavy ? hthr : ~0ull, Hk, Hs, g->ctr);
          if (any_heavy) {
            const uint64_t hblocks = (bound + kLeBlock * kLeK - 1) / (kLeBlock * kLeK);
            const unsigned hgrid = (unsigned)std::min<uint64_t>(
                hblocks, (uint64_t)g->num_sms * g->le_heavy_blocks);
            k_le_heavy<kLeBlock, kLeK><<<hgrid, kLeBlock, 0, g->stream>>>(
                g->off, g->E, dist, Hk, Hs, level, T, cap - 1, limit, FB, next_dist, Lk, Ld,
                g->ctr);
          }
        }
        PSC_CUDA(cudaGetLastError());
        PSC_TRY(read_counters(g));
        if (g->hctr[0].fail == 0) break;
        if (exact) return PSC_ERR_TABLE_FULL;  // load <= 1/2 without a probe limit: unreachable
        // the next frontier and the list keep this attempt's new pairs; the
        // heavy list is rebuilt
        PSC_TRY(grow(p2(2 * (ne + bound) + 1024), nf, g->hctr[0].next));
        PSC_CUDA(cudaMemsetAsync(&g->ctr->heavy, 0, 2 * sizeof(unsigned long long), g->stream));
        exact = true;
      }
      if (trace_on()) {  // ms since the start of the call (the stream is idle here)
        float ms = 0;
        cudaEvent_t ev = take_event(g);
        PSC_CUDA(cudaEventRecord(ev, g->stream));
        PSC_CUDA(cudaEventSynchronize(ev));
        cudaEventElapsedTime(&ms, g->t0, ev);
        give_event(g, ev);
        std::fprintf(stderr, "le batch %llu [%llu,%llu) level %u nf %llu edges %llu new %llu "
                     "probes %llu cap %llu attempts %u t %.3f ms\n",
                     (unsigned long long)g->stats.batches, (unsigned long long)start,
                     (unsigned long long)end, level, (unsigned long long)nf,
                     g->hctr[0].edges, g->hctr[0].next, g->hctr[0].probes,
                     (unsigned long long)cap, attempts, ms);
      }
      const uint64_t added = g->hctr[0].next;
      if (g->profiling)  // 8 per pair + 16 per range, 8 per edge (id,
                         // distance), 8 per probe, 16 per new pair (list entry)
        g->prof[F_LE].bytes += 24.0 * nf + 8.0 * g->hctr[0].edges + 8.0 * g->hctr[0].probes +
                               16.0 * added;
      ratio_next.push_back((double)added / (double)std::max<uint64_t>(bound, 1));
      ne += added;
      L += added;
      bound = g->hctr[0].next_edges;
      std::swap(FA, FB);
      swap_bufs(g, B_PA, B_PB);
      nf = added;
    }
    ratio.swap(ratio_next);
    PSC_CUDA(cudaMemcpyAsync(dist, next_dist, n * 4, cudaMemcpyDeviceToDevice, g->stream));
    prev_ne = (uint64_t)std::ceil((double)ne * beta);
    finished = end;
  }
  // bucket by target, sort by priority, filter, emit triples
  uint64_t* Lk = (uint64_t*)g->bufs[B_PH].p;
  uint32_t* Ld = (uint32_t*)g->bufs[B_AUX3].p;
  uint64_t *boff, *Bk;
  uint32_t *cursor, *tgt;
  uint8_t* keep;
  PSC_TRY(ensure_t(g, B_TMP32, n + 1, &cnt));
  PSC_TRY(ensure_t(g, B_CENTERS, n + 2, &cursor));
  PSC_TRY(ensure_t(g, B_FRONT, n + 2, &boff));
  PSC_TRY(ensure_t(g, B_TB, L + 1, &Bk));
  PSC_TRY(ensure_t(g, B_TS, L + 1, &keep));
  PSC_TRY(ensure_t(g, B_P, L + 1, &tgt));
  PSC_CUDA(cudaMemsetAsync(cnt, 0, (n + 1) * 4, g->stream));
  {
    ProfScope ps(g, F_LE_SORT);
    ps.bytes = 8.0 * L;
    k_le_count<<<grid_for(g, L, tb), tb, 0, g->stream>>>(Lk, L, cnt);
  }
  PSC_TRY(scan_emit(g, n, CountValue{cnt}, BucketOffsets{boff, cursor}, nullptr, F_LE_SORT));
  g->hctr[3].aux1 = L;  // boff[n] = L (pinned staging word)
  PSC_CUDA(cudaMemcpyAsync(boff + n, &g->hctr[3].aux1, 8, cudaMemcpyHostToDevice, g->stream));
  {
    ProfScope ps(g, F_LE_SORT);
    ps.bytes = 20.0 * L;
    k_le_scatter<<<grid_for(g, L, tb), tb, 0, g->stream>>>(Lk, Ld, L, boff, cursor, Bk);
  }
  uint32_t* big;
  PSC_TRY(ensure_t(g, B_QA, n + 1, &big));
  PSC_TRY(zero_counters(g));
  {
    ProfScope ps(g, F_LE_SORT);
    ps.bytes = 8.0 * n + 16.0 * L;
    k_seg_sort_small<<<grid_for(g, n, tb), tb, 0, g->stream>>>(boff, n, Bk, big, g->ctr);
  }
  PSC_TRY(read_counters(g));
  const uint64_t maxlen = g->hctr[0].aux0, nbig = g->hctr[0].heavy;
  uint64_t pad = 64;
  while (pad < maxlen) pad <<= 1;
  const unsigned sgrid = (unsigned)std::min<uint64_t>(nbig, (uint64_t)g->num_sms * 8);
  uint64_t* scratch = nullptr;
  uint64_t slen = 0;
  if (pad > (uint64_t)kSegSmem) {
    slen = pad;
    PSC_TRY(ensure_t(g, B_AUX2, slen * sgrid, &scratch));
  }
  {
    ProfScope ps(g, F_LE_SORT);
    ps.bytes = 16.0 * n + 9.0 * L;  // bucket bounds, the filter's pass and keep flags
    if (nbig)
      k_seg_sort_u64<<<sgrid, kSegBlock, 0, g->stream>>>(big, nbig, boff, Bk, scratch, slen);
    k_le_filter<<<grid_for(g, n, tb), tb, 0, g->stream>>>(boff, n, Bk, keep);
    k_le_target<<<grid_for(g, n, tb), tb, 0, g->stream>>>(boff, n, tgt);
  }
  uint32_t* out;
  PSC_TRY(ensure_t(g, B_AUX0, 3 * L + 3, &out));
  uint64_t kept = 0;
  PSC_TRY(scan_emit_flags(g, L, KeepValue{keep}, TripleEmit{Bk, tgt, centers, out}, &kept,
                          F_LE_SORT));
  *len_out = kept;
  return PSC_OK;
}

}  // namespace psc

using namespace psc;

extern "C" int psc_bfs(psc_graph_t g, uint32_t src, uint32_t* dist_out, uint32_t* rounds) {
  if (!g || !dist_out || src >= g->n) return PSC_ERR_INVALID;
  PSC_TRY(call_begin(g));
  uint32_t* d;
  PSC_TRY(ensure_t(g, B_TMP32, g->n + 1, &d));
  uint32_t r = 0;
  PSC_TRY(bfs_run(g, src, d, &r));
  PSC_CUDA(cudaMemcpyAsync(dist_out, d, g->n * 4, cudaMemcpyDeviceToHost, g->stream));
  g->stats.reach_rounds = r;
  if (rounds) *rounds = r;
  return call_end(g);
}

extern "C" int psc_lelist(psc_graph_t g, const uint32_t* perm, double beta, uint32_t* out,
                          uint64_t cap, uint64_t* len) {
  if (!g || !perm || !len || !(beta > 0) || (cap && !out)) return PSC_ERR_INVALID;
  PSC_TRY(call_begin(g));
  uint32_t* centers;
  // the priority order lives in the pivot slot (u32[n])
  PSC_TRY(ensure_t(g, B_HEAVY2, g->n + 1, &centers));
  PSC_CUDA(cudaMemcpyAsync(centers, perm, g->n * 4, cudaMemcpyHostToDevice, g->stream));
  uint64_t L = 0;
  PSC_TRY(lelist_run(g, centers, beta, &L));
  *len = L;
  if (L > cap) {
    PSC_TRY(call_end(g));
    return PSC_ERR_CAPACITY;
  }
  if (L)
    PSC_CUDA(cudaMemcpyAsync(out, g->bufs[B_AUX0].p, L * 12, cudaMemcpyDeviceToHost, g->stream));
  return call_end(g);
}

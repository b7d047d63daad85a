// Connectivity on the device (src/Connectivity.h:37-119): a low-diameter
// decomposition followed by union-find over the edges that leave the largest
// cluster.  The input graph is symmetric (as the reference requires).
//
// LDD (src/ldd.hpp:325-417) as an exponential-shift multi-source BFS: 1024
// candidate centres hash32(1024 + i) % n are fixed up front; round r adds the
// next floor(exp(r * beta)) of them that are still unlabelled, and every round
// grows all clusters by one hop — a frontier vertex u offers label[u] to its
// neighbours, and atomicCAS(label[v], NONE, label[u]) lets the first offer
// win (the reference's compare_and_swap, ldd.hpp:226,253).  Rounds switch
// between push (queue) and pull (bitmap) by the reference's rule.  Vertices
// no cluster reaches are their own centre.
//
// Union-find (union_find_rules.h) as hook-and-compress: parent = LDD label;
// for every vertex outside the most frequent cluster (get_max_label,
// Connectivity.h:13-35, 10^4 hashed samples), every edge runs the lock-free
// unite: find both roots with path halving, link the larger root under the
// smaller with atomicCAS, retry on contention.  A final pass compresses every
// vertex to its root.  Spanning forest: the LDD tree edges (v, parent[v]) plus
// the edges whose unite linked two trees (Connectivity.h:99-117).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cstdio>

#include "common.cuh"
#include "engines.cuh"
#include "scan.cuh"

namespace psc {

constexpr int kCcBlock = 256;
constexpr int kLddSamples = 1024;   // ldd.hpp:462
constexpr int kMaxLabelSamples = 10000;  // Connectivity.h:14

__global__ void k_cc_init(uint32_t* label, uint32_t* parent, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    label[i] = kNone;
    if (parent) parent[i] = (uint32_t)i;
  }
}

// New centres perm[start .. start+count): claim the unlabelled ones and add
// them to the frontier (queue, or bitmap in pull mode).
__global__ void k_ldd_centres(const uint32_t* __restrict__ perm, uint32_t start, uint32_t count,
                              uint32_t* label, uint32_t* q, uint32_t* fb, Counters* ctr) {
  const unsigned lane = lane_id();
  for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < count;
       base += gridDim.x * blockDim.x) {
    const uint32_t i = base + lane;
    bool take = false;
    uint32_t c = 0;
    if (i < count) {
      c = perm[start + i];
      take = atomicCAS(&label[c], kNone, c) == kNone;
    }
    if (fb) {
      if (take) atomicOr(&fb[c >> 5], 1u << (c & 31));
      const unsigned m = __ballot_sync(kFull, take);
      if (lane == 0 && m) atomicAdd(&ctr->next, (unsigned long long)__popc(m));
    } else {
      unsigned long long pos = warp_append(&ctr->next, take);
      if (take) q[pos] = c;
    }
  }
}

// Big frontier vertices of an LDD round (out-degree >= the VGC queue size),
// listed by k_ldd_vgc with one 64-bit atomic on ctr->heavy = count <<
// kLddPackShift | chunks that gives each entry (vertex << 32 | first chunk)
// its slot and its first chunk of kLddChunk edges, increasing with the slot.
// The chunks of all entries are cut into one contiguous range per warp of the
// grid; a warp finds the entry of its first chunk once, then offers its
// vertex's label to kLddChunk edges per step (atomicCAS from NONE, as in the
// other LDD rounds).  A hub's edges are spread over the whole grid instead of
// one warp.  Field widths: count < 2^30, chunks < 2^34 (m < 2^36).
constexpr int kLddHeavyK = 4;
constexpr uint64_t kLddChunk = 32 * kLddHeavyK;
constexpr int kLddPackShift = 34;
constexpr uint64_t kLddPackMask = (1ull << kLddPackShift) - 1;

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    k_ldd_heavy(const uint64_t* __restrict__ off, const uint32_t* __restrict__ E,
                const uint64_t* __restrict__ big, uint32_t* label, uint32_t* parent,
                uint32_t* qout, Counters* ctr) {
  constexpr int K = kLddHeavyK;
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  const unsigned long long packed = ctr->heavy;
  const uint64_t nh = packed >> kLddPackShift, total = packed & kLddPackMask;
  const uint64_t per = (total + nw - 1) / nw;
  const uint64_t c_beg = gw * per, c_end = c_beg + per < total ? c_beg + per : total;
  if (nh == 0 || c_beg >= c_end) return;
  uint64_t h = 0, hi = nh - 1;  // last entry whose first chunk is <= c_beg
  while (h < hi) {
    const uint64_t mid = (h + hi + 1) >> 1;
    if ((uint32_t)__ldg(&big[mid]) <= c_beg)
      h = mid;
    else
      hi = mid - 1;
  }
  uint64_t ent = __ldg(&big[h]);
  uint64_t cs = (uint32_t)ent, cn = h + 1 < nh ? (uint32_t)__ldg(&big[h + 1]) : total;
  uint32_t u = (uint32_t)(ent >> 32), lu = label[u];
  uint64_t beg = off[u], end = off[u + 1];
  unsigned long long scanned = 0, next_edges = 0;
  for (uint64_t c = c_beg; c < c_end; c++) {
    if (c >= cn) {
      h++;
      ent = __ldg(&big[h]);
      cs = cn;
      cn = h + 1 < nh ? (uint32_t)__ldg(&big[h + 1]) : total;
      u = (uint32_t)(ent >> 32);
      lu = label[u];
      beg = off[u];
      end = off[u + 1];
    }
    const uint64_t e0 = beg + (c - cs) * kLddChunk;
    uint32_t v[K], tm = 0, pre = 0;
#pragma unroll
    for (int k = 0; k < K; k++) {
      const uint64_t e = e0 + k * 32 + lane;
      v[k] = kNone;
      if (e < end) {
        scanned++;
        v[k] = __ldg(&E[e]);
      }
    }
#pragma unroll
    for (int k = 0; k < K; k++)
      if (v[k] != kNone && __ldcg(&label[v[k]]) == kNone) pre |= 1u << k;
#pragma unroll
    for (int k = 0; k < K; k++)
      if ((pre & (1u << k)) && atomicCAS(&label[v[k]], kNone, lu) == kNone) {
        tm |= 1u << k;
        if (parent) parent[v[k]] = u;
      }
    warp_append_batch<K>(tm, v, qout, &ctr->next);
#pragma unroll
    for (int k = 0; k < K; k++)
      if (tm & (1u << k)) next_edges += off[v[k] + 1] - off[v[k]];
  }
  scanned = warp_sum(scanned);
  next_edges = warp_sum(next_edges);
  if (lane == 0) {
    if (scanned) atomicAdd(&ctr->edges, scanned);
    if (next_edges) atomicAdd(&ctr->next_edges, next_edges);
  }
}

// VGC round (the reference's sparse_update with its local queue,
// ldd.hpp:88-161): each warp takes a chunk of up to `chunk` frontier
// vertices (one while the frontier fits the grid, up to 32 when it is much
// larger).  A chunk vertex with 0 < deg < tq seeds a local BFS in the warp's
// shared-memory queue of tq = min(tau, kLddQueue) entries: each wave takes up
// to 32 queued vertices, offers each one's label along its edges (balanced
// expansion, kLddK edges per lane in flight, atomicCAS from NONE), keeps the
// vertices it claims in the queue while there is room and spills the rest to
// the next frontier, as is whatever is left when the queue fills.  Queued
// vertices with deg > tq spill too; chunk vertices with deg >= tq go to the
// `big` list, whose edges k_ldd_heavy spreads over the grid afterwards.
constexpr int kLddQueue = 512;
constexpr int kLddVgcBlock = 128;
constexpr int kLddK = 8;

struct LEnt {
  uint64_t beg;
  uint32_t v;
  uint32_t deg;
};

template <int BLOCK, int QCAP>
__global__ void __launch_bounds__(BLOCK)
    k_ldd_vgc(const uint64_t* __restrict__ off, const uint32_t* __restrict__ E,
              const uint32_t* __restrict__ qin, uint64_t nin, uint32_t* label, uint32_t* parent,
              uint32_t* qout, uint64_t* big, uint32_t tau, uint32_t chunk, Counters* ctr) {
  __shared__ WarpExpandSmem sm[BLOCK / 32];
  __shared__ LEnt sq[BLOCK / 32][QCAP];
  __shared__ uint32_t slab[BLOCK / 32][QCAP];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  const uint32_t tq = tau < (uint32_t)QCAP ? tau : (uint32_t)QCAP;
  uint32_t C = chunk < tq ? chunk : tq;
  C = C < 1 ? 1 : C > 32 ? 32 : C;
  LEnt* Q = sq[wid];
  uint32_t* QL = slab[wid];
  unsigned long long scanned = 0, next_edges = 0;
  const uint64_t nchunks = (nin + C - 1) / C;
  for (uint64_t c = gw; c < nchunks; c += nw) {
    const uint64_t first = c * C;
    const uint64_t left = nin - first;
    const uint32_t cnt = left < C ? (uint32_t)left : C;
    uint32_t u = 0, lu = 0;
    uint64_t ub = 0, du = 0;
    if (lane < cnt) {
      u = qin[first + lane];
      ub = off[u];
      du = off[u + 1] - ub;
      lu = label[u];
    }
    if (lane < cnt && du >= tq) {
      const unsigned long long old = atomicAdd(
          &ctr->heavy, (1ull << kLddPackShift) + (du + kLddChunk - 1) / kLddChunk);
      big[old >> kLddPackShift] = ((uint64_t)u << 32) | (old & kLddPackMask);
    }
    const bool seed = lane < cnt && du > 0 && du < tq;
    const uint32_t smask = __ballot_sync(kFull, seed);
    if (seed) {
      const uint32_t at = __popc(smask & ((1u << lane) - 1));
      Q[at] = LEnt{ub, u, (uint32_t)du};
      QL[at] = lu;
    }
    __syncwarp();
    uint32_t head = 0, tail = __popc(smask);
    while (head < tail && (head == 0 || tail < tq)) {
      const uint32_t wave = min(32u, tail - head);
      uint64_t beg = 0;
      uint32_t deg = 0, x = 0, xl = 0, xdeg = 0;
      bool spill_self = false;
      if (lane < wave) {
        const LEnt q = Q[head + lane];
        x = q.v;
        xl = QL[head + lane];
        beg = q.beg;
        deg = q.deg;
        xdeg = q.deg;
        if (deg > tq) {
          spill_self = true;
          deg = 0;
        }
      }
      head += wave;
      __syncwarp();
      if (__any_sync(kFull, spill_self)) {
        const unsigned long long pos = warp_append(&ctr->next, spill_self);
        if (spill_self) {
          qout[pos] = x;
          next_edges += xdeg;
        }
      }
      scanned += deg;
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
      for (uint32_t base = 0; base < total; base += 32 * kLddK) {
        uint32_t w[kLddK], wl[kLddK], wp[kLddK];
        uint64_t vb[kLddK], ve[kLddK];
#pragma unroll
        for (int k = 0; k < kLddK; k++) {
          const uint32_t gi = base + k * 32 + lane;
          w[k] = kNone;
          wl[k] = 0;
          wp[k] = 0;
          if (gi < total) {
            int lo = 0, hi = 31;
            while (lo < hi) {
              const int mid = (lo + hi + 1) >> 1;
              if (sm[wid].excl[mid] <= gi)
                lo = mid;
              else
                hi = mid - 1;
            }
            w[k] = __ldg(&E[sm[wid].beg[lo] + (gi - sm[wid].excl[lo])]);
            wl[k] = QL[head - wave + lo];
            wp[k] = Q[head - wave + lo].v;
          }
        }
        // claims: the adjacency range is loaded alongside (used if claimed)
        uint32_t tm = 0;
#pragma unroll
        for (int k = 0; k < kLddK; k++) {
          vb[k] = ve[k] = 0;
          if (w[k] != kNone && __ldcg(&label[w[k]]) == kNone) {
            vb[k] = __ldg(&off[w[k]]);
            ve[k] = __ldg(&off[w[k] + 1]);
            tm |= 1u << k;
          }
        }
#pragma unroll
        for (int k = 0; k < kLddK; k++)
          if (tm & (1u << k)) {
            if (atomicCAS(&label[w[k]], kNone, wl[k]) == kNone) {
              if (parent) parent[w[k]] = wp[k];
            } else {
              tm &= ~(1u << k);
            }
          }
        // place: into the queue while it has room, then spill
        const uint32_t cntk = __popc(tm);
        uint32_t inc = cntk;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t t = __shfl_up_sync(kFull, inc, o);
          if ((int)lane >= o) inc += t;
        }
        const uint32_t tot = __shfl_sync(kFull, inc, 31);
        if (tot) {
          const uint32_t room = tail < tq ? tq - tail : 0;
          const uint32_t nloc = tot < room ? tot : room;
          unsigned long long sbase = 0;
          if (tot > nloc && lane == 0) sbase = atomicAdd(&ctr->next, (unsigned long long)(tot - nloc));
          sbase = __shfl_sync(kFull, sbase, 0);
          uint32_t r = inc - cntk;
#pragma unroll
          for (int k = 0; k < kLddK; k++)
            if (tm & (1u << k)) {
              const uint64_t vd = ve[k] - vb[k];
              if (r < nloc) {
                Q[tail + r] = LEnt{vb[k], w[k], (uint32_t)(vd < 0xFFFFFFFFull ? vd : 0xFFFFFFFFull)};
                QL[tail + r] = wl[k];
              } else {
                qout[sbase + (r - nloc)] = w[k];
                next_edges += vd;
              }
              r++;
            }
          tail += nloc;
          __syncwarp();
        }
      }
    }
    // spill what is left in the queue with one reservation
    const uint32_t rem = tail - head;
    if (rem) {
      unsigned long long b0 = 0;
      if (lane == 0) b0 = atomicAdd(&ctr->next, (unsigned long long)rem);
      b0 = __shfl_sync(kFull, b0, 0);
      for (uint32_t k = lane; k < rem; k += 32) {
        qout[b0 + k] = Q[head + k].v;
        next_edges += Q[head + k].deg;
      }
    }
    __syncwarp();
  }
  scanned = warp_sum(scanned);
  next_edges = warp_sum(next_edges);
  if (lane == 0) {
    if (scanned) atomicAdd(&ctr->edges, scanned);
    if (next_edges) atomicAdd(&ctr->next_edges, next_edges);
  }
}

// Pull round (ldd.hpp:163-247): every unlabelled vertex takes the label of
// its first neighbour in the frontier bitmap.  A warp owns 32 consecutive
// vertices and writes their next-frontier word with one store.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    k_ldd_pull(const uint64_t* __restrict__ off, const uint32_t* __restrict__ E,
               const uint32_t* __restrict__ fb_in, uint32_t* label, uint32_t* parent,
               uint32_t* fb_out, uint64_t n, Counters* ctr) {
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  const uint64_t nwords = (n + 31) >> 5;
  unsigned long long cnt = 0, scanned = 0, next_edges = 0;
  for (uint64_t w = gw; w < nwords; w += nw) {
    const uint64_t v = w * 32 + lane;
    bool found = false;
    if (v < n && label[v] == kNone) {
      const uint64_t b = off[v], e = off[v + 1];
      uint64_t j = b;
      for (; j < e; j++) {
        const uint32_t x = __ldg(&E[j]);
        if ((__ldg(&fb_in[x >> 5]) >> (x & 31)) & 1u) {
          label[v] = label[x];
          if (parent) parent[v] = x;
          found = true;
          break;
        }
      }
      scanned += (found ? j + 1 : j) - b;
      if (found) next_edges += e - b;
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

__global__ void k_cc_queue_to_bitmap(const uint32_t* __restrict__ q, uint64_t nq, uint32_t* fb) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nq;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t v = q[i];
    atomicOr(&fb[v >> 5], 1u << (v & 31));
  }
}

__global__ void k_cc_bitmap_to_queue(const uint32_t* __restrict__ fb, uint64_t nwords, uint32_t* q,
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

__global__ void k_set_u64(unsigned long long* p, unsigned long long v) { *p = v; }

__global__ void k_ldd_finish(uint32_t* label, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    if (label[i] == kNone) label[i] = (uint32_t)i;
}

__global__ void k_sample_labels(const uint32_t* __restrict__ label, const uint32_t* __restrict__ idx,
                                uint32_t count, uint32_t* out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    out[i] = label[idx[i]];
}

// find with path halving (union_find_rules.h:80-90, split/halve variants)
__device__ __forceinline__ uint32_t uf_find(uint32_t* p, uint32_t x) {
  uint32_t px = __ldcg(&p[x]);
  while (px != x) {
    const uint32_t gx = __ldcg(&p[px]);
    if (gx != px) atomicCAS(&p[x], px, gx);
    x = px;
    px = gx;
  }
  return x;
}

// Unite over the edges [first, last) of the adjacency list of every vertex
// whose root is not max_root (Connectivity.h:74-93).  Link the larger root
// under the smaller (UniteRemCAS links high -> low,
// union_find_rules.h:193-225).
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    k_uf_edges(const uint64_t* __restrict__ off, const uint32_t* __restrict__ E, uint64_t n,
               uint32_t* parent, const uint32_t* __restrict__ cluster, uint32_t max_root,
               const uint32_t* __restrict__ gid, const uint32_t* __restrict__ groot,
               uint32_t first, uint32_t last, uint32_t* forest, Counters* ctr) {
  __shared__ WarpExpandSmem sm[BLOCK / 32];
  __shared__ uint32_t s_u[BLOCK];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  unsigned long long scanned = 0;
  for (uint64_t base = gw * 32; base < n; base += nw * 32) {
    const uint64_t i = base + lane;
    uint64_t beg = 0, rem = 0;
    if (i < n && uf_find(parent, (uint32_t)i) != (gid ? groot[gid[i]] : max_root)) {
      const uint64_t b = off[i], d = off[i + 1] - b;
      const uint64_t lo = d < first ? d : first, hi = d < last ? d : last;
      beg = b + lo;
      rem = hi - lo;
    }
    scanned += rem;
    s_u[wid * 32 + lane] = (uint32_t)i;
    // adjacency lists in pieces of at most 2^26 edges (32-bit warp scan)
    while (__any_sync(kFull, rem > 0)) {
      const uint32_t piece = (uint32_t)(rem < (1ull << 26) ? rem : (1ull << 26));
      warp_expand(sm[wid], beg, piece, [&](bool act, int s, uint64_t e) {
        bool linked = false;
        uint32_t x = 0, y = 0;
        // an edge inside one LDD cluster joins nothing (both ends already
        // share the cluster's centre as an ancestor)
        if (act) {
          x = s_u[wid * 32 + s];
          y = __ldg(&E[e]);
          if (__ldg(&cluster[y]) == __ldg(&cluster[x])) act = false;
        }
        if (act) {
          for (;;) {
            uint32_t rx = uf_find(parent, x), ry = uf_find(parent, y);
            if (rx == ry) break;
            if (rx < ry) {
              const uint32_t t = rx;
              rx = ry;
              ry = t;
            }
            if (atomicCAS(&parent[rx], rx, ry) == rx) {
              linked = true;
              break;
            }
          }
        }
        if (forest) {
          const unsigned long long pos = warp_append(&ctr->aux1, linked);
          if (linked) {
            forest[2 * pos] = x;
            forest[2 * pos + 1] = y;
          }
        }
      });
      beg += piece;
      rem -= piece;
    }
    __syncwarp();
  }
  scanned = warp_sum(scanned);
  if (lane == 0 && scanned) atomicAdd(&ctr->edges, scanned);
}

__global__ void k_uf_final(uint32_t* parent, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    parent[i] = uf_find(parent, (uint32_t)i);
}

// Most frequent LDD label among kGraphSamples hashed samples of each graph of
// a batch (ties to the smallest label, as the single-graph scan of sorted
// samples): one block per graph, a bitonic sort in shared memory.
constexpr int kGraphSamples = 256;

__global__ void __launch_bounds__(kGraphSamples)
    k_graph_modes(const uint32_t* __restrict__ label, const uint64_t* __restrict__ mbase,
                  const uint64_t* __restrict__ msize, const uint32_t* __restrict__ mk,
                  uint32_t* groot) {
  __shared__ uint32_t a[kGraphSamples];
  const uint32_t t = threadIdx.x;
  const uint64_t b = mbase[blockIdx.x], sz = msize[blockIdx.x];
  const uint64_t seed = hash64(sz + 1);
  a[t] = label[b + hash64(t + seed) % sz];
  __syncthreads();
  for (uint32_t k = 2; k <= (uint32_t)kGraphSamples; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      const uint32_t p = t ^ j;
      if (p > t) {
        const uint32_t x = a[t], y = a[p];
        if ((x > y) == ((t & k) == 0)) {
          a[t] = y;
          a[p] = x;
        }
      }
      __syncthreads();
    }
  }
  if (t == 0) {
    uint32_t best = a[0], best_cnt = 0;
    for (uint32_t i = 0; i < (uint32_t)kGraphSamples;) {
      uint32_t j = 1;
      while (i + j < (uint32_t)kGraphSamples && a[i + j] == a[i]) j++;
      if (j > best_cnt) {
        best_cnt = j;
        best = a[i];
      }
      i += j;
    }
    groot[mk[blockIdx.x]] = best;
  }
}

// Roots of the given labels after a compressing pass: groot[k] = label[groot[k]].
__global__ void k_gather_roots(const uint32_t* __restrict__ label, const uint32_t* __restrict__ mk,
                               uint32_t count, uint32_t* groot) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += gridDim.x * blockDim.x)
    groot[mk[j]] = label[groot[mk[j]]];
}

// LDD tree edges (v, parent[v]) for v != parent[v], appended to the forest.
__global__ void k_ldd_tree_edges(const uint32_t* __restrict__ tree, uint64_t n, uint32_t* forest,
                                 Counters* ctr) {
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n;
       base += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = base + lane_id();
    const bool t = i < n && tree[i] != (uint32_t)i;
    const unsigned long long pos = warp_append(&ctr->aux1, t);
    if (t) {
      forest[2 * pos] = (uint32_t)i;
      forest[2 * pos + 1] = tree[i];
    }
  }
}

// Graphs of a batch with at least one vertex (the whole graph when the
// handle holds no batch): their vertex bases and sizes.
static void ldd_members(const psc_graph_s* g, std::vector<uint64_t>& base,
                        std::vector<uint64_t>& size) {
  base.clear();
  size.clear();
  if (g->num_graphs > 1) {
    for (uint32_t k = 0; k < g->num_graphs; k++)
      if (g->vbase[k + 1] > g->vbase[k]) {
        base.push_back(g->vbase[k]);
        size.push_back(g->vbase[k + 1] - g->vbase[k]);
      }
  } else {
    base.push_back(0);
    size.push_back(g->n);
  }
}

// LDD into d_label (centre ids); tree (optional) receives BFS parents.  In a
// batch every graph draws its own candidate centres (hash32(1024 + i) % n_k,
// as a graph alone would) and all graphs add them on the same schedule, so
// the centre list is laid out sample-major: entry i * G + k.
int ldd_run(psc_graph_s* g, double beta, uint32_t* d_label, uint32_t* tree) {
  const uint64_t n = g->n, m = g->m, nwords = (n + 31) / 32;
  if (m >> 36) return PSC_ERR_TOO_LARGE;  // big-list fields (k_ldd_heavy)
  const unsigned tb = kCcBlock;
  std::vector<uint64_t> mb, ms;
  ldd_members(g, mb, ms);
  const uint64_t G = mb.size();
  const uint64_t ncent = (uint64_t)kLddSamples * G;
  uint32_t *qa, *qb, *fa, *fb, *perm, *samp_idx, *samp;
  PSC_TRY(ensure_t(g, B_QA, n + ncent + 1, &qa));
  PSC_TRY(ensure_t(g, B_QB, n + ncent + 1, &qb));
  PSC_TRY(ensure_t(g, B_FB_A, nwords + 1, &fa));
  PSC_TRY(ensure_t(g, B_FB_B, nwords + 1, &fb));
  PSC_TRY(ensure_t(g, B_AUX2, ncent + 2 * kMaxLabelSamples, &perm));
  samp_idx = perm + ncent;
  samp = samp_idx + kMaxLabelSamples;
  // centres and label samples, hashed on the host (ldd.hpp:463-466,
  // Connectivity.h:16-20)
  std::vector<uint32_t> hp(ncent + kMaxLabelSamples);
  for (int i = 0; i < kLddSamples; i++)
    for (uint64_t k = 0; k < G; k++)
      hp[(uint64_t)i * G + k] = (uint32_t)(mb[k] + hash32(kLddSamples + i) % ms[k]);
  const uint64_t seed = hash64(n + 1);
  for (int i = 0; i < kMaxLabelSamples; i++) hp[ncent + i] = (uint32_t)(hash64(i + seed) % n);
  PSC_CUDA(cudaMemcpyAsync(perm, hp.data(), hp.size() * 4, cudaMemcpyHostToDevice, g->stream));
  {
    ProfScope ps(g, F_CC);
    k_cc_init<<<grid_for(g, n, tb), tb, 0, g->stream>>>(d_label, tree, n);
  }
  const uint64_t threshold = m / 20;
  uint64_t nf = 0, nf_edges = 0;
  uint32_t sampled = 0, round = 0;
  bool pull = false;
  g->ldd_trace.clear();
  while (nf > 0 || sampled < (uint32_t)kLddSamples) {
    round++;
    if (round > n + kLddSamples + 2) return PSC_ERR_ITER_LIMIT;
    const double stepf = std::floor(std::exp((double)round * beta));
    const uint32_t work = (uint32_t)std::min<double>(stepf, (double)(kLddSamples - sampled));
    uint32_t new_centres = 0;
    const uint32_t first = sampled;
    if (work > 0) {
      // new centres join the frontier: appended after the nf queued vertices
      // (counter block 1 is the queue cursor) or set in the frontier bitmap
      PSC_TRY(zero_counters(g));
      k_set_u64<<<1, 1, 0, g->stream>>>(&g->ctr[1].next, pull ? 0ull : (unsigned long long)nf);
      ProfScope ps(g, F_CC);
      k_ldd_centres<<<grid_for(g, work * G, 256), 256, 0, g->stream>>>(
          perm, (uint32_t)(sampled * G), (uint32_t)(work * G), d_label, pull ? nullptr : qa,
          pull ? fa : nullptr, g->ctr + 1);
      sampled += work;
      PSC_TRY(read_counters(g));
      new_centres = (uint32_t)(pull ? g->hctr[1].next : g->hctr[1].next - nf);
      nf = pull ? nf + g->hctr[1].next : g->hctr[1].next;
    }
    g->ldd_trace.insert(g->ldd_trace.end(), {first, work, new_centres});
    if (nf == 0) continue;
    const bool want_pull = (nf + nf_edges) >= threshold;
    if (want_pull && !pull) {
      PSC_CUDA(cudaMemsetAsync(fa, 0, nwords * 4, g->stream));
      k_cc_queue_to_bitmap<<<grid_for(g, nf, 256), 256, 0, g->stream>>>(qa, nf, fa);
      pull = true;
    } else if (!want_pull && pull) {
      PSC_TRY(zero_counters(g));
      k_cc_bitmap_to_queue<<<grid_for(g, nwords, 256), 256, 0, g->stream>>>(fa, nwords, qa, g->ctr);
      pull = false;
    }
    PSC_TRY(zero_counters(g));
    if (!pull) {
      // VGC round on a resident grid, then the big-degree frontier vertices
      // it set aside, their edges cut into chunks over the whole grid, into
      // the same queue
      if (!g->ldd_vgc_blocks) {
        PSC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &g->ldd_vgc_blocks, k_ldd_vgc<kLddVgcBlock, kLddQueue>, kLddVgcBlock, 0));
        if (g->ldd_vgc_blocks < 1) g->ldd_vgc_blocks = 1;
      }
      const uint64_t max_blocks = (uint64_t)g->num_sms * g->ldd_vgc_blocks;
      const uint64_t max_warps = max_blocks * (kLddVgcBlock / 32);
      const uint64_t chunk = std::min<uint64_t>(32, (nf + max_warps - 1) / max_warps);
      const uint64_t chunks = (nf + chunk - 1) / chunk;
      const uint64_t blocks =
          std::min(max_blocks, (chunks + kLddVgcBlock / 32 - 1) / (kLddVgcBlock / 32));
      uint64_t* big;
      PSC_TRY(ensure_t(g, B_HEAVY, n + 1, &big));
      {
        ProfScope ps(g, F_CC);
        k_ldd_vgc<kLddVgcBlock, kLddQueue>
            <<<(unsigned)std::max<uint64_t>(1, blocks), kLddVgcBlock, 0, g->stream>>>(
                g->off, g->E, qa, nf, d_label, tree, qb, big, kLddQueue, (uint32_t)chunk, g->ctr);
      }
      PSC_CUDA(cudaGetLastError());
      PSC_TRY(read_counters(g));
      if (g->hctr[0].heavy >> kLddPackShift) {
        ProfScope ps(g, F_CC);
        k_ldd_heavy<kCcBlock><<<g->num_sms * 4, kCcBlock, 0, g->stream>>>(
            g->off, g->E, big, d_label, tree, qb, g->ctr);
      }
      std::swap(qa, qb);
      swap_bufs(g, B_QA, B_QB);
    } else {
      ProfScope ps(g, F_CC);
      k_ldd_pull<kCcBlock><<<grid_for(g, nwords * 32, tb), tb, 0, g->stream>>>(
          g->off, g->E, fa, d_label, tree, fb, n, g->ctr);
      std::swap(fa, fb);
      swap_bufs(g, B_FB_A, B_FB_B);
    }
    PSC_CUDA(cudaGetLastError());
    PSC_TRY(read_counters(g));
    if (trace_on()) {  // ms since the start of the call (the stream is idle here)
      cudaEvent_t ev = take_event(g);
      PSC_CUDA(cudaEventRecord(ev, g->stream));
      PSC_CUDA(cudaEventSynchronize(ev));
      float ms = 0;
      cudaEventElapsedTime(&ms, g->t0, ev);
      give_event(g, ev);
      std::fprintf(stderr, "ldd round %u mode %s nf %llu new_centres %u next %llu edges %llu t %.3f ms\n",
                   round, pull ? "pull" : "push", (unsigned long long)nf, new_centres,
                   g->hctr[0].next, g->hctr[0].edges, ms);
    }
    if (g->profiling) {
      // algorithmic bytes: push / VGC: 16 per frontier vertex (range), 8 per
      // edge (target id, label CAS), 8 per new vertex; pull: both bitmaps,
      // 8 per scanned in-edge, 4 per new vertex
      const Counters& c = g->hctr[0];
      g->prof[F_CC].bytes += pull ? 0.25 * n + 8.0 * c.edges + 4.0 * c.next
                                  : 16.0 * nf + 8.0 * c.edges + 8.0 * c.next;
    }
    nf = g->hctr[0].next;
    nf_edges = g->hctr[0].next_edges;
  }
  g->stats.reach_rounds = round;
  {
    ProfScope ps(g, F_CC);
    k_ldd_finish<<<grid_for(g, n, tb), tb, 0, g->stream>>>(d_label, n);
    k_sample_labels<<<grid_for(g, kMaxLabelSamples, 256), 256, 0, g->stream>>>(
        d_label, samp_idx, kMaxLabelSamples, samp);
  }
  PSC_CUDA(cudaGetLastError());
  return PSC_OK;
}

int cc_run(psc_graph_s* g, double beta, uint32_t* d_label, uint32_t* d_forest, uint64_t* n_forest) {
  const uint64_t n = g->n;
  const unsigned tb = kCcBlock;
  uint32_t* tree = nullptr;
  if (d_forest) PSC_TRY(ensure_t(g, B_TMP32, n + 1, &tree));
  PSC_TRY(ldd_run(g, beta, d_label, tree));
  std::vector<uint64_t> mb, ms;
  ldd_members(g, mb, ms);
  const bool batched = g->num_graphs > 1;
  const uint64_t ncent = (uint64_t)kLddSamples * mb.size();
  uint32_t* samp = (uint32_t*)g->bufs[B_AUX2].p + ncent + kMaxLabelSamples;
  uint32_t max_label = 0;
  uint32_t *groot = nullptr, *mk = nullptr;
  const uint32_t G = (uint32_t)mb.size();
  if (batched) {
    // a batch: each graph's most frequent cluster, sampled on the device
    uint64_t* mw;
    PSC_TRY(ensure_t(g, B_GRAPHS, 2 * (size_t)G + (size_t)g->num_graphs + G + 2, &mw));
    groot = (uint32_t*)(mw + 2 * (size_t)G);
    mk = groot + g->num_graphs + 1;
    std::vector<uint64_t> hm(2 * (size_t)G);
    std::vector<uint32_t> hk;
    for (uint32_t k = 0; k < g->num_graphs; k++)
      if (g->vbase[k + 1] > g->vbase[k]) hk.push_back(k);
    std::copy(mb.begin(), mb.end(), hm.begin());
    std::copy(ms.begin(), ms.end(), hm.begin() + G);
    PSC_CUDA(cudaMemcpyAsync(mw, hm.data(), hm.size() * 8, cudaMemcpyHostToDevice, g->stream));
    PSC_CUDA(cudaMemcpyAsync(mk, hk.data(), hk.size() * 4, cudaMemcpyHostToDevice, g->stream));
    ProfScope ps(g, F_UF);
    k_graph_modes<<<G, kGraphSamples, 0, g->stream>>>(d_label, mw, mw + G, mk, groot);
  } else {
    // most frequent sampled label (Connectivity.h:21-33): ties go to the
    // smallest label, as the reference's scan of the sorted samples does
    std::vector<uint32_t> hs(kMaxLabelSamples);
    PSC_CUDA(cudaMemcpyAsync(hs.data(), samp, kMaxLabelSamples * 4, cudaMemcpyDeviceToHost,
                             g->stream));
    PSC_CUDA(cudaStreamSynchronize(g->stream));
    std::sort(hs.begin(), hs.end());
    uint32_t max_cnt = 0;
    for (size_t i = 0; i < hs.size();) {
      size_t j = 1;
      while (i + j < hs.size() && hs[i + j] == hs[i]) j++;
      if (j > max_cnt) {
        max_cnt = (uint32_t)j;
        max_label = hs[i];
      }
      i += j;
    }
  }
  const uint32_t* gid = batched ? g->d_gid : nullptr;
  // LDD labels are centre ids and every centre labels itself, so the label
  // array is already a depth-1 union-find forest; max_label is its own root.
  PSC_TRY(zero_counters(g));
  uint32_t* forest = d_forest;
  if (forest) {
    ProfScope ps(g, F_CC);
    k_ldd_tree_edges<<<grid_for(g, n, 256), 256, 0, g->stream>>>(tree, n, forest, g->ctr);
  }
  // the LDD clusters, kept unchanged while the unions rewrite d_label
  uint32_t* cluster;
  PSC_TRY(ensure_t(g, B_AUX1, n + 1, &cluster));
  PSC_CUDA(cudaMemcpyAsync(cluster, d_label, n * 4, cudaMemcpyDeviceToDevice, g->stream));
  // Two passes over the edges of vertices outside the largest component:
  // first each one's first kUfSample edges (adjacency lists are sorted, so
  // these reach low-id hubs, which join most vertices to the largest
  // component), then, after compressing, the rest of the edges of the
  // vertices still outside it.  Every edge is still offered to the union
  // from one side: an edge skipped on both sides joins two vertices already
  // in the largest component.
  constexpr uint32_t kUfSample = 2;
  // algorithmic bytes of a union pass: per vertex its range, its two labels
  // and its cluster; per offered edge the target id and its label
  auto uf_bytes = [&](unsigned long long edges0) -> int {
    if (!g->profiling) return PSC_OK;
    PSC_TRY(read_counters(g));
    g->prof[F_UF].bytes += 28.0 * n + 8.0 * (g->hctr[0].edges - edges0) + 8.0 * n;
    return PSC_OK;
  };
  {
    ProfScope ps(g, F_UF);
    k_uf_edges<kCcBlock><<<grid_for(g, n, tb), tb, 0, g->stream>>>(
        g->off, g->E, n, d_label, cluster, max_label, gid, groot, 0, kUfSample, forest, g->ctr);
  }
  {
    ProfScope ps(g, F_UF);
    k_uf_final<<<grid_for(g, n, tb), tb, 0, g->stream>>>(d_label, n);
  }
  PSC_TRY(uf_bytes(0));
  const unsigned long long uf_edges1 = g->profiling ? g->hctr[0].edges : 0;
  uint32_t max_root = 0;
  if (batched) {
    ProfScope ps(g, F_UF);
    k_gather_roots<<<(G + 255) / 256, 256, 0, g->stream>>>(d_label, mk, G, groot);
  } else {
    PSC_CUDA(cudaMemcpyAsync(&g->hctr->aux1, d_label + max_label, 4, cudaMemcpyDeviceToHost,
                             g->stream));
    PSC_CUDA(cudaStreamSynchronize(g->stream));
    std::memcpy(&max_root, &g->hctr->aux1, 4);
  }
  {
    ProfScope ps(g, F_UF);
    k_uf_edges<kCcBlock><<<grid_for(g, n, tb), tb, 0, g->stream>>>(
        g->off, g->E, n, d_label, cluster, max_root, gid, groot, kUfSample, 0xFFFFFFFFu, forest,
        g->ctr);
  }
  {
    ProfScope ps(g, F_UF);
    k_uf_final<<<grid_for(g, n, tb), tb, 0, g->stream>>>(d_label, n);
  }
  PSC_TRY(uf_bytes(uf_edges1));
  PSC_CUDA(cudaGetLastError());
  if (trace_on()) {
    cudaEvent_t ev = take_event(g);
    PSC_CUDA(cudaEventRecord(ev, g->stream));
    PSC_CUDA(cudaEventSynchronize(ev));
    float ms = 0;
    cudaEventElapsedTime(&ms, g->t0, ev);
    give_event(g, ev);
    std::fprintf(stderr, "cc union-find done t %.3f ms\n", ms);
  }
  if (n_forest) {
    PSC_TRY(read_counters(g));
    *n_forest = g->hctr[0].aux1;
  }
  return PSC_OK;
}

}  // namespace psc

using namespace psc;

extern "C" int psc_cc(psc_graph_t g, double beta, uint32_t* labels_out, uint32_t* forest_out,
                      uint64_t* n_forest) {
  if (!g || !labels_out || !(beta > 0)) return PSC_ERR_INVALID;
  if ((forest_out == nullptr) != (n_forest == nullptr)) return PSC_ERR_INVALID;
  PSC_TRY(call_begin(g));
  uint32_t *d, *df = nullptr;
  PSC_TRY(ensure_t(g, B_AUX0, g->n + 1, &d));
  if (forest_out) PSC_TRY(ensure_t(g, B_AUX3, 2 * g->n + 2, &df));
  uint64_t nfor = 0;
  PSC_TRY(cc_run(g, beta, d, df, forest_out ? &nfor : nullptr));
  PSC_CUDA(cudaMemcpyAsync(labels_out, d, g->n * 4, cudaMemcpyDeviceToHost, g->stream));
  if (forest_out) {
    *n_forest = nfor;
    if (nfor) PSC_CUDA(cudaMemcpyAsync(forest_out, df, nfor * 8, cudaMemcpyDeviceToHost, g->stream));
  }
  return call_end(g);
}

extern "C" int psc_ldd_rounds(psc_graph_t g, uint32_t* out, uint32_t cap, uint32_t* rounds) {
  if (!g || !rounds || (cap && !out)) return PSC_ERR_INVALID;
  const uint32_t r = (uint32_t)(g->ldd_trace.size() / 3);
  *rounds = r;
  if (r > cap) return PSC_ERR_CAPACITY;
  std::copy(g->ldd_trace.begin(), g->ldd_trace.end(), out);
  return PSC_OK;
}

extern "C" int psc_ldd(psc_graph_t g, double beta, uint32_t* label_out, uint32_t* parent_out) {
  if (!g || !label_out || !(beta > 0)) return PSC_ERR_INVALID;
  PSC_TRY(call_begin(g));
  uint32_t *d, *dp = nullptr;
  PSC_TRY(ensure_t(g, B_AUX0, g->n + 1, &d));
  if (parent_out) PSC_TRY(ensure_t(g, B_TMP32, g->n + 1, &dp));
  PSC_TRY(ldd_run(g, beta, d, dp));
  PSC_CUDA(cudaMemcpyAsync(label_out, d, g->n * 4, cudaMemcpyDeviceToHost, g->stream));
  if (parent_out)
    PSC_CUDA(cudaMemcpyAsync(parent_out, dp, g->n * 4, cudaMemcpyDeviceToHost, g->stream));
  return call_end(g);
}

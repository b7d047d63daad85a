// Single-source reachability on the device (REACH, src/reach.hpp:21-243).
//
// Frontier rounds switch between
//   push: the frontier is a u32 queue; warps expand 32 frontier vertices at a
//         time with the balanced warp expansion, claim targets with an
//         atomicOr on the visited bitmap and append winners with one
//         warp-aggregated atomic (the reference's hashbag insert + pack);
//         vertices above kHeavyDeg out-edges go to a heavy list that the
//         whole grid expands next;
//   pull: the frontier is a bitmap; each warp owns 32 consecutive unvisited
//         vertices and scans their in-edges until a frontier bit is found,
//         then writes the visited / next-frontier words with one store
//         (the reference's dense_update, no atomics needed).
// The switch follows the reference's rule (judge, reach.hpp:86-112): push
// while frontier vertices + their out-edges < m / pull_div (pull_div = 20),
// with exact degree sums gathered by the kernels instead of sampling.
//
// VGC (local search, reach.hpp:114-171) runs each low-degree frontier vertex
// as a warp-local BFS in shared memory that claims up to tau vertices in the
// same round before spilling the rest to the global frontier.
#include <mutex>

#include "common.cuh"
#include "engines.cuh"

namespace psc {

constexpr int kReachBlock = 256;
constexpr int kVgcQueue = 512;  // VGC queue entries per warp (16 KB per block)

__global__ void k_reach_init(uint32_t* vis, uint32_t* q, uint32_t src) {
  vis[src >> 5] = 1u << (src & 31);
  q[0] = src;
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    k_reach_push(const uint64_t* __restrict__ off, const uint32_t* __restrict__ E,
                 const uint32_t* __restrict__ qin, uint64_t nin, uint32_t* vis, uint32_t* qout,
                 uint32_t* heavy, Counters* ctr) {
  __shared__ WarpExpandSmem sm[BLOCK / 32];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  unsigned long long scanned = 0, next_edges = 0;
  for (uint64_t base = gw * 32; base < nin; base += nw * 32) {
    const uint64_t i = base + lane;
    uint64_t beg = 0;
    uint32_t deg = 0;
    if (i < nin) {
      uint32_t u = qin[i];
      beg = off[u];
      uint64_t d = off[u + 1] - beg;
      if (d > kHeavyDeg) {
        heavy[atomicAdd(&ctr->heavy, 1ull)] = u;
        d = 0;
      }
      deg = (uint32_t)d;
    }
    scanned += deg;
    warp_expand(sm[wid], beg, deg, [&](bool act, int, uint64_t e) {
      uint32_t v = 0;
      bool take = false;
      if (act) {
        v = __ldg(&E[e]);
        take = bit_set(vis, v);
      }
      unsigned long long pos = warp_append(&ctr->next, take);
      if (take) {
        qout[pos] = v;
        next_edges += off[v + 1] - off[v];
      }
    });
  }
  scanned = warp_sum(scanned);
  next_edges = warp_sum(next_edges);
  if (lane == 0) {
    if (scanned) atomicAdd(&ctr->edges, scanned);
    if (next_edges) atomicAdd(&ctr->next_edges, next_edges);
  }
}

// VGC push round (reach.hpp:114-171): one frontier vertex per warp.  A vertex
// with 0 < deg < tau starts a local BFS in a shared-memory queue of tq =
// min(tau, QCAP) entries: the warp expands up to 32 queued vertices per wave
// with the balanced expansion, claims neighbours on the visited bitmap, and
// keeps a claimed vertex in the queue while it has room, else spills it to the
// next global frontier.  Queued vertices with more than tq out-edges, and
// whatever is left in the queue when it fills, are spilled as well.  Other
// frontier vertices are expanded directly (heavy ones by the whole grid).
template <int BLOCK, int QCAP>
__global__ void __launch_bounds__(BLOCK)
    k_reach_vgc(const uint64_t* __restrict__ off, const uint32_t* __restrict__ E,
                const uint32_t* __restrict__ qin, uint64_t nin, uint32_t* vis, uint32_t* qout,
                uint32_t* heavy, Counters* ctr, uint32_t tau) {
  __shared__ WarpExpandSmem sm[BLOCK / 32];
  __shared__ uint32_t sq[BLOCK / 32][QCAP];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  const uint32_t tq = tau < (uint32_t)QCAP ? tau : (uint32_t)QCAP;
  uint32_t* Q = sq[wid];
  unsigned long long scanned = 0, next_edges = 0;
  auto emit = [&](bool take, uint32_t v) {
    unsigned long long pos = warp_append(&ctr->next, take);
    if (take) {
      qout[pos] = v;
      next_edges += off[v + 1] - off[v];
    }
  };
  for (uint64_t i = gw; i < nin; i += nw) {
    const uint32_t u = qin[i];
    const uint64_t ub = off[u], ue = off[u + 1];
    const uint64_t du = ue - ub;
    if (!(du > 0 && du < tq)) {
      if (du > kHeavyDeg) {
        if (lane == 0) heavy[atomicAdd(&ctr->heavy, 1ull)] = u;
        continue;
      }
      if (lane == 0) scanned += du;
      for (uint64_t b = ub; b < ue; b += 32) {
        const uint64_t e = b + lane;
        uint32_t v = 0;
        bool take = false;
        if (e < ue) {
          v = __ldg(&E[e]);
          take = bit_set(vis, v);
        }
        emit(take, v);
      }
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
      __syncwarp();
      emit(spill_self, x);
      scanned += deg;
      warp_expand(sm[wid], beg, deg, [&](bool act, int, uint64_t e) {
        uint32_t v = 0;
        bool take = false;
        if (act) {
          v = __ldg(&E[e]);
          take = bit_set(vis, v);
        }
        const unsigned mask = __ballot_sync(kFull, take);
        const uint32_t rank = __popc(mask & ((1u << lane) - 1u));
        const uint32_t room = tq - tail;
        const bool local = take && rank < room;
        if (local) Q[tail + rank] = v;
        const uint32_t nt = __popc(mask);
        tail += nt < room ? nt : room;
        emit(take && !local, v);
      });
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
  next_edges = warp_sum(next_edges);
  if (lane == 0) {
    if (scanned) atomicAdd(&ctr->edges, scanned);
    if (next_edges) atomicAdd(&ctr->next_edges, next_edges);
  }
}

// The whole grid walks the edges of every heavy vertex, 32 edges per warp step.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    k_reach_heavy(const uint64_t* __restrict__ off, const uint32_t* __restrict__ E,
                  const uint32_t* __restrict__ heavy, Counters* ctr, uint32_t* vis, uint32_t* qout) {
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t nh = *(volatile unsigned long long*)&ctr->heavy;
  const uint64_t stride = (uint64_t)gridDim.x * BLOCK;
  unsigned long long scanned = 0, next_edges = 0;
  for (uint64_t h = 0; h < nh; h++) {
    const uint32_t u = heavy[h];
    const uint64_t beg = off[u], end = off[u + 1];
    for (uint64_t b = beg + (uint64_t)blockIdx.x * BLOCK + wid * 32; b < end; b += stride) {
      const uint64_t e = b + lane;
      const bool act = e < end;
      uint32_t v = 0;
      bool take = false;
      if (act) {
        scanned++;
        v = __ldg(&E[e]);
        take = bit_set(vis, v);
      }
      unsigned long long pos = warp_append(&ctr->next, take);
      if (take) {
        qout[pos] = v;
        next_edges += off[v + 1] - off[v];
      }
    }
  }
  scanned = warp_sum(scanned);
  next_edges = warp_sum(next_edges);
  if (lane == 0) {
    if (scanned) atomicAdd(&ctr->edges, scanned);
    if (next_edges) atomicAdd(&ctr->next_edges, next_edges);
  }
}

// Pull round: B_* is the reverse direction of the search, A_off the forward
// offsets (for the next round's edge count).
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    k_reach_pull(const uint64_t* __restrict__ B_off, const uint32_t* __restrict__ B_E,
                 const uint64_t* __restrict__ A_off, const uint32_t* __restrict__ fb_in,
                 uint32_t* vis, uint32_t* fb_out, uint64_t n, Counters* ctr) {
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  const uint64_t nwords = (n + 31) >> 5;
  unsigned long long cnt = 0, scanned = 0, next_edges = 0;
  for (uint64_t w = gw; w < nwords; w += nw) {
    const uint64_t v = w * 32 + lane;
    const uint32_t vw = vis[w];
    bool found = false;
    if (v < n && !((vw >> lane) & 1u)) {
      const uint64_t b = B_off[v], e = B_off[v + 1];
      uint64_t j = b;
      for (; j < e; j++) {
        uint32_t x = __ldg(&B_E[j]);
        if ((__ldg(&fb_in[x >> 5]) >> (x & 31)) & 1u) {
          found = true;
          break;
        }
      }
      scanned += (found ? j + 1 : j) - b;
      if (found) next_edges += A_off[v + 1] - A_off[v];
    }
    const uint32_t mask = __ballot_sync(kFull, found);
    if (lane == 0) {
      fb_out[w] = mask;
      if (mask) vis[w] = vw | mask;
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

int reach_run(psc_graph_s* g, uint32_t src, bool backward, bool local, uint32_t tau,
              uint32_t pull_div, uint32_t* vis, uint32_t* rounds_out) {
  const uint64_t n = g->n, nwords = (n + 31) / 32;
  // VGC rounds while the frontier is below one vertex per resident warp
  const uint64_t vgc_limit = (uint64_t)g->num_sms * 64;
  const uint64_t* A_off = backward ? g->in_off : g->off;
  const uint32_t* A_E = backward ? g->in_E : g->E;
  const uint64_t* B_off = backward ? g->off : g->in_off;
  const uint32_t* B_E = backward ? g->E : g->in_E;
  uint32_t *qa, *qb, *fa, *fb, *heavy;
  PSC_TRY(ensure_t(g, B_QA, n + 1, &qa));
  PSC_TRY(ensure_t(g, B_QB, n + 1, &qb));
  PSC_TRY(ensure_t(g, B_FB_A, nwords + 1, &fa));
  PSC_TRY(ensure_t(g, B_FB_B, nwords + 1, &fb));
  PSC_TRY(ensure_t(g, B_HEAVY, n + 1, &heavy));
  PSC_CUDA(cudaMemsetAsync(vis, 0, nwords * 4, g->stream));
  k_reach_init<<<1, 1, 0, g->stream>>>(vis, qa, src);
  if (pull_div == 0) pull_div = 20;
  const uint64_t threshold = g->m / pull_div;
  uint64_t nf = 1, nf_edges = 0;
  bool pull = false;
  uint32_t rounds = 0;
  while (nf > 0) {
    rounds++;
    if (rounds > n + 2) return PSC_ERR_ITER_LIMIT;
    const bool want_pull = (nf + nf_edges) >= threshold;
    if (want_pull && !pull) {
      ProfScope ps(g, F_REACH_PULL);
      PSC_CUDA(cudaMemsetAsync(fa, 0, nwords * 4, g->stream));
      k_queue_to_bitmap<<<grid_for(g, nf, 256), 256, 0, g->stream>>>(qa, nf, fa);
      pull = true;
    } else if (!want_pull && pull) {
      ProfScope ps(g, F_REACH_PUSH);
      PSC_TRY(zero_counters(g));
      k_bitmap_to_queue<<<grid_for(g, nwords, 256), 256, 0, g->stream>>>(fa, nwords, qa, g->ctr);
      pull = false;
    }
    PSC_TRY(zero_counters(g));
    if (!pull) {
      if (local && nf <= vgc_limit) {
        ProfScope ps(g, F_REACH_VGC);
        k_reach_vgc<kReachBlock, kVgcQueue>
            <<<grid_for(g, nf * 32, kReachBlock), kReachBlock, 0, g->stream>>>(
                A_off, A_E, qa, nf, vis, qb, heavy, g->ctr, tau ? tau : 512);
      } else {
        ProfScope ps(g, F_REACH_PUSH);
        k_reach_push<kReachBlock><<<grid_for(g, nf, kReachBlock), kReachBlock, 0, g->stream>>>(
            A_off, A_E, qa, nf, vis, qb, heavy, g->ctr);
      }
      {
        ProfScope ps(g, F_HEAVY);
        k_reach_heavy<kReachBlock><<<g->num_sms * 4, kReachBlock, 0, g->stream>>>(A_off, A_E, heavy,
                                                                                  g->ctr, vis, qb);
      }
      std::swap(qa, qb);
      swap_bufs(g, B_QA, B_QB);
    } else {
      ProfScope ps(g, F_REACH_PULL);
      k_reach_pull<kReachBlock><<<grid_for(g, nwords * 32, kReachBlock), kReachBlock, 0, g->stream>>>(
          B_off, B_E, A_off, fa, vis, fb, n, g->ctr);
      std::swap(fa, fb);
      swap_bufs(g, B_FB_A, B_FB_B);
    }
    PSC_CUDA(cudaGetLastError());
    PSC_TRY(read_counters(g));
    nf = g->hctr->next;
    nf_edges = g->hctr->next_edges;
  }
  if (rounds_out) *rounds_out = rounds;
  return PSC_OK;
}

__global__ void k_bitmap_to_bytes(const uint32_t* __restrict__ vis, uint64_t n, uint8_t* out) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = (vis[i >> 5] >> (i & 31)) & 1u;
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
constexpr size_t kNaHeavy = kNaQb + kNaQueue;
constexpr size_t kNaCtr = kNaHeavy + kNaQueue;
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
  if (n > kNaMaxN) return PSC_ERR_TOO_LARGE;
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
  uint32_t* heavy = nd.scratch + kNaHeavy;
  Counters* ctr = (Counters*)(nd.scratch + kNaCtr);
  Counters hc;  // host copy of the counters (stack memory)

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
      k_reach_push<kReachBlock><<<na_grid(nd.num_sms, nf, kReachBlock), kReachBlock, 0, s>>>(
          A_off, A_E, qa, nf, vis, qb, heavy, ctr);
      k_reach_heavy<kReachBlock><<<nd.num_sms * 4, kReachBlock, 0, s>>>(A_off, A_E, heavy, ctr,
                                                                       vis, qb);
      std::swap(qa, qb);
    } else {
      k_reach_pull<kReachBlock><<<na_grid(nd.num_sms, nwords * 32, kReachBlock), kReachBlock, 0, s>>>(
          B_off, B_E, A_off, fa, vis, fb, n, ctr);
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

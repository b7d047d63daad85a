// Device transpose (make_directed, src/graph.hpp:222-245): in-degree count,
// exclusive scan into in_off, then a scatter of every edge u -> v to
// in_E[in_off[v] + k] through per-target atomic cursors, then a per-list sort
// so in-lists come out ordered by source as the reference's sort-based
// transpose leaves them.
#include "common.cuh"
#include "engines.cuh"
#include "scan.cuh"

namespace psc {

__global__ void k_indeg(const uint32_t* __restrict__ E, uint64_t m, uint32_t* cnt) {
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m;
       j += (uint64_t)gridDim.x * blockDim.x)
    atomicAdd(&cnt[E[j]], 1u);
}

struct CntValue {
  const uint32_t* cnt;
  __device__ uint32_t operator()(uint64_t i) const { return cnt[i]; }
};

struct OffEmit {
  uint64_t* in_off;
  uint32_t* cursor_reset;
  __device__ void operator()(uint64_t i, uint64_t excl, uint32_t) const {
    in_off[i] = excl;
    cursor_reset[i] = 0;
  }
};

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    k_scatter(const uint64_t* __restrict__ off, const uint32_t* __restrict__ E, uint64_t n,
              const uint64_t* __restrict__ in_off, uint32_t* cursor, uint32_t* in_E) {
  __shared__ WarpExpandSmem sm[BLOCK / 32];
  __shared__ uint32_t s_u[BLOCK];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * (BLOCK / 32) + wid;
  const uint64_t nw = (uint64_t)gridDim.x * (BLOCK / 32);
  for (uint64_t base = gw * 32; base < n; base += nw * 32) {
    const uint64_t u = base + lane;
    uint64_t beg = 0;
    uint64_t deg = 0;
    if (u < n) {
      beg = off[u];
      deg = off[u + 1] - beg;
    }
    s_u[wid * 32 + lane] = (uint32_t)u;
    __syncwarp();
    // lists in pieces of at most 2^26 edges keep the 32-lane degree sum of
    // the warp expansion below 2^31
    while (__any_sync(kFull, deg > 0)) {
      uint32_t piece = (uint32_t)(deg > (1ull << 26) ? (1ull << 26) : deg);
      warp_expand(sm[wid], beg, piece, [&](bool act, int s, uint64_t e) {
        if (act) {
          const uint32_t v = E[e];
          const uint32_t k = atomicAdd(&cursor[v], 1u);
          in_E[in_off[v] + k] = s_u[wid * 32 + s];
        }
      });
      beg += piece;
      deg -= piece;
    }
    __syncwarp();
  }
}

// Sorts each in-list.  Lists up to kSmemSort entries: one block, bitonic
// network in shared memory.  Longer lists: the block runs the same network
// over global memory.
constexpr int kSortBlock = 512;
constexpr int kSmemSort = 4096;

__device__ void bitonic_sort_span(uint32_t* a, uint32_t len, uint32_t pad) {
  // a has room for `pad` (power of two >= len) entries; the tail is filled
  // with 0xFFFFFFFF so it sorts last.
  for (uint32_t i = len + threadIdx.x; i < pad; i += blockDim.x) a[i] = 0xFFFFFFFFu;
  __syncthreads();
  for (uint32_t k = 2; k <= pad; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < pad; i += blockDim.x) {
        uint32_t p = i ^ j;
        if (p > i) {
          uint32_t x = a[i], y = a[p];
          bool up = (i & k) == 0;
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

__global__ void __launch_bounds__(kSortBlock)
    k_sort_lists(const uint64_t* __restrict__ in_off, uint64_t n, uint32_t* in_E, uint32_t* gscratch,
                 uint64_t scratch_len) {
  __shared__ uint32_t buf[kSmemSort];
  for (uint64_t v = blockIdx.x; v < n; v += gridDim.x) {
    const uint64_t b = in_off[v], e = in_off[v + 1];
    const uint64_t len = e - b;
    if (len < 2) continue;
    if (len <= 32) {
      // one warp: odd-even transposition sort, one element per lane
      if (threadIdx.x < 32) {
        const int t = (int)threadIdx.x;
        uint32_t x = t < (int)len ? in_E[b + t] : 0xFFFFFFFFu;
        for (int r = 0; r < 32; r++) {
          int partner = ((t & 1) == (r & 1)) ? t + 1 : t - 1;
          uint32_t y = __shfl_sync(kFull, x, partner & 31);
          if (partner >= 0 && partner < 32) {
            bool low = t < partner;
            x = low ? min(x, y) : max(x, y);
          }
        }
        if (t < (int)len) in_E[b + t] = x;
      }
      __syncthreads();
      continue;
    }
    uint32_t pad = 64;
    while (pad < len) pad <<= 1;
    if (pad <= kSmemSort) {
      for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) buf[i] = in_E[b + i];
      bitonic_sort_span(buf, (uint32_t)len, pad);
      for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) in_E[b + i] = buf[i];
      __syncthreads();
    } else if (pad <= scratch_len) {
      uint32_t* a = gscratch + (uint64_t)blockIdx.x * scratch_len;
      for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) a[i] = in_E[b + i];
      __syncthreads();
      bitonic_sort_span(a, (uint32_t)len, pad);
      for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) in_E[b + i] = a[i];
      __syncthreads();
    }
  }
}

__global__ void k_max_len(const uint64_t* __restrict__ in_off, uint64_t n, unsigned long long* out) {
  unsigned long long mx = 0;
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (uint64_t)gridDim.x * blockDim.x) {
    unsigned long long l = in_off[v + 1] - in_off[v];
    mx = l > mx ? l : mx;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long t = __shfl_xor_sync(kFull, mx, o);
    mx = t > mx ? t : mx;
  }
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(out, mx);
}

int build_transpose(psc_graph_s* g, bool sorted) {
  const uint64_t n = g->n, m = g->m;
  uint32_t* cnt;
  PSC_TRY(ensure_t(g, B_TMP32, n + 1, &cnt));
  PSC_CUDA(cudaMemsetAsync(cnt, 0, (n + 1) * 4, g->stream));
  {
    ProfScope ps(g, F_TRANSPOSE);
    ps.bytes = 8.0 * m;
    k_indeg<<<grid_for(g, m, 256), 256, 0, g->stream>>>(g->E, m, cnt);
  }
  // in_off[i] = prefix of counts; the count array doubles as the cursor
  // (reset to zero by the emit step after it is read).
  uint64_t total = 0;
  PSC_TRY(scan_emit(g, n, CntValue{cnt}, OffEmit{g->in_off, cnt}, &total, F_TRANSPOSE));
  PSC_CUDA(cudaMemcpyAsync(g->in_off + n, &g->m, 8, cudaMemcpyHostToDevice, g->stream));
  {
    ProfScope ps(g, F_TRANSPOSE);
    ps.bytes = 16.0 * n + 16.0 * m;
    k_scatter<256><<<grid_for(g, n, 256), 256, 0, g->stream>>>(g->off, g->E, n, g->in_off, cnt,
                                                               g->in_E);
  }
  if (!sorted) return PSC_OK;
  // longest in-list decides the global scratch of the sort
  PSC_TRY(zero_counters(g));
  k_max_len<<<grid_for(g, n, 256), 256, 0, g->stream>>>(g->in_off, n, &g->ctr->aux0);
  PSC_TRY(read_counters(g));
  const uint64_t maxlen = g->hctr->aux0;
  uint64_t pad = 64;
  while (pad < maxlen) pad <<= 1;
  const unsigned sort_grid = (unsigned)std::min<uint64_t>(n, (uint64_t)g->num_sms * 4);
  uint32_t* scratch = nullptr;
  uint64_t scratch_len = 0;
  if (pad > (uint64_t)kSmemSort) {
    scratch_len = pad;
    PSC_TRY(ensure_t(g, B_AUX3, scratch_len * sort_grid, &scratch));
  }
  {
    ProfScope ps(g, F_TRANSPOSE);
    ps.bytes = 8.0 * m;
    k_sort_lists<<<sort_grid, kSortBlock, 0, g->stream>>>(g->in_off, n, g->in_E, scratch, scratch_len);
  }
  PSC_CUDA(cudaGetLastError());
  (void)total;
  return PSC_OK;
}

}  // namespace psc

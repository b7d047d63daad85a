// Device-wide exclusive scan and order-preserving compaction.
//
// scan_emit(g, n, value, emit): computes value(i) (u32) for i < n, and calls
// emit(i, excl, value(i)) for every i, where excl (u64) is the exclusive
// prefix sum of value over [0, i).  Returns the total through *total (host).
// Three launches: per-tile sums, a single-block scan of the tile sums, then a
// per-tile block scan that emits.  Tiles are 256 threads x 8 striped passes.
#pragma once
#include "common.cuh"

namespace psc {

constexpr int kScanBlock = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanBlock * kScanItems;

template <int BLOCK>
__device__ __forceinline__ uint64_t block_excl_scan(uint64_t v, uint64_t* sm, uint64_t* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr int NW = BLOCK / 32;
  uint64_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint64_t t = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) sm[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    uint64_t x = lane < NW ? sm[lane] : 0;
    uint64_t xi = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint64_t t = __shfl_up_sync(kFull, xi, o);
      if (lane >= o) xi += t;
    }
    if (lane < NW) sm[lane] = xi - x;
    if (lane == NW - 1) sm[32] = xi;
  }
  __syncthreads();
  uint64_t r = sm[wid] + incl - v;
  *total = sm[32];
  __syncthreads();
  return r;
}

template <class Value>
__global__ void __launch_bounds__(kScanBlock) k_tile_sum(Value value, uint64_t n, uint64_t* tile_sums) {
  __shared__ uint64_t sm[33];
  uint64_t base = (uint64_t)blockIdx.x * kScanTile;
  uint64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    uint64_t i = base + (uint64_t)k * kScanBlock + threadIdx.x;
    if (i < n) s += value(i);
  }
  uint64_t tot;
  block_excl_scan<kScanBlock>(s, sm, &tot);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

// Single block, exclusive scan in place; total written to tile_sums[ntiles].
__global__ void __launch_bounds__(1024) k_scan_tile_sums(uint64_t* tile_sums, uint64_t ntiles);

template <class Value, class Emit>
__global__ void __launch_bounds__(kScanBlock) k_tile_emit(Value value, Emit emit, uint64_t n,
                                                          const uint64_t* tile_off) {
  __shared__ uint64_t sm[33];
  uint64_t base = (uint64_t)blockIdx.x * kScanTile;
  uint64_t carry = tile_off[blockIdx.x];
#pragma unroll 1
  for (int k = 0; k < kScanItems; k++) {
    uint64_t i = base + (uint64_t)k * kScanBlock + threadIdx.x;
    uint32_t v = i < n ? value(i) : 0;
    uint64_t tot;
    uint64_t ex = block_excl_scan<kScanBlock>(v, sm, &tot);
    if (i < n) emit(i, carry + ex, v);
    carry += tot;
  }
}

// Host driver.  total may be null.  item_bytes / sel_bytes: algorithmic
// bytes per input item and per selected item, for the profiling counters.
template <class Value, class Emit>
int scan_emit(psc_graph_s* g, uint64_t n, Value value, Emit emit, uint64_t* total, int fam = F_COMPACT,
              double item_bytes = 0, double sel_bytes = 0) {
  if (n == 0) {
    if (total) *total = 0;
    return PSC_OK;
  }
  uint64_t ntiles = (n + kScanTile - 1) / kScanTile;
  uint64_t* ts = nullptr;
  PSC_TRY(ensure_t(g, B_SCAN, ntiles + 2, &ts));
  {
    ProfScope ps(g, fam);
    k_tile_sum<<<(unsigned)ntiles, kScanBlock, 0, g->stream>>>(value, n, ts);
  }
  {
    ProfScope ps(g, fam);
    k_scan_tile_sums<<<1, 1024, 0, g->stream>>>(ts, ntiles);
  }
  {
    ProfScope ps(g, fam);
    k_tile_emit<<<(unsigned)ntiles, kScanBlock, 0, g->stream>>>(value, emit, n, ts);
  }
  PSC_CUDA(cudaGetLastError());
  if (total) {
    PSC_CUDA(cudaMemcpyAsync(&g->hctr->aux0, ts + ntiles, sizeof(uint64_t), cudaMemcpyDeviceToHost,
                             g->stream));
    PSC_CUDA(cudaStreamSynchronize(g->stream));
    *total = g->hctr->aux0;
  }
  if (g->profiling) g->prof[fam].bytes += item_bytes * n + sel_bytes * (total ? *total : 0);
  return PSC_OK;
}

// Selections shared by the SCC drivers: in/out-degree-zero vertices
// (src/scc.hpp:288-301), and live (not done) entries of a vertex list.
struct ZeroFlag {
  const uint64_t* off;
  const uint64_t* in_off;
  __device__ uint32_t operator()(uint64_t i) const {
    return (off[i + 1] == off[i] || in_off[i + 1] == in_off[i]) ? 1u : 0u;
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

// Not done according to a bitmap of finished vertices (see k_label_first).
struct NotDoneBitAt {
  const uint32_t* src;
  const uint32_t* done;
  __device__ uint32_t operator()(uint64_t i) const {
    const uint32_t v = src[i];
    return ((__ldg(&done[v >> 5]) >> (v & 31)) & 1u) ^ 1u;
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

}  // namespace psc

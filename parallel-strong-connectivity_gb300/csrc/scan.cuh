// Device-wide exclusive scan and order-preserving compaction.
//
// scan_emit(g, n, value, emit): computes value(i) (u32) for i < n, and calls
// emit(i, excl, value(i)) for every i, where excl (u64) is the exclusive
// prefix sum of value over [0, i).  Returns the total through *total (host).
// Three launches: per-tile sums, a single-block scan of the tile sums, then a
// per-tile block scan that emits.  Tiles are 256 threads x 8 striped passes
// (item k * 256 + t of a tile belongs to thread t); a tile's 8 values are
// loaded together and scanned with one block pass.  scan_emit_flags is the
// same for 0/1 values: the first pass also stores them as a bitmap, which the
// emit pass reads instead of evaluating the value again.
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

// Exclusive scan of a tile in striped order: ex[k] = sum of all items before
// item (k, thread); *total = the tile's sum.  sm: K * BLOCK / 32 + 1 words.
template <int BLOCK, int K>
__device__ __forceinline__ void block_scan_striped(const uint32_t (&v)[K], uint64_t (&ex)[K],
                                                   uint64_t* sm, uint64_t* total) {
  constexpr int NW = BLOCK / 32;
  constexpr int NE = K * NW;             // warp totals, k-major
  constexpr int PER = (NE + 31) / 32;    // per lane of warp 0
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint64_t incl[K];
#pragma unroll
  for (int k = 0; k < K; k++) {
    incl[k] = v[k];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t t = __shfl_up_sync(kFull, incl[k], o);
      if (lane >= o) incl[k] += t;
    }
  }
  if (lane == 31)
#pragma unroll
    for (int k = 0; k < K; k++) sm[k * NW + wid] = incl[k];
  __syncthreads();
  if (wid == 0) {
    uint64_t x[PER], run = 0;
#pragma unroll
    for (int e = 0; e < PER; e++) {
      const int p = lane * PER + e;
      x[e] = p < NE ? sm[p] : 0;
      run += x[e];
    }
    uint64_t inc = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t t = __shfl_up_sync(kFull, inc, o);
      if (lane >= o) inc += t;
    }
    uint64_t pre = inc - run;
#pragma unroll
    for (int e = 0; e < PER; e++) {
      const int p = lane * PER + e;
      if (p < NE) sm[p] = pre;
      pre += x[e];
    }
    if (lane == 31) sm[NE] = inc;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; k++) ex[k] = sm[k * NW + wid] + incl[k] - v[k];
  *total = sm[NE];
  __syncthreads();
}

template <class Value, class Emit>
__global__ void __launch_bounds__(kScanBlock) k_tile_emit(Value value, Emit emit, uint64_t n,
                                                          const uint64_t* tile_off) {
  __shared__ uint64_t sm[kScanItems * kScanBlock / 32 + 1];
  const uint64_t base = (uint64_t)blockIdx.x * kScanTile;
  uint32_t v[kScanItems];
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    const uint64_t i = base + (uint64_t)k * kScanBlock + threadIdx.x;
    v[k] = i < n ? value(i) : 0;
  }
  uint64_t ex[kScanItems], tot;
  block_scan_striped<kScanBlock, kScanItems>(v, ex, sm, &tot);
  const uint64_t carry = tile_off[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    const uint64_t i = base + (uint64_t)k * kScanBlock + threadIdx.x;
    if (i < n) emit(i, carry + ex[k], v[k]);
  }
}

// First pass of scan_emit_flags: tile sums of 0/1 values, which are also
// stored as bits[i / 32] (one ballot per 32 items).
template <class Value>
__global__ void __launch_bounds__(kScanBlock) k_flag_tile_sum(Value value, uint64_t n,
                                                              uint64_t* tile_sums, uint32_t* bits) {
  __shared__ uint64_t sm[33];
  const uint64_t base = (uint64_t)blockIdx.x * kScanTile;
  uint32_t f[kScanItems];
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    const uint64_t i = base + (uint64_t)k * kScanBlock + threadIdx.x;
    f[k] = i < n ? value(i) : 0u;
  }
  uint64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    const uint64_t i = base + (uint64_t)k * kScanBlock + threadIdx.x;
    const uint32_t word = __ballot_sync(kFull, f[k] != 0);
    if ((threadIdx.x & 31) == 0 && i < n) bits[i >> 5] = word;
    s += f[k];
  }
  uint64_t tot;
  block_excl_scan<kScanBlock>(s, sm, &tot);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

// scan_emit_flags of at most one tile in one launch: flags, scan, emits and
// the total (written to *total).
template <class Value, class Emit>
__global__ void __launch_bounds__(kScanBlock) k_flag_emit_tile(Value value, Emit emit, uint64_t n,
                                                               uint64_t* total) {
  __shared__ uint64_t sm[kScanItems * kScanBlock / 32 + 1];
  uint32_t v[kScanItems];
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    const uint64_t i = (uint64_t)k * kScanBlock + threadIdx.x;
    v[k] = i < n ? value(i) : 0u;
  }
  uint64_t ex[kScanItems], tot;
  block_scan_striped<kScanBlock, kScanItems>(v, ex, sm, &tot);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    const uint64_t i = (uint64_t)k * kScanBlock + threadIdx.x;
    if (i < n) emit(i, ex[k], v[k]);
  }
  if (threadIdx.x == 0) *total = tot;
}

struct BitValue {
  const uint32_t* bits;
  __device__ uint32_t operator()(uint64_t i) const { return (bits[i >> 5] >> (i & 31)) & 1u; }
};

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

// scan_emit for a value that is 0 or 1 (a selection); see the file comment.
// total_dev (optional): receives the device address of the total (valid
// until the next scan on this handle), for kernels that read the count
// without a wait on the host.
template <class Value, class Emit>
int scan_emit_flags(psc_graph_s* g, uint64_t n, Value value, Emit emit, uint64_t* total,
                    int fam = F_COMPACT, double item_bytes = 0, double sel_bytes = 0,
                    const unsigned long long** total_dev = nullptr) {
  if (n == 0) {
    if (total) *total = 0;
    return PSC_OK;
  }
  const uint64_t ntiles = (n + kScanTile - 1) / kScanTile;
  uint64_t* ts = nullptr;
  PSC_TRY(ensure_t(g, B_SCAN, ntiles + 2, &ts));
  if (ntiles == 1) {
    ProfScope ps(g, fam);
    k_flag_emit_tile<<<1, kScanBlock, 0, g->stream>>>(value, emit, n, ts + 1);
  } else {
    uint32_t* bits = nullptr;
    PSC_TRY(ensure_t(g, B_SCANBITS, (n + 31) / 32 + 1, &bits));
    {
      ProfScope ps(g, fam);
      k_flag_tile_sum<<<(unsigned)ntiles, kScanBlock, 0, g->stream>>>(value, n, ts, bits);
    }
    {
      ProfScope ps(g, fam);
      k_scan_tile_sums<<<1, 1024, 0, g->stream>>>(ts, ntiles);
    }
    {
      ProfScope ps(g, fam);
      k_tile_emit<<<(unsigned)ntiles, kScanBlock, 0, g->stream>>>(BitValue{bits}, emit, n, ts);
    }
  }
  PSC_CUDA(cudaGetLastError());
  if (total_dev) *total_dev = (const unsigned long long*)(ts + ntiles);
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

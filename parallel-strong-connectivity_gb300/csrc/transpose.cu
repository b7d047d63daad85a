// Device transpose (make_directed, src/graph.hpp:222-245): the in-lists,
// sorted by source as the reference's sort-based transpose leaves them, from
// a stable radix sort of the (target, source) pairs by target.
#include "common.cuh"
#include "engines.cuh"
#include "scan.cuh"

namespace psc {

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

// ---------------------------------------------------------------------------
// Radix transpose: the (target, source) pairs of all edges, generated in CSR
// order (sorted by source), sorted by target with a stable LSD radix sort of
// kRsBits-bit digits.  Stability keeps every in-list ordered by source, as
// the reference's sort-based transpose leaves it.  Each pass: a per-tile
// digit histogram in shared memory, one scan over (digit, tile), and a stable
// scatter in which every warp ranks its sub-tile with __match_any_sync.  No
// global atomics, so hub targets cost nothing extra.
// ---------------------------------------------------------------------------
constexpr int kRsBits = 8;
constexpr int kRsBins = 1 << kRsBits;
constexpr int kRsBlock = 256;
constexpr int kRsTile = 4096;  // pairs per block and pass (16 per thread)

// src[e] = the vertex whose adjacency holds edge e.  A warp takes 32 * 32
// consecutive edges; the sources of its first and last edge bound a small
// vertex range (one vertex for a hub), which every lane's binary search then
// covers; stores are coalesced.
constexpr int kSrcRun = 32 * 32;

__device__ __forceinline__ uint64_t edge_owner(const uint64_t* __restrict__ off, uint64_t lo,
                                               uint64_t hi, uint64_t e) {
  while (lo < hi) {  // largest u in [lo, hi] with off[u] <= e
    const uint64_t mid = (lo + hi + 1) >> 1;
    if (__ldg(&off[mid]) <= e)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__global__ void k_edge_sources(const uint64_t* __restrict__ off, uint64_t n, uint64_t m,
                               uint32_t* src) {
  const unsigned lane = lane_id();
  const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t runs = (m + kSrcRun - 1) / kSrcRun;
  for (uint64_t r = gw; r < runs; r += nw) {
    const uint64_t e0 = r * kSrcRun;
    const uint64_t e1 = e0 + kSrcRun < m ? e0 + kSrcRun : m;
    uint64_t b = 0;
    if (lane == 0) b = edge_owner(off, 0, n - 1, e0);
    if (lane == 1) b = edge_owner(off, 0, n - 1, e1 - 1);
    const uint64_t lo = __shfl_sync(kFull, b, 0), hi = __shfl_sync(kFull, b, 1);
    for (uint64_t e = e0 + lane; e < e1; e += 32) src[e] = (uint32_t)edge_owner(off, lo, hi, e);
  }
}

// Per-tile digit histograms.  Every thread holds kRsPer keys of its warp's
// sub-tile in registers (loaded first, so their latencies overlap); equal
// digits of a warp add to the shared histogram once.
constexpr int kRsPer = kRsTile / kRsBlock;  // 16 keys per thread

__global__ void __launch_bounds__(kRsBlock)
    k_rs_hist(const uint32_t* __restrict__ keys, uint64_t m, int shift, uint64_t ntiles,
              uint32_t* hist) {
  __shared__ uint32_t cnt[kRsBins];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1;
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    for (int b = threadIdx.x; b < kRsBins; b += kRsBlock) cnt[b] = 0;
    __syncthreads();
    const uint64_t base = tile * kRsTile + (uint64_t)wid * (kRsTile / (kRsBlock / 32));
    uint32_t d[kRsPer];
#pragma unroll
    for (int c = 0; c < kRsPer; c++) {
      const uint64_t i = base + c * 32 + lane;
      d[c] = i < m ? (__ldg(&keys[i]) >> shift) & (kRsBins - 1) : kRsBins;
    }
#pragma unroll
    for (int c = 0; c < kRsPer; c++) {
      const unsigned peers = __match_any_sync(kFull, d[c]);
      if (d[c] < (uint32_t)kRsBins && (peers & lt) == 0) atomicAdd(&cnt[d[c]], (uint32_t)__popc(peers));
    }
    __syncthreads();
    for (int b = threadIdx.x; b < kRsBins; b += kRsBlock) hist[(uint64_t)b * ntiles + tile] = cnt[b];
    __syncthreads();
  }
}

// Stable scatter of one pass.  Each warp owns kRsTile / 8 consecutive pairs
// of the tile (chunks of 32 in order, lanes in order), held in registers.
// The tile is first sorted by digit in shared memory (warp counts, a block
// scan over digits, ranked placement), then written out so that consecutive
// threads write consecutive positions of one digit's run: coalesced stores
// instead of one sector per pair.
__global__ void __launch_bounds__(kRsBlock)
    k_rs_scatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint64_t m,
                 int shift, uint64_t ntiles, const uint64_t* __restrict__ offs, uint32_t* kout,
                 uint32_t* vout) {
  constexpr int NW = kRsBlock / 32;
  constexpr int PER_WARP = kRsTile / NW;
  static_assert(kRsBins == kRsBlock, "one digit per thread in the digit scan");
  __shared__ uint32_t skey[kRsTile];
  __shared__ uint32_t sval[kRsTile];
  __shared__ uint32_t wcnt[NW][kRsBins];
  __shared__ uint32_t lstart[kRsBins];
  __shared__ uint64_t gbase[kRsBins];
  __shared__ uint64_t scan_sm[33];
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5, tid = threadIdx.x;
  const unsigned lt = (1u << lane) - 1;
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t tbase = tile * kRsTile;
    const uint64_t base = tbase + (uint64_t)wid * PER_WARP;
    const uint32_t tcount = (uint32_t)(m - tbase < (uint64_t)kRsTile ? m - tbase : kRsTile);
    uint32_t key[kRsPer], val[kRsPer], d[kRsPer];
#pragma unroll
    for (int c = 0; c < kRsPer; c++) {
      const uint64_t i = base + c * 32 + lane;
      key[c] = 0;
      val[c] = 0;
      d[c] = kRsBins;
      if (i < m) {
        key[c] = __ldg(&kin[i]);
        val[c] = __ldg(&vin[i]);
        d[c] = (key[c] >> shift) & (kRsBins - 1);
      }
    }
    for (int b = lane; b < kRsBins; b += 32) wcnt[wid][b] = 0;
    __syncwarp();
    unsigned peers[kRsPer];
#pragma unroll
    for (int c = 0; c < kRsPer; c++) {
      peers[c] = __match_any_sync(kFull, d[c]);
      if (d[c] < (uint32_t)kRsBins && (peers[c] & lt) == 0) wcnt[wid][d[c]] += __popc(peers[c]);
      __syncwarp();
    }
    __syncthreads();
    // digit tid: its start in the sorted tile, each warp's base inside it, and
    // the global start of its run for this tile
    {
      uint32_t total = 0;
#pragma unroll
      for (int w = 0; w < NW; w++) total += wcnt[w][tid];
      uint64_t all = 0;
      const uint32_t start = (uint32_t)block_excl_scan<kRsBlock>(total, scan_sm, &all);
      lstart[tid] = start;
      gbase[tid] = offs[(uint64_t)tid * ntiles + tile];
      uint32_t run = start;
#pragma unroll
      for (int w = 0; w < NW; w++) {
        const uint32_t c = wcnt[w][tid];
        wcnt[w][tid] = run;
        run += c;
      }
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < kRsPer; c++) {
      uint32_t lp = 0;
      if (d[c] < (uint32_t)kRsBins) lp = wcnt[wid][d[c]] + __popc(peers[c] & lt);
      __syncwarp();
      if (d[c] < (uint32_t)kRsBins) {
        skey[lp] = key[c];
        sval[lp] = val[c];
        if ((peers[c] & lt) == 0) wcnt[wid][d[c]] += __popc(peers[c]);
      }
      __syncwarp();
    }
    __syncthreads();
    for (uint32_t j = tid; j < tcount; j += kRsBlock) {
      const uint32_t k = skey[j];
      const uint32_t dj = (k >> shift) & (kRsBins - 1);
      const uint64_t pos = gbase[dj] + (j - lstart[dj]);
      kout[pos] = k;
      vout[pos] = sval[j];
    }
    __syncthreads();
  }
}

struct HistValue {
  const uint32_t* hist;
  __device__ uint32_t operator()(uint64_t i) const { return hist[i]; }
};

struct HistEmit {
  uint64_t* offs;
  __device__ void operator()(uint64_t i, uint64_t excl, uint32_t) const { offs[i] = excl; }
};

// In-degrees from the sorted targets: run starts record their position,
// run ends turn it into the run length.
__global__ void k_run_starts(const uint32_t* __restrict__ t, uint64_t m, uint64_t* rs) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x)
    if (i == 0 || t[i - 1] != t[i]) rs[t[i]] = i;
}

__global__ void k_run_lengths(const uint32_t* __restrict__ t, uint64_t m,
                              const uint64_t* __restrict__ rs, uint32_t* cnt) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x)
    if (i == m - 1 || t[i + 1] != t[i]) cnt[t[i]] = (uint32_t)(i + 1 - rs[t[i]]);
}

int build_transpose(psc_graph_s* g) {
  const uint64_t n = g->n, m = g->m;
  uint32_t* cnt;
  PSC_TRY(ensure_t(g, B_TMP32, n + 1, &cnt));
  PSC_CUDA(cudaMemsetAsync(cnt, 0, (n + 1) * 4, g->stream));
  if (m > 0) {
    int bits = 1;
    while (bits < 32 && ((uint64_t)1 << bits) < n) bits++;
    const int passes = (bits + kRsBits - 1) / kRsBits;
    const uint64_t ntiles = (m + kRsTile - 1) / kRsTile;
    uint32_t *x, *ka, *kb, *hist;
    uint64_t* offs;
    PSC_TRY(ensure_t(g, B_AUX0, m, &x));
    PSC_TRY(ensure_t(g, B_AUX1, m, &ka));
    PSC_TRY(ensure_t(g, B_AUX2, m, &kb));
    PSC_TRY(ensure_t(g, B_AUX3, (uint64_t)kRsBins * ntiles, &hist));
    PSC_TRY(ensure_t(g, B_SCAN2, (uint64_t)kRsBins * ntiles + 1, &offs));
    // value buffers alternate so that the last pass writes in_E
    uint32_t* vb[2] = {passes % 2 ? x : g->in_E, passes % 2 ? g->in_E : x};
    uint32_t* kbuf[2] = {ka, kb};
    {
      ProfScope ps(g, F_TRANSPOSE);
      ps.bytes = 16.0 * n + 4.0 * m;
      k_edge_sources<<<grid_for(g, (m + kSrcRun - 1) / kSrcRun * 32, 256), 256, 0, g->stream>>>(
          g->off, n, m, vb[0]);
    }
    const uint32_t* kin = g->E;
    const unsigned grid = (unsigned)std::min<uint64_t>(ntiles, (uint64_t)g->num_sms * 8);
    for (int p = 0; p < passes; p++) {
      const int shift = p * kRsBits;
      {
        ProfScope ps(g, F_TRANSPOSE);
        ps.bytes = 4.0 * m;
        k_rs_hist<<<grid, kRsBlock, 0, g->stream>>>(kin, m, shift, ntiles, hist);
      }
      PSC_TRY(scan_emit(g, (uint64_t)kRsBins * ntiles, HistValue{hist}, HistEmit{offs}, nullptr,
                        F_TRANSPOSE));
      {
        ProfScope ps(g, F_TRANSPOSE);
        ps.bytes = 16.0 * m;
        k_rs_scatter<<<grid, kRsBlock, 0, g->stream>>>(kin, vb[p & 1], m, shift, ntiles, offs,
                                                       kbuf[p & 1], vb[(p + 1) & 1]);
      }
      kin = kbuf[p & 1];
    }
    uint64_t* rs;
    PSC_TRY(ensure_t(g, B_SCAN3, n + 1, &rs));
    {
      ProfScope ps(g, F_TRANSPOSE);
      ps.bytes = 8.0 * m;
      k_run_starts<<<grid_for(g, m, 256), 256, 0, g->stream>>>(kin, m, rs);
      k_run_lengths<<<grid_for(g, m, 256), 256, 0, g->stream>>>(kin, m, rs, cnt);
    }
  }
  uint64_t total = 0;
  PSC_TRY(scan_emit(g, n, CntValue{cnt}, OffEmit{g->in_off, cnt}, &total, F_TRANSPOSE));
  PSC_CUDA(cudaMemcpyAsync(g->in_off + n, &g->m, 8, cudaMemcpyHostToDevice, g->stream));
  PSC_CUDA(cudaGetLastError());
  return PSC_OK;
}


// ---------------------------------------------------------------------------
// Device symmetrisation (make_symmetric, src/graph.hpp:187-220): every edge in
// both directions, each adjacency list sorted, duplicates and self-loops
// dropped.  The 2m pairs (a, b) -- a's list holds b -- are sorted by b and
// then stably by a with the radix passes above (an LSD sort of the key
// (a, b)); one compaction keeps the first pair of every run of equal pairs
// when a != b, writing the targets; out-degrees come from the run lengths of
// the kept sources.
// ---------------------------------------------------------------------------
__global__ void k_sym_pairs(const uint32_t* __restrict__ E, const uint32_t* __restrict__ src,
                            uint64_t m, uint32_t* key, uint32_t* val) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t a = src[i], b = E[i];
    key[i] = b;  // first pass set: sort by the target
    val[i] = a;
    key[m + i] = a;  // the reverse edge b -> a
    val[m + i] = b;
  }
}

struct SymKeep {  // first of a run of equal (a, b) pairs, a != b
  const uint32_t* A;
  const uint32_t* B;
  __device__ uint32_t operator()(uint64_t i) const {
    const uint32_t a = A[i], b = B[i];
    if (a == b) return 0u;
    return (i == 0 || A[i - 1] != a || B[i - 1] != b) ? 1u : 0u;
  }
};

struct SymEmit {
  const uint32_t* A;
  const uint32_t* B;
  uint32_t* a_out;
  uint32_t* b_out;
  __device__ void operator()(uint64_t i, uint64_t excl, uint32_t v) const {
    if (v) {
      a_out[excl] = A[i];
      b_out[excl] = B[i];
    }
  }
};

// Stable LSD radix sort of cnt (key, val) pairs by the low `bits` bits of
// key, from (k[0], v[0]) through (k[1], v[1]) and back; *at receives the
// index of the pair of buffers holding the result.
static int radix_pairs(psc_graph_s* g, uint64_t cnt, int bits, uint32_t* k[2], uint32_t* v[2],
                       uint32_t* hist, uint64_t* offs, int* at) {
  const int passes = (bits + kRsBits - 1) / kRsBits;
  const uint64_t ntiles = (cnt + kRsTile - 1) / kRsTile;
  const unsigned grid = (unsigned)std::min<uint64_t>(ntiles, (uint64_t)g->num_sms * 8);
  int cur = 0;
  for (int p = 0; p < passes; p++) {
    const int shift = p * kRsBits;
    {
      ProfScope ps(g, F_TRANSPOSE);
      ps.bytes = 4.0 * cnt;
      k_rs_hist<<<grid, kRsBlock, 0, g->stream>>>(k[cur], cnt, shift, ntiles, hist);
    }
    PSC_TRY(scan_emit(g, (uint64_t)kRsBins * ntiles, HistValue{hist}, HistEmit{offs}, nullptr,
                      F_TRANSPOSE));
    {
      ProfScope ps(g, F_TRANSPOSE);
      ps.bytes = 16.0 * cnt;
      k_rs_scatter<<<grid, kRsBlock, 0, g->stream>>>(k[cur], v[cur], cnt, shift, ntiles, offs,
                                                     k[cur ^ 1], v[cur ^ 1]);
    }
    cur ^= 1;
  }
  *at = cur;
  return PSC_OK;
}

static void release(psc_graph_s* g, int b) {
  DevBuf& d = g->bufs[b];
  if (d.p) cudaFreeAsync(d.p, g->stream);
  d.p = nullptr;
  d.bytes = 0;
}

int build_symmetric(psc_graph_s* g) {
  const uint64_t n = g->n, m = g->m;
  uint64_t* off_s = nullptr;
  uint32_t* E_s = nullptr;
  uint64_t ms = 0;
  uint32_t* cnt;
  PSC_TRY(ensure_t(g, B_TMP32, n + 1, &cnt));
  PSC_CUDA(cudaMemsetAsync(cnt, 0, (n + 1) * 4, g->stream));
  if (m > 0) {
    const uint64_t c = 2 * m;
    int bits = 1;
    while (bits < 32 && ((uint64_t)1 << bits) < n) bits++;
    const uint64_t ntiles = (c + kRsTile - 1) / kRsTile;
    uint32_t *k[2], *v[2], *hist, *asel;
    uint64_t* offs;
    PSC_TRY(ensure_t(g, B_AUX0, c, &k[0]));
    PSC_TRY(ensure_t(g, B_AUX1, c, &v[0]));
    PSC_TRY(ensure_t(g, B_AUX2, c, &k[1]));
    PSC_TRY(ensure_t(g, B_QA, c, &v[1]));
    PSC_TRY(ensure_t(g, B_AUX3, (uint64_t)kRsBins * ntiles, &hist));
    PSC_TRY(ensure_t(g, B_SCAN2, (uint64_t)kRsBins * ntiles + 1, &offs));
    {
      ProfScope ps(g, F_TRANSPOSE);
      ps.bytes = 16.0 * n + 4.0 * m;
      k_edge_sources<<<grid_for(g, (m + kSrcRun - 1) / kSrcRun * 32, 256), 256, 0, g->stream>>>(
          g->off, n, m, v[1]);
    }
    {
      ProfScope ps(g, F_TRANSPOSE);
      ps.bytes = 8.0 * m + 16.0 * m;
      k_sym_pairs<<<grid_for(g, m, 256), 256, 0, g->stream>>>(g->E, v[1], m, k[0], v[0]);
    }
    int at = 0;
    PSC_TRY(radix_pairs(g, c, bits, k, v, hist, offs, &at));  // by target
    // second pass set: the sources become the keys
    uint32_t* k2[2] = {v[at], k[at ^ 1]};
    uint32_t* v2[2] = {k[at], v[at ^ 1]};
    PSC_TRY(radix_pairs(g, c, bits, k2, v2, hist, offs, &at));  // stably by source
    const uint32_t* A = k2[at];
    const uint32_t* B = v2[at];
    release(g, B_AUX3);
    release(g, B_SCAN2);
    // the kept pairs: targets and sources into the free pair of buffers
    asel = v2[at ^ 1];
    uint32_t* bsel = k2[at ^ 1];
    PSC_TRY(scan_emit_flags(g, c, SymKeep{A, B}, SymEmit{A, B, asel, bsel}, &ms, F_TRANSPOSE,
                            8.0, 8.0));
    PSC_CUDA(cudaMallocAsync((void**)&E_s, (ms ? ms : 1) * 4, g->stream));
    if (ms) PSC_CUDA(cudaMemcpyAsync(E_s, bsel, ms * 4, cudaMemcpyDeviceToDevice, g->stream));
    if (ms) {
      uint64_t* rs;
      PSC_TRY(ensure_t(g, B_SCAN3, n + 1, &rs));
      ProfScope ps(g, F_TRANSPOSE);
      ps.bytes = 8.0 * ms;
      k_run_starts<<<grid_for(g, ms, 256), 256, 0, g->stream>>>(asel, ms, rs);
      k_run_lengths<<<grid_for(g, ms, 256), 256, 0, g->stream>>>(asel, ms, rs, cnt);
    }
    release(g, B_AUX0);
    release(g, B_AUX1);
    release(g, B_AUX2);
    release(g, B_QA);
    release(g, B_SCAN3);
  } else {
    PSC_CUDA(cudaMallocAsync((void**)&E_s, 4, g->stream));
  }
  PSC_CUDA(cudaMallocAsync((void**)&off_s, (n + 1) * 8, g->stream));
  uint64_t total = 0;
  PSC_TRY(scan_emit(g, n, CntValue{cnt}, OffEmit{off_s, cnt}, &total, F_TRANSPOSE));
  PSC_CUDA(cudaMemcpyAsync(off_s + n, &ms, 8, cudaMemcpyHostToDevice, g->stream));
  PSC_CUDA(cudaStreamSynchronize(g->stream));  // ms lives on this stack frame
  release(g, B_TMP32);
  if (g->in_off && g->in_off != g->off) cudaFreeAsync(g->in_off, g->stream);
  if (g->in_E && g->in_E != g->E) cudaFreeAsync(g->in_E, g->stream);
  cudaFreeAsync(g->off, g->stream);
  cudaFreeAsync(g->E, g->stream);
  g->off = g->in_off = off_s;
  g->E = g->in_E = E_s;
  g->m = ms;
  g->symmetric = true;
  PSC_CUDA(cudaGetLastError());
  return PSC_OK;
}

}  // namespace psc

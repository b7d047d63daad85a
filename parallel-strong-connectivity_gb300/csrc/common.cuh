// Device-side building blocks shared by every kernel of libpsc_cuda.so:
// the graph handle, status codes, the workspace arena, warp-aggregated
// frontier appends, the balanced warp edge expansion and the 64-bit
// open-addressing (vertex, pivot) table.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/psc.h"
#include "psc_hash.h"

namespace psc {

constexpr uint64_t kTopBit = 1ull << 32;       // src/scc.hpp:22
constexpr uint64_t kValMask = 0xFFFFFFFFull;   // src/scc.hpp:23
constexpr uint32_t kNone = 0xFFFFFFFFu;        // UINT_N_MAX
constexpr uint64_t kEmpty = ~0ull;             // empty (vertex, pivot) slot
constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr int kWarp = 32;
// Frontier vertices with more out-edges than this are expanded by the whole
// grid instead of by one warp.
constexpr uint32_t kHeavyDeg = 8192;
// Heavy-list counters: count << kPackShift | work units (edges or chunks),
// updated with one 64-bit atomic per listed item.
constexpr int kPackShift = 40;
constexpr uint64_t kPackMask = (1ull << kPackShift) - 1;

// ---------------------------------------------------------------------------
// Kernel families for profiling (launch counts, event time, algorithmic bytes)
// ---------------------------------------------------------------------------
enum Family : int {
  F_TRIM = 0,
  F_REACH_PUSH,
  F_REACH_PULL,
  F_REACH_VGC,
  F_HEAVY,
  F_LABEL_FIRST,
  F_COMPACT,
  F_MS_SEED,
  F_MS_EXPAND,
  F_MS_VGC,
  F_TABLE,
  F_PARTITION,
  F_FINALISE,
  F_CC,
  F_LE,
  F_TRANSPOSE,
  F_BATCH,
  F_UF,
  F_LE_SORT,
  F_COUNT
};
extern const char* const kFamilyName[F_COUNT];

// Device counters written by the round kernels and read back between rounds.
// One block per search side (forward / backward run in the same launches).
struct Counters {
  unsigned long long next;       // items appended to the next frontier
  unsigned long long next_edges; // out-edges of the appended items (direction heuristic)
  unsigned long long heavy;      // items sent to the heavy list
  unsigned long long fail;       // failed table inserts (table needs to grow)
  unsigned long long edges;      // edges scanned (algorithmic bytes)
  unsigned long long probes;     // table slots probed (algorithmic bytes)
  unsigned long long aux0;       // kernel-specific (queue cursor of bitmap -> queue)
  unsigned long long aux1;       // kernel-specific (re-queued pairs)
  unsigned long long expanded;   // vertices whose adjacency was read
  unsigned long long unvisited;  // vertices examined by a pull round
  unsigned long long heavy_edges;  // edges scanned by the heavy-vertex kernels
  unsigned long long heavy_probes; // table slots probed by the heavy-pair kernel
  unsigned long long inserted;     // new table entries (multi-search)
  unsigned long long waves;        // local-search waves of VGC rounds (trace)
  unsigned long long pad[2];
};
// sets 0-1: search sides; 2-3: staging; 4-19: the rounds of a chained VGC
// sequence (reach.cu), two sides per round
constexpr int kCounterSets = 20;

// ---------------------------------------------------------------------------
// Host-side helpers
// ---------------------------------------------------------------------------
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

struct ProfEntry {
  uint64_t launches = 0;
  double ms = 0;
  double bytes = 0;
};

struct PendingEvent {
  int fam;
  cudaEvent_t a, b;
  double bytes;
};

}  // namespace psc

struct psc_graph_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  uint64_t n = 0, m = 0;
  bool symmetric = false;
  uint64_t* off = nullptr;
  uint32_t* E = nullptr;
  uint64_t* in_off = nullptr;  // aliases off for symmetric graphs
  uint32_t* in_E = nullptr;
  int num_sms = 0;
  int vgc_blocks = 0;     // resident blocks per SM of the reach VGC kernel
  int ms_vgc_blocks = 0;  // same for the multi-search VGC kernel
  int ldd_vgc_blocks = 0; // same for the LDD VGC kernel
  int le_heavy_blocks = 0; // same for the LE-list heavy-pair kernel
  bool deg_known = false;    // max_deg holds the largest out- / in-degree
  bool dead_known = false;   // B_DEAD holds the unreachable-vertex bitmaps
  uint64_t dead_count[2] = {0, 0};  // vertices with no in-edge / no out-edge
  // per LDD round of the last psc_ldd / psc_cc call: first candidate index,
  // candidates offered, new centres (psc_ldd_rounds)
  std::vector<uint32_t> ldd_trace;
  uint64_t max_deg[2] = {0, 0};
  uint32_t block = 0;     // threads per block of the expansion kernels (0: 256)
  // named scratch buffers, grown on demand (stream-ordered allocator)
  std::vector<psc::DevBuf> bufs;
  psc::Counters* ctr = nullptr;   // device, kCounterSets blocks
  psc::Counters* hctr = nullptr;  // pinned host mirror
  // statistics / profiling
  psc_stats_t stats{};
  bool profiling = false;
  psc::ProfEntry prof[psc::F_COUNT];
  std::vector<psc::PendingEvent> pending;
  std::vector<cudaEvent_t> event_pool;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  cudaEvent_t u0 = nullptr, u1 = nullptr;  // caller timer (psc_timer_*)
  cudaEvent_t ph[4] = {nullptr, nullptr, nullptr, nullptr};  // SCC phase marks
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> grow_events;  // table resizes
  // graph-offset table of a batch of disjoint graphs (psc_batch_set)
  uint32_t num_graphs = 0;
  std::vector<uint64_t> vbase;     // host copy, num_graphs + 1 vertex bases
  uint64_t* d_vbase = nullptr;     // device copy
  uint32_t* d_gid = nullptr;       // u32[n] graph of each vertex
};

namespace psc {

// Scratch buffer slots (indices into psc_graph_s::bufs).
enum Buf : int {
  B_LABELS = 0,   // u64[n] labels when the caller passes host memory
  B_P,            // u32[n] pivot order
  B_CENTERS,      // u32[n]
  B_FRONT,        // u32[n] batch pivots
  B_VIS_F,        // u32[n/32] visited bitmap (forward)
  B_VIS_B,        // u32[n/32] visited bitmap (backward)
  B_QA,           // u32[n] vertex frontier A
  B_QB,           // u32[n] vertex frontier B
  B_FB_A,         // u32[n/32] frontier bitmap A
  B_FB_B,         // u32[n/32] frontier bitmap B
  B_HEAVY,        // heavy list
  B_SCAN,         // scan scratch
  B_SCAN2,        // radix offsets of the device transpose
  B_SCAN3,        // run starts of the device transpose
  B_TMP32,        // u32[n] misc
  B_TF,           // forward label table
  B_TB,           // backward label table
  B_TS,           // spare table for rehash
  B_PA,           // u64 pair frontier A
  B_PB,           // u64 pair frontier B
  B_PH,           // u64 pair heavy list
  B_QA2,          // second search side (backward) of a two-sided reach
  B_QB2,
  B_FB_A2,
  B_FB_B2,
  B_HEAVY2,
  B_PA2,          // second multi-search side's pair frontiers / heavy list / flags
  B_PB2,
  B_PH2,
  B_HF2,
  B_AUX0,
  B_AUX1,
  B_AUX2,
  B_AUX3,
  B_GRAPHS,       // per-graph arrays of a batch
  B_FLAB,         // u32 labels of a batch's pivots
  B_SCHED,        // window schedule of a batch's prefix-doubling rounds
  B_SCANBITS,     // u32[n/32] selection bits of scan_emit_flags
  B_DEAD,         // u32[2][n/32 + 1] vertices with no in-edge, then no out-edge
  B_COUNT
};

// Status plumbing: PSC_TRY returns the status of a failing expression.
#define PSC_TRY(expr)                 \
  do {                                \
    int _s = (expr);                  \
    if (_s != PSC_OK) return _s;      \
  } while (0)

#define PSC_CUDA(expr)                                         \
  do {                                                         \
    cudaError_t _e = (expr);                                   \
    if (_e != cudaSuccess) return ::psc::cuda_status(_e);      \
  } while (0)

int cuda_status(cudaError_t e);
// Round tracing to stderr when the environment sets PSC_TRACE (the reference
// prints per-round frontier sizes under DEBUG, src/reach.hpp:218-239).
bool trace_on();
// Per-batch server timeline only (PSC_TRACE_SERVER, or PSC_TRACE), without the
// per-round lines and their waits.
bool trace_server_on();
void set_last_cuda_error(cudaError_t e);

// Returns a device pointer of at least `bytes` for slot `b` (contents of a
// regrown buffer are not preserved).
int ensure(psc_graph_s* g, int b, size_t bytes, void** out);
template <class T>
inline int ensure_t(psc_graph_s* g, int b, size_t count, T** out) {
  void* p = nullptr;
  int s = ensure(g, b, count * sizeof(T) + 16, &p);
  *out = (T*)p;
  return s;
}
// Swap two slots (ping-pong buffers).
void swap_bufs(psc_graph_s* g, int a, int b);

// Reads the device counters to the host mirror and waits for the stream.
int read_counters(psc_graph_s* g);
int zero_counters(psc_graph_s* g);

// Profiling brackets (no-ops unless profiling is on).
void prof_begin(psc_graph_s* g, int fam, cudaEvent_t* a);
void prof_end(psc_graph_s* g, int fam, cudaEvent_t a, double bytes);
int prof_flush(psc_graph_s* g);
cudaEvent_t take_event(psc_graph_s* g);
void give_event(psc_graph_s* g, cudaEvent_t e);

struct ProfScope {
  psc_graph_s* g;
  int fam;
  cudaEvent_t a = nullptr;
  double bytes = 0;
  ProfScope(psc_graph_s* g_, int f) : g(g_), fam(f) {
    g->stats.kernel_launches++;
    prof_begin(g, fam, &a);
  }
  ~ProfScope() { prof_end(g, fam, a, bytes); }
};

inline unsigned grid_for(psc_graph_s* g, uint64_t items, unsigned block, unsigned per_thread = 1) {
  uint64_t want = (items + (uint64_t)block * per_thread - 1) / ((uint64_t)block * per_thread);
  uint64_t cap = (uint64_t)g->num_sms * 16;
  if (want < 1) want = 1;
  if (want > cap) want = cap;
  return (unsigned)want;
}

// ---------------------------------------------------------------------------
// Device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Rejects a CSR whose offsets do not run from 0 to m without decreasing or
// whose targets are not vertex ids: sets *bad.  Only the arrays themselves
// are read (no access is indexed by their values), so any input of the
// declared sizes is safe to check.  16-byte aligned arrays are read with
// 128-bit loads (two offsets or four targets per load); others one element
// at a time.  A template so that every translation unit that launches it
// holds its own instance.
template <int kUnused = 0>
__global__ void k_validate_csr(const uint64_t* __restrict__ off, uint64_t n,
                               const uint32_t* __restrict__ E, uint64_t m,
                               unsigned long long* bad) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool b = t == 0 && (off[0] != 0 || off[n] != m);
  if (((uintptr_t)off & 15) == 0) {
    // pair j = off[2j], off[2j + 1]; its successor off[2j + 2] (<= off[n])
    const uint64_t np = n / 2;
    const ulonglong2* o2 = reinterpret_cast<const ulonglong2*>(off);
    for (uint64_t j = t; j < np; j += stride) {
      const ulonglong2 a = __ldg(&o2[j]);
      b |= a.x > a.y || a.y > __ldg(&off[2 * j + 2]);
    }
    if ((n & 1) && t == 0) b |= off[n - 1] > off[n];
  } else {
    for (uint64_t v = t; v < n; v += stride) b |= off[v] > off[v + 1];
  }
  if (((uintptr_t)E & 15) == 0) {
    const uint64_t nq = m / 4;
    const uint4* e4 = reinterpret_cast<const uint4*>(E);
    for (uint64_t q = t; q < nq; q += stride) {
      const uint4 x = __ldg(&e4[q]);
      b |= x.x >= n || x.y >= n || x.z >= n || x.w >= n;
    }
    for (uint64_t i = nq * 4 + t; i < m; i += stride) b |= E[i] >= n;
  } else {
    for (uint64_t i = t; i < m; i += stride) b |= E[i] >= n;
  }
  if (__any_sync(kFull, b) && lane_id() == 0) atomicOr(bad, 1ull);
}

__device__ __forceinline__ uint64_t ld_cg(const uint64_t* p) { return __ldcg((const unsigned long long*)p); }
__device__ __forceinline__ uint32_t ld_cg(const uint32_t* p) { return __ldcg(p); }

// Warp-aggregated append: every lane of the (converged) warp calls it; lanes
// with take == true receive consecutive slots of *counter.
__device__ __forceinline__ unsigned long long warp_append(unsigned long long* counter, bool take) {
  unsigned mask = __ballot_sync(kFull, take);
  if (mask == 0) return 0;
  unsigned lane = lane_id();
  int leader = __ffs(mask) - 1;
  unsigned long long base = 0;
  if ((int)lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(mask));
  base = __shfl_sync(kFull, base, leader);
  return base + __popc(mask & ((1u << lane) - 1u));
}

// Warp-aggregated append of a batch: lane's values vals[k] with bit k of tm
// set are written to consecutive slots of out claimed with one atomicAdd on
// *counter for the whole warp.  Every lane of the warp calls it.
template <int K, class T>
__device__ __forceinline__ void warp_append_batch(uint32_t tm, const T* vals, T* out,
                                                  unsigned long long* counter) {
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
  unsigned long long base = 0;
  if (lane == 31) base = atomicAdd(counter, (unsigned long long)total);
  base = __shfl_sync(kFull, base, 31) + (incl - cnt);
#pragma unroll
  for (int k = 0; k < K; k++)
    if (tm & (1u << k)) out[base++] = vals[k];
}

// Warp sum of a u64 value.
__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// Largest k in [0, cnt) with a[k] <= x, for a nondecreasing a with a[0] <= x.
template <class T>
__device__ __forceinline__ uint32_t last_le(const T* __restrict__ a, uint32_t cnt, uint64_t x) {
  uint32_t lo = 0, hi = cnt;  // a[lo] <= x, a[hi] > x (virtually for hi == cnt)
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if ((uint64_t)a[mid] <= x)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Per-warp shared state of the balanced expansion.
struct WarpExpandSmem {
  uint32_t excl[32];
  uint64_t beg[32];
  uint32_t fail;  // per-source-lane failure bits (multi-search)
};

// Balanced edge expansion over the 32 lanes' adjacency ranges [beg, beg+deg):
// the warp walks the concatenation of the ranges 32 edges at a time, every
// lane owning one edge per step (coalesced reads of E).  visit(src_lane, e)
// returns nothing; all lanes call it with active == false past the end so
// warp collectives inside visit stay converged.
template <class Visit>
__device__ __forceinline__ void warp_expand(WarpExpandSmem& sm, uint64_t beg, uint32_t deg,
                                            Visit&& visit) {
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
  for (uint32_t base = 0; base < total; base += 32) {
    const uint32_t gi = base + lane;
    const bool active = gi < total;
    int src = 0;
    uint64_t e = 0;
    if (active) {
      // largest lane s with excl[s] <= gi
      int lo = 0, hi = 31;
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (sm.excl[mid] <= gi)
          lo = mid;
        else
          hi = mid - 1;
      }
      src = lo;
      e = sm.beg[src] + (gi - sm.excl[src]);
    }
    visit(active, src, e);
  }
  __syncwarp();
}

// Insert key into a linear-probing table of 2^k slots.
// Returns 1 if inserted, 0 if already present, -1 after `limit` probes.
__device__ __forceinline__ int table_insert(unsigned long long* T, uint64_t mask, uint64_t key,
                                            uint32_t limit, uint32_t* probes) {
  uint64_t h = hash64(key) & mask;
  for (uint32_t i = 0; i < limit; i++) {
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
    h = (h + 1) & mask;
  }
  *probes += limit;
  return -1;
}

__device__ __forceinline__ bool table_contains(const unsigned long long* T, uint64_t mask,
                                               uint64_t key) {
  uint64_t h = hash64(key) & mask;
  for (uint64_t i = 0; i <= mask; i++) {
    uint64_t cur = T[h];
    if (cur == key) return true;
    if (cur == kEmpty) return false;
    h = (h + 1) & mask;
  }
  return false;
}

__device__ __forceinline__ bool bit_test(const uint32_t* bm, uint32_t v) {
  return (__ldcg(&bm[v >> 5]) >> (v & 31)) & 1u;
}

// Sets bit v; returns true if this call flipped it from 0 to 1.
__device__ __forceinline__ bool bit_set(uint32_t* bm, uint32_t v) {
  uint32_t b = 1u << (v & 31);
  if (__ldcg(&bm[v >> 5]) & b) return false;
  return !(atomicOr(&bm[v >> 5], b) & b);
}

}  // namespace psc

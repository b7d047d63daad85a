// Handle lifecycle, scratch buffers, counters, profiling and graph upload
// for libpsc_cuda.so.  Declared in include/psc.h.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "engines.cuh"
#include "scan.cuh"

namespace psc {

const char* const kFamilyName[F_COUNT] = {
    "trim",        "reach_push", "reach_pull", "reach_vgc", "heavy",     "label_first",
    "compact",     "ms_seed",    "ms_expand",  "ms_vgc",    "table",     "partition",
    "finalise",    "cc",         "lelist",     "transpose",  "batch",     "union_find",
    "lelist_sort"};

static thread_local cudaError_t g_last_cuda = cudaSuccess;

void set_last_cuda_error(cudaError_t e) { g_last_cuda = e; }

// Counter blocks (device + pinned host) are recycled across handles instead
// of freed: cudaFree and cudaFreeHost synchronize the whole device, which
// would stall every other stream (the request server's other workers) each
// time a handle goes away.
namespace {
struct CtrBlock {
  int device;
  Counters* d;
  Counters* h;
};
std::mutex g_ctr_mu;
std::vector<CtrBlock> g_ctr_pool;

cudaError_t ctr_take(int dev, Counters** d, Counters** h) {
  {
    std::lock_guard<std::mutex> lk(g_ctr_mu);
    for (size_t i = 0; i < g_ctr_pool.size(); i++)
      if (g_ctr_pool[i].device == dev) {
        *d = g_ctr_pool[i].d;
        *h = g_ctr_pool[i].h;
        g_ctr_pool[i] = g_ctr_pool.back();
        g_ctr_pool.pop_back();
        return cudaSuccess;
      }
  }
  cudaError_t e = cudaMalloc(d, kCounterSets * sizeof(Counters));
  if (e != cudaSuccess) return e;
  e = cudaMallocHost(h, kCounterSets * sizeof(Counters));
  if (e != cudaSuccess) {
    cudaFree(*d);
    *d = nullptr;
  }
  return e;
}

void ctr_give(int dev, Counters* d, Counters* h) {
  std::lock_guard<std::mutex> lk(g_ctr_mu);
  g_ctr_pool.push_back(CtrBlock{dev, d, h});
}
}  // namespace

bool trace_on() {
  static const bool on = [] {
    const char* v = std::getenv("PSC_TRACE");
    return v && *v && *v != '0';
  }();
  return on;
}

bool trace_server_on() {
  static const bool on = [] {
    const char* v = std::getenv("PSC_TRACE_SERVER");
    return trace_on() || (v && *v && *v != '0');
  }();
  return on;
}

int cuda_status(cudaError_t e) {
  g_last_cuda = e;
  if (e == cudaErrorMemoryAllocation) return PSC_ERR_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return PSC_ERR_NO_DEVICE;
  return PSC_ERR_CUDA;
}

int ensure(psc_graph_s* g, int b, size_t bytes, void** out) {
  DevBuf& d = g->bufs[b];
  if (d.bytes < bytes) {
    if (d.p) PSC_CUDA(cudaFreeAsync(d.p, g->stream));
    d.p = nullptr;
    d.bytes = 0;
    cudaError_t e = cudaMallocAsync(&d.p, bytes, g->stream);
    if (e != cudaSuccess) {
      cudaGetLastError();
      d.p = nullptr;
      return cuda_status(e);
    }
    d.bytes = bytes;
  }
  *out = d.p;
  return PSC_OK;
}

int ensure_keep(psc_graph_s* g, int b, size_t bytes, size_t keep, void** out) {
  DevBuf& d = g->bufs[b];
  if (d.bytes >= bytes) {
    *out = d.p;
    return PSC_OK;
  }
  void* np = nullptr;
  cudaError_t e = cudaMallocAsync(&np, bytes, g->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return cuda_status(e);
  }
  if (d.p && keep) PSC_CUDA(cudaMemcpyAsync(np, d.p, keep, cudaMemcpyDeviceToDevice, g->stream));
  if (d.p) PSC_CUDA(cudaFreeAsync(d.p, g->stream));
  d.p = np;
  d.bytes = bytes;
  *out = np;
  return PSC_OK;
}

void swap_bufs(psc_graph_s* g, int a, int b) { std::swap(g->bufs[a], g->bufs[b]); }

int zero_counters(psc_graph_s* g) {
  PSC_CUDA(cudaMemsetAsync(g->ctr, 0, kCounterSets * sizeof(Counters), g->stream));
  return PSC_OK;
}

int read_counters(psc_graph_s* g) {
  PSC_CUDA(cudaMemcpyAsync(g->hctr, g->ctr, kCounterSets * sizeof(Counters),
                           cudaMemcpyDeviceToHost, g->stream));
  PSC_CUDA(cudaStreamSynchronize(g->stream));
  return PSC_OK;
}

cudaEvent_t take_event(psc_graph_s* g) {
  if (!g->event_pool.empty()) {
    cudaEvent_t e = g->event_pool.back();
    g->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void give_event(psc_graph_s* g, cudaEvent_t e) { g->event_pool.push_back(e); }

void prof_begin(psc_graph_s* g, int, cudaEvent_t* a) {
  if (!g->profiling) return;
  *a = take_event(g);
  cudaEventRecord(*a, g->stream);
}

void prof_end(psc_graph_s* g, int fam, cudaEvent_t a, double bytes) {
  if (!g->profiling || !a) return;
  cudaEvent_t b = take_event(g);
  cudaEventRecord(b, g->stream);
  g->pending.push_back(PendingEvent{fam, a, b, bytes});
  if (g->pending.size() > 4096) prof_flush(g);
}

int prof_flush(psc_graph_s* g) {
  if (g->pending.empty()) return PSC_OK;
  PSC_CUDA(cudaStreamSynchronize(g->stream));
  for (auto& p : g->pending) {
    float ms = 0;
    cudaEventElapsedTime(&ms, p.a, p.b);
    g->prof[p.fam].launches++;
    g->prof[p.fam].ms += ms;
    g->prof[p.fam].bytes += p.bytes;
    g->event_pool.push_back(p.a);
    g->event_pool.push_back(p.b);
  }
  g->pending.clear();
  return PSC_OK;
}

__global__ void __launch_bounds__(1024) k_scan_tile_sums(uint64_t* a, uint64_t nt) {
  __shared__ uint64_t sm[33];
  uint64_t carry = 0;
  for (uint64_t base = 0; base < nt; base += 1024) {
    uint64_t i = base + threadIdx.x;
    uint64_t v = i < nt ? a[i] : 0;
    uint64_t tot;
    uint64_t ex = block_excl_scan<1024>(v, sm, &tot);
    if (i < nt) a[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) a[nt] = carry;
}

int call_begin(psc_graph_s* g) {
  PSC_CUDA(cudaSetDevice(g->device));
  std::memset(&g->stats, 0, sizeof(g->stats));
  PSC_CUDA(cudaEventRecord(g->t0, g->stream));
  return PSC_OK;
}

int call_end(psc_graph_s* g) {
  PSC_CUDA(cudaEventRecord(g->t1, g->stream));
  PSC_CUDA(cudaEventSynchronize(g->t1));
  float ms = 0;
  PSC_CUDA(cudaEventElapsedTime(&ms, g->t0, g->t1));
  g->stats.total_ms = ms;
  PSC_TRY(prof_flush(g));
  PSC_CUDA(cudaGetLastError());
  return PSC_OK;
}

int make_handle(uint64_t n, uint64_t m, psc_graph_s** out, int priority) {
  int dev = 0;
  PSC_CUDA(cudaGetDevice(&dev));
  auto* g = new psc_graph_s();
  g->device = dev;
  g->n = n;
  g->m = m;
  g->bufs.resize(B_COUNT);
  cudaError_t e;
  if ((e = cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
      (e = cudaStreamCreateWithPriority(&g->stream, cudaStreamNonBlocking, priority)) != cudaSuccess ||
      (e = ctr_take(dev, &g->ctr, &g->hctr)) != cudaSuccess ||
      (e = cudaEventCreate(&g->t0)) != cudaSuccess || (e = cudaEventCreate(&g->t1)) != cudaSuccess ||
      (e = cudaEventCreate(&g->u0)) != cudaSuccess || (e = cudaEventCreate(&g->u1)) != cudaSuccess ||
      (e = cudaEventCreate(&g->ph[0])) != cudaSuccess || (e = cudaEventCreate(&g->ph[1])) != cudaSuccess ||
      (e = cudaEventCreate(&g->ph[2])) != cudaSuccess || (e = cudaEventCreate(&g->ph[3])) != cudaSuccess) {
    psc_graph_free(g);
    return cuda_status(e);
  }
  // keep freed scratch in the pool between calls
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  *out = g;
  return PSC_OK;
}

// Graph arrays come from the device's stream-ordered pool (kept between
// handles), so repeated uploads of same-sized graphs do not map new memory.
int alloc_graph_arrays(psc_graph_s* g, bool symmetric) {
  const uint64_t n = g->n, m = g->m;
  g->symmetric = symmetric;
  PSC_CUDA(cudaMallocAsync((void**)&g->off, (n + 1) * sizeof(uint64_t), g->stream));
  PSC_CUDA(cudaMallocAsync((void**)&g->E, (m ? m : 1) * sizeof(uint32_t), g->stream));
  if (symmetric) {
    g->in_off = g->off;
    g->in_E = g->E;
  } else {
    PSC_CUDA(cudaMallocAsync((void**)&g->in_off, (n + 1) * sizeof(uint64_t), g->stream));
    PSC_CUDA(cudaMallocAsync((void**)&g->in_E, (m ? m : 1) * sizeof(uint32_t), g->stream));
  }
  return PSC_OK;
}

// Copies the caller's arrays (host or device) into the handle's graph arrays
// on its stream and waits for them, so the caller may reuse its buffers.
// Malformed arrays are refused by k_validate_csr (common.cuh) before any
// traversal kernel, which indexes by their values, runs on them.
// Checks the graph arrays of a fresh handle (the transpose too when it was
// given and does not alias); PSC_ERR_INVALID if one is malformed.
static int validate_graph(psc_graph_s* g, bool with_transpose) {
  unsigned long long* bad = &g->ctr[2].aux0;  // staging set of the fresh handle
  PSC_CUDA(cudaMemsetAsync(bad, 0, sizeof(unsigned long long), g->stream));
  const unsigned grid = grid_for(g, std::max<uint64_t>(g->n, g->m), 256);
  k_validate_csr<><<<grid, 256, 0, g->stream>>>(g->off, g->n, g->E, g->m, bad);
  if (with_transpose && g->in_off && g->in_off != g->off)
    k_validate_csr<><<<grid, 256, 0, g->stream>>>(g->in_off, g->n, g->in_E, g->m, bad);
  PSC_CUDA(cudaGetLastError());
  PSC_TRY(read_counters(g));
  return g->hctr[2].aux0 ? PSC_ERR_INVALID : PSC_OK;
}

static int copy_graph_arrays(psc_graph_s* g, const uint64_t* off, const uint32_t* E,
                             const uint64_t* in_off, const uint32_t* in_E) {
  const uint64_t n = g->n, m = g->m;
  PSC_CUDA(cudaMemcpyAsync(g->off, off, (n + 1) * 8, cudaMemcpyDefault, g->stream));
  if (m) PSC_CUDA(cudaMemcpyAsync(g->E, E, m * 4, cudaMemcpyDefault, g->stream));
  if (!g->symmetric && in_off) {
    PSC_CUDA(cudaMemcpyAsync(g->in_off, in_off, (n + 1) * 8, cudaMemcpyDefault, g->stream));
    if (m) PSC_CUDA(cudaMemcpyAsync(g->in_E, in_E, m * 4, cudaMemcpyDefault, g->stream));
  }
  PSC_CUDA(cudaStreamSynchronize(g->stream));
  return PSC_OK;
}

}  // namespace psc

using namespace psc;

extern "C" {

void psc_params_default(psc_params_t* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->beta = 1.5;
  p->tau = 512;
  p->lambda = 1024;
  p->local_reach = 1;
  p->local_scc = 1;
  p->seed = 1;
}

int psc_graph_upload(const uint64_t* off, const uint32_t* E, const uint64_t* in_off,
                     const uint32_t* in_E, uint64_t n, uint64_t m, psc_graph_t* out) {
  if (!out || !off || (m && !E) || n == 0 || n >= 0xFFFFFFFFull) return PSC_ERR_INVALID;
  if ((in_off == nullptr) != (in_E == nullptr)) return PSC_ERR_INVALID;
  if (off[0] != 0 || off[n] != m) return PSC_ERR_INVALID;
  if (in_off && (in_off[0] != 0 || in_off[n] != m)) return PSC_ERR_INVALID;
  psc_graph_s* g = nullptr;
  PSC_TRY(make_handle(n, m, &g));
  bool sym = in_off == nullptr;
  int s = alloc_graph_arrays(g, sym);
  if (s == PSC_OK) s = copy_graph_arrays(g, off, E, in_off, in_E);
  if (s == PSC_OK) s = validate_graph(g, true);
  if (s != PSC_OK) {
    psc_graph_free(g);
    return s;
  }
  *out = g;
  return PSC_OK;
}

int psc_graph_upload_device(const uint64_t* d_off, const uint32_t* d_E, const uint64_t* d_in_off,
                            const uint32_t* d_in_E, uint64_t n, uint64_t m, psc_graph_t* out) {
  if (!out || !d_off || (m && !d_E) || n == 0 || n >= 0xFFFFFFFFull) return PSC_ERR_INVALID;
  if ((d_in_off == nullptr) != (d_in_E == nullptr)) return PSC_ERR_INVALID;
  psc_graph_s* g = nullptr;
  PSC_TRY(make_handle(n, m, &g));
  bool sym = d_in_off == nullptr;
  int s = alloc_graph_arrays(g, sym);
  if (s == PSC_OK) s = copy_graph_arrays(g, d_off, d_E, d_in_off, d_in_E);
  if (s == PSC_OK) s = validate_graph(g, true);
  if (s != PSC_OK) {
    psc_graph_free(g);
    return s;
  }
  *out = g;
  return PSC_OK;
}

int psc_graph_upload_directed(const uint64_t* off, const uint32_t* E, uint64_t n, uint64_t m,
                              psc_graph_t* out) {
  if (!out || !off || (m && !E) || n == 0 || n >= 0xFFFFFFFFull) return PSC_ERR_INVALID;
  if (off[0] != 0 || off[n] != m) return PSC_ERR_INVALID;
  psc_graph_s* g = nullptr;
  PSC_TRY(make_handle(n, m, &g));
  int s = alloc_graph_arrays(g, false);
  if (s == PSC_OK) s = copy_graph_arrays(g, off, E, nullptr, nullptr);
  if (s == PSC_OK) s = validate_graph(g, false);  // the transpose build indexes by E
  if (s == PSC_OK) s = build_transpose(g);
  if (s == PSC_OK) {
    cudaError_t e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) s = cuda_status(e);
  }
  if (s != PSC_OK) {
    psc_graph_free(g);
    return s;
  }
  *out = g;
  return PSC_OK;
}

int psc_graph_upload_symmetrize(const uint64_t* off, const uint32_t* E, uint64_t n, uint64_t m,
                                psc_graph_t* out) {
  if (!out || !off || (m && !E) || n == 0 || n >= 0xFFFFFFFFull || m >= (1ull << 39))
    return PSC_ERR_INVALID;
  psc_graph_s* g = nullptr;
  PSC_TRY(make_handle(n, m, &g));
  int s = alloc_graph_arrays(g, true);
  if (s == PSC_OK) s = copy_graph_arrays(g, off, E, nullptr, nullptr);
  if (s == PSC_OK) s = validate_graph(g, false);  // the pair build indexes by off and E
  if (s == PSC_OK) s = build_symmetric(g);
  if (s == PSC_OK) {
    cudaError_t e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) s = cuda_status(e);
  }
  if (s != PSC_OK) {
    psc_graph_free(g);
    return s;
  }
  *out = g;
  return PSC_OK;
}

int psc_graph_download(psc_graph_t g, uint64_t* off, uint32_t* E) {
  if (!g || !off || (g->m && !E)) return PSC_ERR_INVALID;
  PSC_CUDA(cudaSetDevice(g->device));
  PSC_CUDA(cudaStreamSynchronize(g->stream));
  PSC_CUDA(cudaMemcpy(off, g->off, (g->n + 1) * 8, cudaMemcpyDeviceToHost));
  if (g->m) PSC_CUDA(cudaMemcpy(E, g->E, g->m * 4, cudaMemcpyDeviceToHost));
  return PSC_OK;
}

int psc_graph_download_transpose(psc_graph_t g, uint64_t* in_off, uint32_t* in_E) {
  if (!g || !in_off || (g->m && !in_E)) return PSC_ERR_INVALID;
  PSC_CUDA(cudaSetDevice(g->device));
  PSC_CUDA(cudaStreamSynchronize(g->stream));
  PSC_CUDA(cudaMemcpy(in_off, g->in_off, (g->n + 1) * 8, cudaMemcpyDeviceToHost));
  if (g->m) PSC_CUDA(cudaMemcpy(in_E, g->in_E, g->m * 4, cudaMemcpyDeviceToHost));
  return PSC_OK;
}

int psc_graph_free(psc_graph_t g) {
  if (!g) return PSC_OK;
  cudaSetDevice(g->device);
  if (g->stream) cudaStreamSynchronize(g->stream);
  for (auto& b : g->bufs)
    if (b.p) cudaFreeAsync(b.p, g->stream);
  if (g->in_off && g->in_off != g->off) cudaFreeAsync(g->in_off, g->stream);
  if (g->in_E && g->in_E != g->E) cudaFreeAsync(g->in_E, g->stream);
  if (g->off) cudaFreeAsync(g->off, g->stream);
  if (g->E) cudaFreeAsync(g->E, g->stream);
  if (g->d_vbase) cudaFreeAsync(g->d_vbase, g->stream);
  if (g->d_gid) cudaFreeAsync(g->d_gid, g->stream);
  if (g->stream) cudaStreamSynchronize(g->stream);
  if (g->ctr) ctr_give(g->device, g->ctr, g->hctr);
  for (auto& p : g->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto e : g->event_pool) cudaEventDestroy(e);
  if (g->t0) cudaEventDestroy(g->t0);
  if (g->t1) cudaEventDestroy(g->t1);
  for (auto e : g->ph)
    if (e) cudaEventDestroy(e);
  for (auto& pr : g->grow_events) {
    cudaEventDestroy(pr.first);
    cudaEventDestroy(pr.second);
  }
  if (g->u0) cudaEventDestroy(g->u0);
  if (g->u1) cudaEventDestroy(g->u1);
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
  return PSC_OK;
}

uint64_t psc_graph_num_vertices(psc_graph_t g) { return g ? g->n : 0; }
uint64_t psc_graph_num_edges(psc_graph_t g) { return g ? g->m : 0; }

int psc_last_stats(psc_graph_t g, psc_stats_t* out) {
  if (!g || !out) return PSC_ERR_INVALID;
  *out = g->stats;
  return PSC_OK;
}

int psc_set_profiling(psc_graph_t g, int on) {
  if (!g) return PSC_ERR_INVALID;
  g->profiling = on != 0;
  return PSC_OK;
}

int psc_profile_count(void) { return F_COUNT; }

int psc_profile_get(psc_graph_t g, int k, const char** name, uint64_t* launches, double* ms,
                    double* bytes) {
  if (!g || k < 0 || k >= F_COUNT) return PSC_ERR_INVALID;
  if (name) *name = kFamilyName[k];
  if (launches) *launches = g->prof[k].launches;
  if (ms) *ms = g->prof[k].ms;
  if (bytes) *bytes = g->prof[k].bytes;
  return PSC_OK;
}

int psc_profile_reset(psc_graph_t g) {
  if (!g) return PSC_ERR_INVALID;
  for (auto& p : g->prof) p = ProfEntry{};
  return PSC_OK;
}

const char* psc_strerror(int s) {
  switch (s) {
    case PSC_OK: return "ok";
    case PSC_ERR_INVALID: return "invalid argument";
    case PSC_ERR_OOM: return "device out of memory";
    case PSC_ERR_CUDA: return cudaGetErrorString(g_last_cuda);
    case PSC_ERR_ITER_LIMIT: return "round loop exceeded its iteration bound";
    case PSC_ERR_TABLE_FULL: return "label table could not grow";
    case PSC_ERR_NO_DEVICE: return "no usable CUDA device";
    case PSC_ERR_CAPACITY: return "output buffer too small";
    case PSC_ERR_TOO_LARGE:
      return "graph exceeds the fixed scratch of psc_reach_noalloc (PSC_NOALLOC_MAX_VERTICES)";
    default: return "unknown status";
  }
}

int psc_host_alloc(size_t bytes, void** ptr) {
  if (!ptr) return PSC_ERR_INVALID;
  *ptr = nullptr;
  PSC_CUDA(cudaMallocHost(ptr, bytes ? bytes : 1));
  return PSC_OK;
}

int psc_host_free(void* ptr) {
  if (ptr) PSC_CUDA(cudaFreeHost(ptr));
  return PSC_OK;
}

int psc_device_alloc(size_t bytes, void** ptr) {
  if (!ptr) return PSC_ERR_INVALID;
  *ptr = nullptr;
  PSC_CUDA(cudaMalloc(ptr, bytes ? bytes : 1));
  return PSC_OK;
}

int psc_device_free(void* ptr) {
  if (ptr) PSC_CUDA(cudaFree(ptr));
  return PSC_OK;
}

int psc_copy(void* dst, const void* src, size_t bytes) {
  if ((!dst || !src) && bytes) return PSC_ERR_INVALID;
  if (bytes) PSC_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDefault));
  return PSC_OK;
}

int psc_timer_start(psc_graph_t g) {
  if (!g) return PSC_ERR_INVALID;
  PSC_CUDA(cudaSetDevice(g->device));
  PSC_CUDA(cudaEventRecord(g->u0, g->stream));
  return PSC_OK;
}

int psc_timer_stop(psc_graph_t g, double* ms) {
  if (!g || !ms) return PSC_ERR_INVALID;
  PSC_CUDA(cudaEventRecord(g->u1, g->stream));
  PSC_CUDA(cudaEventSynchronize(g->u1));
  float f = 0;
  PSC_CUDA(cudaEventElapsedTime(&f, g->u0, g->u1));
  *ms = f;
  return PSC_OK;
}

int psc_set_device(int device) {
  PSC_CUDA(cudaSetDevice(device));
  return PSC_OK;
}

int psc_device_count(void) {
  int c = 0;
  if (cudaGetDeviceCount(&c) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return c;
}

const char* psc_version(void) { return "psc-gb300 0.1 (sm_103a)"; }

}  // extern "C"

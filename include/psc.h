/*
 * psc.h — C ABI of the GB300 (sm_103a) strong-connectivity library
 * (libpsc_cuda.so).  Plain pointers and sizes only; every call is
 * host-synchronous and runs on the handle's own CUDA stream.  Distinct handles
 * may be used from different threads at once; one handle is used by one
 * thread at a time (the reference's SCC / REACH / LE_LIST objects are not
 * thread-safe either, src/scc.hpp:38-115).
 *
 * Graph layout (struct Graph, src/graph.hpp:35-43): CSR offsets u64[n+1],
 * targets u32[m], and the transpose in_off/in_E.  Vertex ids are u32.
 *
 * Return value: 0 (PSC_OK) or a PSC_ERR_* status; psc_strerror() names it.
 * The reference returns no errors (I/O failures abort, a full label table is
 * retried internally, src/scc.hpp:256-275); this library retries the same
 * cases internally and reports only what it cannot recover from.
 */
#ifndef PSC_H
#define PSC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  PSC_OK = 0,
  PSC_ERR_INVALID = 1,    /* bad argument */
  PSC_ERR_OOM = 2,        /* device allocation failed */
  PSC_ERR_CUDA = 3,       /* CUDA runtime error */
  PSC_ERR_ITER_LIMIT = 4, /* a round loop exceeded its bound */
  PSC_ERR_TABLE_FULL = 5, /* label table could not grow further */
  PSC_ERR_NO_DEVICE = 6,  /* no usable CUDA device */
  PSC_ERR_CAPACITY = 7,   /* caller buffer too small (see the function) */
  PSC_ERR_TOO_LARGE = 8   /* graph exceeds psc_reach_noalloc's fixed scratch */
};

typedef struct psc_graph_s* psc_graph_t;

/* Parameters of SCC (src/scc.cpp:40-55 flags and their defaults). */
typedef struct {
  double beta;         /* prefix-doubling growth, -beta (1.5) */
  uint32_t tau;        /* VGC local-search budget, global `tau` (512) */
  uint32_t lambda;     /* -lambda min bag size; device frontiers need no bag, accepted for parity */
  int32_t local_reach; /* -local_reach: VGC in the first-pivot reach */
  int32_t local_scc;   /* -local_scc: VGC in the multi-search */
  uint64_t seed;       /* pivot permutation seed (stands in for parlay::random_shuffle) */
  /* tuning knobs (0 = library default) */
  uint32_t block;      /* threads per block of the push / pull / expansion kernels: 128, 256 or 512 (256) */
  uint32_t pull_div;   /* reach switches to pull when frontier edges > m / pull_div (20) */
} psc_params_t;

/* Fills the reference defaults: beta 1.5, tau 512, lambda 1024,
 * local_reach = local_scc = 1 (the paper setting), seed 1. */
void psc_params_default(psc_params_t* p);

/* Uploads a CSR and its transpose (SCC's constructor, src/scc.hpp:81-92,
 * holds the caller's Graph by reference; this copies it into HBM once).
 * in_off/in_E may be NULL for a symmetric graph (transpose = itself).
 * All three uploads check the arrays on the device before any other kernel
 * reads them: offsets from 0 to m, never decreasing, and targets below n;
 * otherwise PSC_ERR_INVALID (the reference would read out of bounds). */
int psc_graph_upload(const uint64_t* off, const uint32_t* E, const uint64_t* in_off,
                     const uint32_t* in_E, uint64_t n, uint64_t m, psc_graph_t* out);
/* Uploads a CSR and builds the transpose on the device
 * (make_directed, src/graph.hpp:222-245). */
int psc_graph_upload_directed(const uint64_t* off, const uint32_t* E, uint64_t n, uint64_t m,
                              psc_graph_t* out);
/* Same graph as psc_graph_upload, but the arrays are already in device memory
 * of the current device; they are copied (device to device). */
int psc_graph_upload_device(const uint64_t* d_off, const uint32_t* d_E, const uint64_t* d_in_off,
                            const uint32_t* d_in_E, uint64_t n, uint64_t m, psc_graph_t* out);
int psc_graph_free(psc_graph_t g);
uint64_t psc_graph_num_vertices(psc_graph_t g);
uint64_t psc_graph_num_edges(psc_graph_t g);
/* Copies the device transpose back (in_off u64[n+1], in_E u32[m]). */
int psc_graph_download_transpose(psc_graph_t g, uint64_t* in_off, uint32_t* in_E);
/* Uploads a directed CSR (host or device memory) and symmetrises it on the
 * device: make_symmetric (src/graph.hpp:187-220) -- every edge in both
 * directions, each adjacency list sorted, duplicate edges and self-loops
 * dropped -- as read_graph(.., symmetric = true) does (:248-277).  The handle
 * holds the symmetric graph: psc_graph_num_edges gives its edge count,
 * psc_graph_download its arrays.  The input is checked as psc_graph_upload
 * checks it (PSC_ERR_INVALID). */
int psc_graph_upload_symmetrize(const uint64_t* off, const uint32_t* E, uint64_t n, uint64_t m,
                                psc_graph_t* out);
/* Copies the handle's CSR back (off u64[n+1], E u32[m]). */
int psc_graph_download(psc_graph_t g, uint64_t* off, uint32_t* E);

/* SCC::scc (src/scc.hpp:277-476).  labels_out: host u64[n], the reference's
 * sequence<size_t> (final value = (label & 0xFFFFFFFF) - 1). */
int psc_scc(psc_graph_t g, const psc_params_t* p, uint64_t* labels_out);
/* Same, labels left in device memory d_labels (u64[n]) of the handle's device. */
int psc_scc_device(psc_graph_t g, const psc_params_t* p, uint64_t* d_labels);

/* REACH::reach (src/reach.hpp:208-243): dst_out host u8[n], 1 = reachable
 * from src.  dir 0 = forward (out-edges), 1 = backward (in-edges, as after
 * REACH::swap_graph).  Returns rounds via *rounds if non-NULL. */
int psc_reach(psc_graph_t g, uint32_t src, int dir, int local, uint32_t tau, uint8_t* dst_out,
              uint32_t* rounds);

/* BFS::bfs (src/bfs.hpp:200-238): dist_out host u32[n], hop distance from
 * src along out-edges, UINT32_MAX = unreached.  *rounds (if non-NULL)
 * receives the number of levels. */
int psc_bfs(psc_graph_t g, uint32_t src, uint32_t* dist_out, uint32_t* rounds);

/* LE_LIST::le_list (src/LeList.hpp:219-328) with the priority order supplied
 * by the caller: perm[i] = vertex of priority i (u32[n], a permutation of
 * [0, n); the reference draws it from parlay::random_permutation).  Distances
 * follow out-edges (the reference runs it on symmetric graphs).  Output:
 * triples (target, source vertex, distance), u32 each, sorted by (target,
 * priority of the source) — the reference's list and seq_le_list's.  out holds
 * cap triples (u32[3*cap]); *len receives the count.  If cap is too small,
 * returns PSC_ERR_CAPACITY with *len = the required count. */
int psc_lelist(psc_graph_t g, const uint32_t* perm, double beta, uint32_t* out, uint64_t cap,
               uint64_t* len);

/* Connectivity (src/Connectivity.h:37-119) on a symmetric graph (upload with
 * in_off = in_E = NULL, or any graph whose transpose equals itself): an LDD
 * with parameter beta (0.2 in the reference CLI) then hook-and-compress
 * union-find.  labels_out: host u32[n], each vertex's component root (a vertex
 * id of the component).  If forest_out is non-NULL it receives a spanning
 * forest as n_forest (u, v) edge pairs (u32[2*(n-1)] suffices; the reference's
 * spanning_forest option, Connectivity.h:99-117); forest_out and n_forest are
 * both NULL or both non-NULL. */
int psc_cc(psc_graph_t g, double beta, uint32_t* labels_out, uint32_t* forest_out,
           uint64_t* n_forest);

/* LDD::ldd (src/ldd.hpp:325-417) on a symmetric graph: label_out host u32[n]
 * = the centre (a vertex id) whose cluster holds each vertex; parent_out
 * (optional) host u32[n] = BFS-tree parent inside the cluster (parent[v] = v
 * for centres), the reference's spanning_tree output. */
int psc_ldd(psc_graph_t g, double beta, uint32_t* label_out, uint32_t* parent_out);
/* The centre schedule of the last psc_ldd / psc_cc call on g, one triple per
 * LDD round r = 1, 2, ...: (first candidate index i, candidates offered, new
 * centres).  Round r offers candidates hash32(1024 + i) % n for the next
 * floor(exp(r * beta)) indices i below 1024 (src/ldd.hpp:343-373); the
 * unlabelled ones become centres.  out holds cap triples (u32[3 * cap]);
 * *rounds receives the number of rounds (PSC_ERR_CAPACITY if above cap). */
int psc_ldd_rounds(psc_graph_t g, uint32_t* out, uint32_t cap, uint32_t* rounds);

/* Batches of independent graphs.  No counterpart in the reference, which
 * solves one graph per call (src/scc.cpp:57-67).
 *
 * A batch is one uploaded graph that is the disjoint union of num_graphs
 * graphs: graph k owns the vertex ids [vbase[k], vbase[k+1]) and all its edges
 * (and transpose edges) stay inside that range.  psc_batch_set attaches the
 * graph-offset table vbase (host u64[num_graphs+1], vbase[0] = 0,
 * vbase[num_graphs] = n, nondecreasing) to the handle and checks every edge
 * against it on the device: PSC_ERR_INVALID if one crosses two graphs. */
int psc_batch_set(psc_graph_t g, const uint64_t* vbase, uint32_t num_graphs);
uint32_t psc_batch_num_graphs(psc_graph_t g);
/* SCC of every graph of the batch in one lockstep solve.  labels_out: host
 * u64[n]; labels_out[vbase[k] + i] is vertex i's label in graph k, identical
 * to psc_scc on graph k alone with the same parameters and with p->seed
 * replaced by seeds[k] (seeds: host u64[num_graphs], or NULL for p->seed). */
int psc_scc_batch(psc_graph_t g, const psc_params_t* p, const uint64_t* seeds, uint64_t* labels_out);
int psc_scc_batch_device(psc_graph_t g, const psc_params_t* p, const uint64_t* seeds,
                         uint64_t* d_labels);
/* Connectivity of every graph of a batch of symmetric graphs: labels_out host
 * u32[n], each vertex's component root as a vertex id local to its graph (the
 * same partition as psc_cc on each graph alone). */
int psc_cc_batch(psc_graph_t g, double beta, uint32_t* labels_out);

/* Autotuner of the SCC parameters on this graph (or batch, with per-graph
 * seeds as psc_scc_batch; seeds is ignored for a plain graph).  No
 * counterpart in the reference.  Coordinate descent from *p over tau
 * {32, 64, 128, 256, 512}, pull_div {5, 10, 20, 40, 80}, block
 * {128, 256, 512} and beta {1.5, 2, 3, 4}; each candidate solve is timed
 * `reps` times (0: 2) and must be 2 % faster to be kept.  *p receives the
 * best parameters.  tau, pull_div and block never change the labels; beta
 * changes label values, never the partition. */
typedef struct {
  double start_ms;  /* solve time with the starting parameters */
  double best_ms;   /* solve time with the returned parameters */
  uint32_t trials;  /* parameter settings timed */
} psc_tune_report_t;
int psc_tune_scc(psc_graph_t g, const uint64_t* seeds, uint32_t reps, psc_params_t* p,
                 psc_tune_report_t* report);

/* Request server: SCC and connectivity solves of independent graphs served
 * with continuous batching under a device-memory budget.  No counterpart in
 * the reference.
 *
 * Submitted requests queue in arrival order.  Each of 2 * `workers` threads
 * (one CUDA stream per batch) takes, whenever it is free, the queued requests of the
 * kind at the head of the queue while their estimated device footprint fits
 * hbm_budget minus what running batches hold (at most max_batch requests
 * and max_batch_edges edges), packs them into one batch on the device, solves
 * it with the batched path and copies each member's labels to its caller.
 * At most `workers` batches solve at a time; the other threads' batches copy
 * their inputs meanwhile and wait for a solve slot, so the host link stays
 * busy while every slot solves.  Batches copy their inputs to the device one
 * after another in the order they were taken, so each reaches the device at
 * full link speed and solves while later batches copy.  Requests arriving while
 * batches run are admitted as workers and budget free up; their work overlaps
 * the running batches.  A request larger than the whole budget is refused at
 * submission (PSC_ERR_TOO_LARGE).  Results do not depend on the mix: SCC
 * labels equal psc_scc on the graph alone with p->seed = the request's seed,
 * connectivity labels give psc_cc's partition (roots local to the graph). */
typedef struct psc_server_s* psc_server_t;
#define PSC_REQ_SCC 0 /* directed CSR; labels_out u64[n] as psc_scc */
#define PSC_REQ_CC 1  /* symmetric CSR; labels_out u32[n] as psc_cc */
typedef struct {
  uint64_t hbm_budget;  /* device bytes admitted batches may hold (120 GiB) */
  uint32_t workers;     /* batches solving at a time (4); twice as many in flight */
  uint32_t max_batch;   /* requests per batch (4096) */
  double cc_beta;       /* LDD beta of connectivity requests (0.2) */
  psc_params_t scc;     /* SCC parameters; the seed comes with each request */
  uint64_t max_batch_edges; /* edges per batch (2^28; a larger request goes
                             * alone; 0 = no cap) */
} psc_server_config_t;
typedef struct {
  uint64_t submitted, completed, failed, rejected, batches;
  uint64_t peak_bytes;    /* largest admitted footprint at one time */
  uint64_t max_running;   /* most batches in flight at one time */
  uint64_t queued, bytes_in_use;
  uint64_t kernel_launches; /* kernels launched by completed batches */
  double busy_ms;         /* sum of batch wall times over workers */
} psc_server_stats_t;
typedef struct {
  int32_t status;       /* PSC_OK or the batch's error */
  uint32_t batch_size;  /* requests solved together with this one */
  double queue_ms;      /* submission to the start of its batch */
  double latency_ms;    /* submission to its labels in host memory */
} psc_request_info_t;
void psc_server_config_default(psc_server_config_t* cfg);
/* cfg NULL: the defaults.  The server uses the calling thread's device. */
int psc_server_create(const psc_server_config_t* cfg, psc_server_t* out);
/* off u64[n+1], E u32[m] (and for SCC optionally the transpose in_off /
 * in_E, as struct Graph carries it; built on the device when NULL) and
 * labels_out stay owned by the caller and must stay valid until
 * psc_server_wait returns for the request's id; off and in_off are host
 * memory.  Checks: at submission, off[0] = 0 and off[n] = m (in_off the
 * same); on the device, before its batch is solved, every offset of the
 * request no larger than the next and every target below n (the checks of
 * psc_graph_upload).  A malformed request fails alone: psc_server_wait
 * returns PSC_ERR_INVALID for it, and the other requests of its batch are
 * solved without it. */
int psc_server_submit(psc_server_t s, int kind, const uint64_t* off, const uint32_t* E,
                      const uint64_t* in_off, const uint32_t* in_E, uint64_t n, uint64_t m,
                      uint64_t seed, void* labels_out, uint64_t* id_out);
/* Blocks until the request is done, fills info (may be NULL), forgets the id
 * and returns the request's status. */
int psc_server_wait(psc_server_t s, uint64_t id, psc_request_info_t* info);
/* Blocks until nothing is queued or running. */
int psc_server_drain(psc_server_t s);
int psc_server_stats(psc_server_t s, psc_server_stats_t* out);
/* Serves what is still queued, then stops the workers and frees the server;
 * call it after the last psc_server_wait. */
int psc_server_destroy(psc_server_t s);

/* psc_reach without any memory allocation.  No counterpart in the reference.
 *
 * For callers that may not allocate device memory themselves: engines that
 * own the GPU's memory budget and hand out every buffer through their own
 * allocator, and latency-critical code that cannot afford the device-wide
 * synchronisation cudaMalloc / cudaFree may imply.  The caller passes device
 * pointers to the graph (d_in_off / d_in_E may be NULL for a symmetric graph)
 * and to the output d_dst (u8[n], 1 = reachable from src; dir 0 = forward,
 * 1 = backward), and the stream to run on (NULL = the legacy default stream).
 * The call allocates nothing: it uses no psc_graph_t, no cudaMalloc/cudaFree
 * and no allocating library routine.  Its scratch (visited and frontier
 * bitmaps, two frontier queues, the heavy list and the round counters) is one
 * file-scope __device__ array sized for PSC_NOALLOC_MAX_VERTICES vertices,
 * about 34 MB, which every GPU that loads the library holds until the
 * process exits.  Larger graphs are rejected with PSC_ERR_TOO_LARGE before
 * any device work.  The arrays are checked on the device before any kernel
 * indexes by them, as psc_graph_upload checks its input (offsets from 0 to m,
 * never decreasing; targets below n): PSC_ERR_INVALID otherwise.
 *
 * The first call on a device looks up that array's device address
 * (cudaGetSymbolAddress) with the device current; make that first call before
 * any stream capture.  All calls share the one array, which keeps the previous
 * call's contents (each call clears what must start at zero): calls that
 * overlap on the GPU — on different streams or from different host threads —
 * race and give wrong results.  Host-synchronous like psc_reach; *rounds (if
 * non-NULL) receives the number of frontier rounds. */
#define PSC_NOALLOC_MAX_VERTICES (1u << 21)
int psc_reach_noalloc(const uint64_t* d_off, const uint32_t* d_E, const uint64_t* d_in_off,
                      const uint32_t* d_in_E, uint64_t n, uint64_t m, uint32_t src, int dir,
                      uint8_t* d_dst, void* stream, uint32_t* rounds);

/* Per-call statistics of the last psc_scc / psc_reach / psc_cc / psc_lelist
 * on this handle. */
typedef struct {
  double total_ms;          /* device time of the call (CUDA events) */
  uint64_t reach_rounds;    /* first-pivot forward + backward rounds */
  uint64_t batches;         /* prefix-doubling batches run */
  uint64_t subrounds;       /* multi-search sub-rounds, both directions */
  uint64_t table_grows;     /* label-table rehashes */
  uint64_t kernel_launches; /* kernels launched by the call */
  /* SCC phase times in ms (the breakdown of src/scc.hpp:94-114):
   * [0] init/trim, [1] first round, [2] multi-search, [3] table resizing */
  double phase_ms[4];
} psc_stats_t;
int psc_last_stats(psc_graph_t g, psc_stats_t* out);

/* Profiling of kernel families (off by default).  When on, every launch of
 * family k is bracketed by CUDA events on the handle's stream and its
 * algorithmic byte count is accumulated.  psc_profile_get returns, for family
 * index k < psc_profile_count(), its name, launches, total ms and bytes. */
int psc_set_profiling(psc_graph_t g, int on);
int psc_profile_count(void);
int psc_profile_get(psc_graph_t g, int k, const char** name, uint64_t* launches, double* ms,
                    double* bytes);
int psc_profile_reset(psc_graph_t g);

/* Memory and timing plumbing for callers without a CUDA runtime of their own
 * (ctypes, FFI).  No reference counterpart.
 *   psc_host_alloc / psc_host_free     page-locked host memory (fast H2D/D2H)
 *   psc_device_alloc / psc_device_free device memory on the current device
 *   psc_copy(dst, src, bytes)          cudaMemcpy with the direction inferred
 *   psc_timer_start / psc_timer_stop   CUDA events on the handle's stream;
 *                                      stop waits and returns elapsed ms */
int psc_host_alloc(size_t bytes, void** ptr);
int psc_host_free(void* ptr);
int psc_device_alloc(size_t bytes, void** ptr);
int psc_device_free(void* ptr);
int psc_copy(void* dst, const void* src, size_t bytes);
int psc_timer_start(psc_graph_t g);
int psc_timer_stop(psc_graph_t g, double* ms);

/* Selects the CUDA device that later psc_graph_upload* calls on this thread
 * bind to (cudaSetDevice of the library's runtime). */
int psc_set_device(int device);

/* Number of visible CUDA devices (0 when there is none or the driver is
 * unusable).  No reference counterpart; lets callers probe before uploading. */
int psc_device_count(void);

const char* psc_strerror(int status);
const char* psc_version(void);

#ifdef __cplusplus
}
#endif
#endif

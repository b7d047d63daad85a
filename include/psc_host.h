/*
 * psc_host.h — host-side graph construction for the GB300 strong-connectivity
 * library: seeded synthetic generators, CSR/transpose construction,
 * symmetrisation and the GBBS binary graph format.  CPU only (C++17/OpenMP,
 * libpsc_host.so); no CUDA dependency.
 *
 * Reference interfaces replaced:
 *   psc_hgraph_read_bin / write_bin  <- read_binary, src/graph.hpp:120-185
 *   psc_hgraph_read_adj              <- read_pbbs, src/graph.hpp:73-118
 *   psc_hgraph_read_large            <- read_large_graph, src/graph.hpp:279-315
 *   psc_hgraph_build_transpose       <- make_directed, src/graph.hpp:222-245
 *   psc_hgraph_symmetrize            <- make_symmetric, src/graph.hpp:187-220
 *   psc_random_permutation           <- parlay::random_permutation as used by
 *                                       src/LeList.hpp:67 (own Feistel bijection)
 * The generators have no reference counterpart: the reference reads real
 * graphs from disk; these produce the seeded synthetic inputs that stand in
 * for them.
 *
 * Ownership: every psc_hgraph_t is owned by the caller and released with
 * psc_hgraph_free.  Functions returning a handle return NULL on failure and
 * set a message readable through psc_host_last_error().
 */
#ifndef PSC_HOST_H
#define PSC_HOST_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct psc_hgraph_s* psc_hgraph_t;

/* Directed R-MAT: n = 2^log2n vertices, `draws` edge draws with quadrant
 * probabilities (a, b, c, 1-a-b-c) per level, counter-based SplitMix64
 * stream keyed by `seed`; self-loops dropped, duplicates removed. */
psc_hgraph_t psc_hgraph_rmat(uint32_t log2n, uint64_t draws, double a, double b, double c,
                             uint64_t seed);

/* Directed 2-D kNN: npts points uniform in [0,1)^2 (seeded), edge i -> j for
 * each of the k nearest neighbours j != i (ties broken by smaller id). */
psc_hgraph_t psc_hgraph_knn(uint64_t npts, uint32_t k, uint64_t seed);

/* Directed 2-D grid rows x cols: each lattice edge oriented by a fair coin
 * and kept in both directions with probability p_bidir. */
psc_hgraph_t psc_hgraph_grid(uint32_t rows, uint32_t cols, double p_bidir, uint64_t seed);

/* CSR from an edge list (src[i] -> dst[i]); drop_self removes self-loops,
 * duplicates are always removed; adjacency lists sorted by target. */
psc_hgraph_t psc_hgraph_from_edges(uint64_t n, uint64_t m, const uint32_t* src,
                                   const uint32_t* dst, int drop_self);

/* Copy of a caller CSR (offsets u64[n+1], targets u32[m]). */
psc_hgraph_t psc_hgraph_from_csr(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E);

/* GBBS binary format: u64 n, u64 m, u64 sizes, u64 off[n+1], u32 E[m]. */
psc_hgraph_t psc_hgraph_read_bin(const char* path);
int psc_hgraph_write_bin(psc_hgraph_t g, const char* path);
/* PBBS text format "AdjacencyGraph n m off[0..n) E[0..m)" (read_pbbs,
 * src/graph.hpp:73-118). */
psc_hgraph_t psc_hgraph_read_adj(const char* path);
/* Two CSRs back to back (forward then transpose), as read_large_graph. */
psc_hgraph_t psc_hgraph_read_large(const char* path);

/* Builds in_off/in_E (in-lists sorted by source). Returns 0 on success. */
int psc_hgraph_build_transpose(psc_hgraph_t g);
/* New symmetric graph: both directions, deduplicated, no self-loops; its
 * transpose is itself (in_* alias the forward arrays). */
psc_hgraph_t psc_hgraph_symmetrize(psc_hgraph_t g);

uint64_t psc_hgraph_n(psc_hgraph_t g);
uint64_t psc_hgraph_m(psc_hgraph_t g);
const uint64_t* psc_hgraph_off(psc_hgraph_t g);
const uint32_t* psc_hgraph_E(psc_hgraph_t g);
const uint64_t* psc_hgraph_in_off(psc_hgraph_t g); /* NULL until built */
const uint32_t* psc_hgraph_in_E(psc_hgraph_t g);
void psc_hgraph_free(psc_hgraph_t g);

/* Packs count graphs into one disjoint union for psc_batch_set: graph k's
 * vertex i becomes vertex vbase_out[k] + i (vbase_out: u64[count+1]).  The
 * transpose of every member is built if missing and packed too; the union is
 * symmetric when every member is.  The members stay owned by the caller. */
psc_hgraph_t psc_hgraph_pack(const psc_hgraph_t* graphs, uint32_t count, uint64_t* vbase_out);

/* Seeded batch workload.  Member k uses seed seed0 + k and a size exponent u
 * uniform in [log2_min, log2_max): even k is an R-MAT graph with
 * 2^round(u) vertices, 16 * 2^round(u) draws and (a,b,c) = (0.57,0.19,0.19);
 * odd k is a 2D kNN graph (k = 5) of floor(2^u) points.  spec returns
 * kind 0 (R-MAT, size = log2 n) or 1 (kNN, size = points); 0 on success. */
int psc_batch_member_spec(uint32_t k, uint64_t seed0, double log2_min, double log2_max,
                          uint32_t* kind, uint64_t* size);
psc_hgraph_t psc_hgraph_batch_member(uint32_t k, uint64_t seed0, double log2_min, double log2_max);
/* Members 0..count-1 generated in parallel and packed (as psc_hgraph_pack). */
psc_hgraph_t psc_hgraph_batch(uint32_t count, uint64_t seed0, double log2_min, double log2_max,
                              uint64_t* vbase_out);

/* out[i] = Feistel bijection of i on [0, n) keyed by seed. */
void psc_random_permutation(uint64_t n, uint64_t seed, uint32_t* out);

const char* psc_host_last_error(void);

#ifdef __cplusplus
}
#endif
#endif

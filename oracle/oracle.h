/*
 * CPU oracle for the parallel strong-connectivity path — TEST INFRASTRUCTURE.
 *
 * Plain-C (C11 + OpenMP) restatement of the reference algorithms of
 * ucrparlay/Parallel-Strong-Connectivity.  Each function cites the reference
 * file:line it follows.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference arm may load this library, and only as the checker
 * or the timed CPU baseline; the product library never calls it.
 *
 * Parity status: pinned to the reference's own code.  The reference's headers
 * compile unmodified against this project's ParlayLib-API stand-in
 * (oracle/ref_shim/, oracle/ref.mk -> oracle/_ref/), whose hashes and
 * permutations are the ones used here; tests/golden/ref_vectors.npz holds
 * what that build computes (raw SCC labels, reach sets, transpose,
 * symmetrisation, connectivity partitions, BFS distances, LE-lists) and
 * tests/test_ref_pin.py holds this oracle to it bit for bit.  Partition-level
 * fixtures from scipy (tests/golden/graphs.npz) stay as an independent check.
 *
 * Graph layout everywhere: CSR offsets u64[n+1], targets u32[m] and the
 * transpose (in_off, in_E), as struct Graph in src/graph.hpp:35-43.
 */
#ifndef PSC_ORACLE_H
#define PSC_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Transpose CSR (src/graph.hpp:222-245 make_directed): in-lists sorted by
 * source id. */
void orc_transpose(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E,
                   uint64_t* in_off, uint32_t* in_E);

/* P = NON_ZEROS permuted by the Feistel bijection with `seed`
 * (src/scc.hpp:295-303).  Returns |P|; also returns |ZEROS| via n_zeros. */
uint64_t orc_pivot_order(uint64_t n, const uint64_t* off, const uint64_t* in_off,
                         uint64_t seed, uint32_t* P, uint64_t* n_zeros);

/* One-source reachability, sequential BFS (src/reach.hpp:57-74 reach_seq). */
void orc_reach_seq(uint64_t n, const uint64_t* off, const uint32_t* E, uint32_t src,
                   uint8_t* dst);

/* Parallel direction-optimising reach with VGC (src/reach.hpp:86-243). */
int orc_reach(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E,
              const uint64_t* in_off, const uint32_t* in_E, uint32_t src, uint8_t* dst,
              int local, uint32_t tau, int nthreads);

/* Parallel SCC (src/scc.hpp:277-476).  labels: u64[n] as sequence<size_t>.
 * Returns 0 on success.  Raw labels are those of the reference given the
 * same pivot order P. */
int orc_scc(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E,
            const uint64_t* in_off, const uint32_t* in_E, double beta, uint32_t tau,
            int local_reach, int local_scc, uint64_t seed, uint64_t* labels, int nthreads);

/* Iterative Tarjan (baselines/tarjan_scc/tarjan_scc.hpp:39-76); labels in
 * 1..#SCC in order of completion, as the recursive reference assigns them. */
uint32_t orc_tarjan(uint64_t n, const uint64_t* off, const uint32_t* E, uint32_t* scc);

/* Canonicalise any partition to "min vertex id of the class". */
void orc_canon_u64(uint64_t n, const uint64_t* labels, uint32_t* out);
void orc_canon_u32(uint64_t n, const uint32_t* labels, uint32_t* out);

/* Sequential BFS distances (src/bfs.hpp:59-76 bfs_seq); UINT32_MAX = unreached. */
void orc_bfs_seq(uint64_t n, const uint64_t* off, const uint32_t* E, uint32_t src,
                 uint32_t* dist);

/* Connectivity = LDD + union-find (src/Connectivity.h:37-119, src/ldd.hpp:325-417,
 * src/union_find_rules.h).  Symmetric graph.  labels u32[n] (union-find roots). */
int orc_cc(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E, double beta,
           uint32_t* labels, int nthreads);

/* LE-lists.  perm = centers (priority order -> vertex).  Output triples
 * (target, source vertex, dist) sorted by (target, priority); *len entries.
 * orc_lelist_seq follows src/LeList.hpp:76-115; orc_lelist_par follows
 * src/LeList.hpp:127-328.  out must hold `cap` triples; returns 0, or -1 if
 * cap is too small (then *len holds the needed size). */
int orc_lelist_seq(uint64_t n, const uint64_t* off, const uint32_t* E, const uint32_t* perm,
                   uint32_t* out, uint64_t cap, uint64_t* len);
int orc_lelist_par(uint64_t n, const uint64_t* off, const uint32_t* E, const uint32_t* perm,
                   double beta, uint32_t* out, uint64_t cap, uint64_t* len, int nthreads);

/* The permutation function itself, exported so tests can compare the GPU
 * library's implementation with this one. */
uint64_t orc_perm_at(uint64_t i, uint64_t k, uint64_t seed);
uint32_t orc_hash32_at(uint32_t x);
uint64_t orc_hash64_at(uint64_t x);

#ifdef __cplusplus
}
#endif
#endif

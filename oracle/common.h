/*
 * Shared definitions for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a CPU restatement of the
 * reference algorithms (ucrparlay/Parallel-Strong-Connectivity, src/).  It is
 * linked only by the test suite, by __graft_entry__.smoke() as the checker and
 * by bench.py's CPU-baseline / reference arm.  The product (libpsc_cuda.so)
 * never calls it.
 *
 * The hash functions and the pivot permutation below are this project's own
 * published constructions.  The reference takes them from ParlayLib
 * (parlay::hash32 / hash64 / random_shuffle, via src/utilities.h:108-118 and
 * src/scc.hpp:303), but that submodule is empty in the reference checkout, so
 * their exact constants are unknown.  The GPU library implements the same
 * specification independently (csrc/common.cuh); the tests check the two agree.
 */
#ifndef PSC_ORACLE_COMMON_H
#define PSC_ORACLE_COMMON_H

#include <stddef.h>
#include <stdint.h>

#define ORC_TOP_BIT ((uint64_t)1 << 32)          /* src/scc.hpp:22 */
#define ORC_VAL_MASK ((uint64_t)0xFFFFFFFFu)     /* src/scc.hpp:23 */
#define ORC_NMAX ((uint32_t)0xFFFFFFFFu)         /* UINT_N_MAX, src/utilities.h:26 */

/* lowbias32 (C. Wellons, "hash-prospector", public domain): a 32-bit
 * integer mixer used wherever the reference calls parlay::hash32. */
static inline uint32_t orc_hash32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

/* SplitMix64 finaliser (S. Vigna, public domain): used wherever the
 * reference calls parlay::hash64. */
static inline uint64_t orc_hash64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

/* Keyed pseudo-random bijection on [0, k): a 4-round balanced Feistel network
 * over the smallest even-bit power-of-two domain D >= k (so D < 4k), with
 * cycle walking back into [0, k).  Round r uses key
 *   K_r = (uint32_t)(hash64(seed ^ (0x9E3779B97F4A7C15 * (r + 1))) >> 32)
 * and round function F(R) = hash32(R ^ K_r) & half_mask.
 * P[i] = NON_ZEROS[orc_perm(i)] replaces parlay::random_shuffle
 * (src/scc.hpp:303), and perm[i] = orc_perm(i) over [0, n) replaces
 * parlay::random_permutation (src/LeList.hpp:67). */
static inline uint64_t orc_perm(uint64_t i, uint64_t k, uint64_t seed) {
  if (k <= 1) return 0;
  unsigned bits = 0;
  while (((uint64_t)1 << bits) < k) bits++;
  unsigned half = (bits + 1) / 2;
  uint64_t hmask = ((uint64_t)1 << half) - 1;
  uint32_t key[4];
  for (int r = 0; r < 4; r++)
    key[r] = (uint32_t)(orc_hash64(seed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(r + 1))) >> 32);
  uint64_t x = i;
  do {
    uint64_t L = x >> half, R = x & hmask;
    for (int r = 0; r < 4; r++) {
      uint64_t F = (uint64_t)orc_hash32((uint32_t)R ^ key[r]) & hmask;
      uint64_t nL = R;
      R = L ^ F;
      L = nL;
    }
    x = (L << half) | R;
  } while (x >= k);
  return x;
}

/* GCC atomics standing in for the reference's CAS helpers
 * (src/utilities.h:36-63, write_max :94-101). */
static inline int orc_cas8(uint8_t* p, uint8_t o, uint8_t n) {
  return __atomic_compare_exchange_n(p, &o, n, 0, __ATOMIC_ACQ_REL, __ATOMIC_RELAXED);
}
static inline int orc_cas32(uint32_t* p, uint32_t o, uint32_t n) {
  return __atomic_compare_exchange_n(p, &o, n, 0, __ATOMIC_ACQ_REL, __ATOMIC_RELAXED);
}
static inline int orc_cas64(uint64_t* p, uint64_t o, uint64_t n) {
  return __atomic_compare_exchange_n(p, &o, n, 0, __ATOMIC_ACQ_REL, __ATOMIC_RELAXED);
}
static inline uint64_t orc_load64(const uint64_t* p) { return __atomic_load_n(p, __ATOMIC_RELAXED); }
static inline uint32_t orc_load32(const uint32_t* p) { return __atomic_load_n(p, __ATOMIC_RELAXED); }
static inline uint8_t orc_load8(const uint8_t* p) { return __atomic_load_n(p, __ATOMIC_RELAXED); }

static inline void orc_write_max64(uint64_t* p, uint64_t v) {
  uint64_t c = orc_load64(p);
  while (c < v && !orc_cas64(p, c, v)) c = orc_load64(p);
}

/* Growable per-thread vector of u32 used as an exact frontier container in
 * place of the reference's hashbag (src/hash_bag.h); only the set of
 * vertices it holds matters. */
typedef struct {
  uint32_t* a;
  size_t n, cap;
} orc_vec;

void orc_vec_push(orc_vec* v, uint32_t x);
/* Concatenate nt per-thread vectors into out (returns total), clearing them. */
size_t orc_vec_gather(orc_vec* vs, int nt, uint32_t* out);
void orc_vec_free(orc_vec* vs, int nt);

#endif

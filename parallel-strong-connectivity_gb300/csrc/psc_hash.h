// Integer hashing, counter-based random numbers and the keyed pseudo-random
// permutation used by the library, host and device.
//
// The reference draws these from ParlayLib (parlay::hash32 / hash64 and
// random_shuffle / random_permutation; src/utilities.h:108-118,
// src/scc.hpp:303, src/LeList.hpp:67), whose sources are not available, so the
// library fixes its own published constructions:
//   hash32  — lowbias32 (C. Wellons, hash-prospector)
//   hash64  — SplitMix64 finaliser (S. Vigna)
//   rng     — SplitMix64 output for state hash64(seed) + (i+1)*golden
//   perm    — 4-round balanced Feistel network on the smallest even-bit
//             power-of-two domain >= k, with cycle walking into [0, k)
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define PSC_HD __host__ __device__ __forceinline__
#else
#define PSC_HD inline
#endif

namespace psc {

PSC_HD uint32_t hash32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

PSC_HD uint64_t hash64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ull;

// i-th 64-bit output of a SplitMix64 stream keyed by seed.
PSC_HD uint64_t rng64(uint64_t seed, uint64_t i) { return hash64(hash64(seed) + (i + 1) * kGolden); }

// Uniform double in [0, 1) from the top 53 bits.
PSC_HD double rng_unit(uint64_t seed, uint64_t i) {
  return (double)(rng64(seed, i) >> 11) * (1.0 / 9007199254740992.0);
}

struct FeistelKey {
  uint32_t half;
  uint64_t hmask;
  uint64_t k;
  uint32_t key[4];
};

PSC_HD FeistelKey feistel_key(uint64_t k, uint64_t seed) {
  FeistelKey f;
  uint32_t bits = 0;
  while (bits < 64 && ((uint64_t)1 << bits) < k) bits++;
  f.half = (bits + 1) / 2;
  f.hmask = ((uint64_t)1 << f.half) - 1;
  f.k = k;
  for (int r = 0; r < 4; r++) f.key[r] = (uint32_t)(hash64(seed ^ (kGolden * (uint64_t)(r + 1))) >> 32);
  return f;
}

// One pass of the 4-round network over the power-of-two domain.
PSC_HD uint64_t feistel_net(const FeistelKey& f, uint64_t x) {
  uint64_t L = x >> f.half, R = x & f.hmask;
  for (int r = 0; r < 4; r++) {
    uint64_t F = (uint64_t)hash32((uint32_t)R ^ f.key[r]) & f.hmask;
    uint64_t nL = R;
    R = L ^ F;
    L = nL;
  }
  return (L << f.half) | R;
}

// Bijection on [0, k): the network repeated until the value falls in [0, k).
PSC_HD uint64_t feistel(const FeistelKey& f, uint64_t i) {
  if (f.k <= 1) return 0;
  uint64_t x = i;
  do {
    x = feistel_net(f, x);
  } while (x >= f.k);
  return x;
}

}  // namespace psc

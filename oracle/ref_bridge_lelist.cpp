// C entry points over the reference's own LE-list code (src/LeList.hpp,
// src/resizable_set.hpp, src/bfs.hpp), compiled unmodified against the
// ParlayLib-API stand-in in oracle/ref_shim/.  Built by oracle/ref.mk into
// oracle/_ref/libref_lelist.so.
//
// TEST INFRASTRUCTURE ONLY (tests and the fixture generator); the product
// never loads it.
#include "LeList.hpp"

#include "ref_bridge_common.hpp"

extern "C" {

// LE_LIST::le_list(beta) (src/LeList.hpp:219-328), or seq_le_list (:76-115)
// when sequential != 0, under the caller's permutation perm (what
// parlay::random_permutation returns in the constructor, :67).  Writes up to
// cap (target, source, distance) triples to out; returns the list's length
// (which may exceed cap: call again with a larger buffer).
int64_t ref_lelist(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E,
                   const uint32_t* perm, double beta, int sequential, uint32_t* out, uint64_t cap) {
  if (n == 0) return 0;
  Graph g = ref_graph(n, m, off, E, off, E);
  parlay::shim_perm() = perm;
  LE_LIST le(g);
  parlay::shim_perm() = nullptr;
  if (sequential)
    le.seq_le_list();
  else
    le.le_list(beta);
  uint64_t len = le.list_offset;
  for (uint64_t i = 0; i < len && i < cap; i++) {
    out[3 * i] = get<0>(le.list[i]);
    out[3 * i + 1] = get<1>(le.list[i]);
    out[3 * i + 2] = get<2>(le.list[i]);
  }
  return (int64_t)len;
}

}  // extern "C"

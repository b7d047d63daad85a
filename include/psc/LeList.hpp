// psc/LeList.hpp — drop-in for the reference's src/LeList.hpp (class
// LE_LIST, src/LeList.hpp:35-74), running on a GB300.
//
//   LE_LIST(Graph&)            fixes the priority order (centers) and uploads
//   void le_list(double beta)  LeList.hpp:219-328
//   void seq_le_list()         the sequential definition, LeList.hpp:76-115
//   sequence<tuple<NodeId, NodeId, NodeId>> list   (target, source, dist)
//   size_t list_offset (entries in list), num_round
// The priority order is the library's seeded permutation (`le_seed`, default
// 4) in place of parlay::random_permutation.  seq_le_list runs the same device
// computation with one priority per batch — the sequential definition's order
// — so `le_list` vs `seq_le_list` compares one-source batches against
// prefix-doubling batches.  Link with -lpsc_cuda -lpsc_host.
#pragma once
#include <tuple>

#include "device_graph.hpp"

inline uint64_t le_seed = 4;

class LE_LIST {
 private:
  Graph& G;
  psc_graph_t h = nullptr;
  psc::sequence<NodeId> centers;

  void run(double beta) {
    uint64_t cap = list.size();
    psc::sequence<NodeId> flat(3 * (cap ? cap : 1));
    uint64_t len = 0;
    int st = psc_lelist(h, centers.data(), beta, flat.data(), cap, &len);
    if (st == PSC_ERR_CAPACITY) {
      cap = len;
      flat = psc::sequence<NodeId>(3 * cap);
      st = psc_lelist(h, centers.data(), beta, flat.data(), cap, &len);
    }
    psc_detail::check(st, "psc_lelist");
    if (list.size() < len) list = psc::sequence<std::tuple<NodeId, NodeId, NodeId>>(len);
    for (uint64_t i = 0; i < len; i++) list[i] = {flat[3 * i], flat[3 * i + 1], flat[3 * i + 2]};
    list_offset = len;
    psc_stats_t s;
    psc_last_stats(h, &s);
    num_round = s.batches;
  }

 public:
  size_t list_offset = 0;
  size_t num_round = 0;
  psc::sequence<std::tuple<NodeId, NodeId, NodeId>> list;
  LE_LIST() = delete;
  explicit LE_LIST(Graph& _G) : G(_G) {
    centers = psc::sequence<NodeId>(G.n);
    psc_random_permutation(G.n, le_seed, centers.data());
    h = psc_detail::upload(G);
  }
  LE_LIST(const LE_LIST&) = delete;
  LE_LIST& operator=(const LE_LIST&) = delete;
  ~LE_LIST() { psc_graph_free(h); }

  void le_list(double beta) { run(beta); }
  void seq_le_list() { run(1.0); }
};

// psc/scc.hpp — drop-in for the reference's src/scc.hpp, running on a GB300.
//
//   class SCC { SCC(Graph&); void scc(sequence<size_t>& labels, double beta,
//               bool local_reach, bool local_scc); timer_reset();
//               breakdown_report(int); size_t front_thresh, num_round; }
//                                                   src/scc.hpp:38-115
//   size_t tau            (global, src/reach.hpp:19)   — VGC budget
//   size_t _min_bag_size_ (global, src/scc.hpp:24)     — accepted, unused
// As in the reference, set the globals before constructing SCC.  The
// constructor uploads the graph (CSR + transpose) to the current device once;
// scc() runs SCC::scc there and writes the reference's labels
// ((label & 0xFFFFFFFF) - 1, src/scc.hpp:475-476).  The pivot order comes from
// the library's seeded permutation (`scc_seed`, default 1) in place of
// parlay::random_shuffle.  Link with -lpsc_cuda -lpsc_host.
#pragma once
#include <cstdint>
#include <iostream>

#include "device_graph.hpp"
#include "graph.hpp"
#include "sequence.hpp"

inline size_t tau = 512;
inline size_t _min_bag_size_ = 1 << 10;
inline uint64_t scc_seed = 1;

class SCC {
 private:
  Graph& graph;
  psc_graph_t h = nullptr;
  double t_init = 0, t_first = 0, t_multi = 0, t_resize = 0;

 public:
  size_t front_thresh = 0;
  size_t num_round = 0;
  SCC() = delete;
  explicit SCC(Graph& G) : graph(G) { h = psc_detail::upload(graph); }
  SCC(const SCC&) = delete;
  SCC& operator=(const SCC&) = delete;
  ~SCC() { psc_graph_free(h); }

  void scc(psc::sequence<size_t>& labels, double beta, bool local1, bool local2) {
    if (labels.size() < graph.n) labels = psc::sequence<size_t>(graph.n);
    psc_params_t p;
    psc_params_default(&p);
    p.beta = beta;
    p.tau = (uint32_t)tau;
    p.lambda = (uint32_t)_min_bag_size_;
    p.local_reach = local1;
    p.local_scc = local2;
    p.seed = scc_seed;
    static_assert(sizeof(size_t) == sizeof(uint64_t), "labels are u64");
    psc_detail::check(psc_scc(h, &p, reinterpret_cast<uint64_t*>(labels.data())), "psc_scc");
    psc_stats_t st;
    psc_last_stats(h, &st);
    num_round = st.batches;
    t_init += st.phase_ms[0] / 1e3;
    t_first += st.phase_ms[1] / 1e3;
    t_multi += st.phase_ms[2] / 1e3;
    t_resize += st.phase_ms[3] / 1e3;
  }

  void timer_reset() { t_init = t_first = t_multi = t_resize = 0; }

  // Same lines as src/scc.hpp:106-114 (seconds).
  void breakdown_report(int repeat) {
    std::cout << "average init_time " << t_init / repeat << std::endl;
    std::cout << "average first_round_time " << t_first / repeat << std::endl;
    std::cout << "average multi_search time " << t_multi / repeat << std::endl;
    std::cout << "average hash table resize time " << t_resize / repeat << std::endl;
  }
};

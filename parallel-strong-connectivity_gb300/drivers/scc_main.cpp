// `scc` command-line driver: the flags and output lines of the reference's
// src/scc.cpp:31-72 (so scripts that parse "average cost" keep working), over
// the drop-in headers include/psc/scc.hpp.  Extra flag: -seed (pivot order).
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>

#include "cli_common.hpp"
#include "psc/graph.hpp"
#include "psc/scc.hpp"

namespace {

// src/scc.cpp:13-29
void SCC_status(const psc::sequence<size_t>& label, size_t n) {
  psc::sequence<NodeId> flag(n + 1, 0);
  const NodeId MASK = UINT_N_MAX >> 1;
  for (size_t i = 0; i < n; i++) flag[label[i] & MASK]++;
  size_t n_scc = 0;
  NodeId largest = 0;
  for (size_t i = 0; i <= n; i++) {
    if (flag[i]) n_scc++;
    if (flag[i] > largest) largest = flag[i];
  }
  std::cout << "n_scc = " << n_scc << std::endl;
  std::cout << "Largest StronglyConnectedComponents has " << largest << std::endl;
}

}  // namespace

int main(int argc, char** argv) {
  CommandLine P{argc, argv};
  if (argc < 2) {
    std::cout << "usage: ./scc fileName" << std::endl;
    return 0;
  }
  char* fileName = argv[1];
  double beta = P.getOptionDouble("-beta", 1.5);
  std::cout << "--beta " << beta << "--" << std::endl;
  Graph graph = P.getOption("-large") ? read_large_graph(fileName) : read_graph(fileName);
  bool local_reach = P.getOption("-local_reach");
  bool local_scc = P.getOption("-local_scc");
  _min_bag_size_ = P.getOptionInt("-lambda", 1 << 10);
  tau = P.getOptionInt("-tau", 512);
  scc_seed = (uint64_t)P.getOptionInt("-seed", 1);
  std::cout << "tau " << tau << std::endl;
  std::cout << "input graph: " << fileName << std::endl;
  std::cout << "number of vertices: " << graph.n << ", number of edges: " << graph.m << std::endl;
  std::cout << "enable VGC1: " << local_reach << ", enable VGC_multi: " << local_scc << std::endl;

  psc::sequence<size_t> label(graph.n);
  int repeat = (int)P.getOptionInt("-t", 10);
  SCC SCC_P(graph);
  SCC_P.scc(label, beta, local_reach, local_scc);
  SCC_P.timer_reset();
  double total = 0;
  for (int i = 0; i < repeat; i++) {
    double t = wall_seconds();
    SCC_P.scc(label, beta, local_reach, local_scc);
    double c = wall_seconds() - t;
    total += c;
    std::cout << "scc cost: " << c << std::endl;
  }
  std::cout << "average cost " << total / repeat << std::endl;
  SCC_P.breakdown_report(repeat);
  if (P.getOption("-status")) SCC_status(label, graph.n);
  if (P.getOption("-labels")) {
    const char* out = P.getOptionValue("-labels");
    FILE* f = out ? std::fopen(out, "wb") : nullptr;
    if (!f || std::fwrite(label.data(), sizeof(size_t), graph.n, f) != graph.n) {
      std::cerr << "Error: cannot write labels" << std::endl;
      return 1;
    }
    std::fclose(f);
  }
  return 0;
}

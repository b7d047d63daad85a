// `Connectivity` command-line driver: flags and output lines of the
// reference's src/Connectivity.cpp:11-37, over include/psc/Connectivity.h.
// Extra flag: -labels <file> writes the u32 component roots.
#include <cstdio>
#include <iostream>

#include "cli_common.hpp"
#include "psc/Connectivity.h"
#include "psc/graph.hpp"

int main(int argc, char** argv) {
  CommandLine P{argc, argv};
  if (argc < 2) {
    std::cout << "usage: ./Connectivity filename" << std::endl;
    return 0;
  }
  char* filename = argv[1];
  Graph G = P.getOption("-large") ? read_large_sym_graph(filename)
                                  : read_graph(filename, !P.getOption("-nmmap"));
  std::cout << "#vertices: " << G.n << " #edges: " << G.m << '\n';
  int repeat = (int)P.getOptionInt("-t", 10);
  double beta = P.getOptionDouble("-beta", 0.2);
  auto res = Connectivity(G, beta);
  double total = 0;
  for (int i = 0; i < repeat; i++) {
    double t = wall_seconds();
    res = Connectivity(G, beta);
    double c = wall_seconds() - t;
    total += c;
    std::cout << "Connectivity time: " << c << std::endl;
  }
  std::cout << "average_time: " << total / repeat << std::endl;
  if (const char* out = P.getOptionValue("-labels")) {
    const auto& label = std::get<0>(res);
    FILE* f = std::fopen(out, "wb");
    if (!f || std::fwrite(label.data(), sizeof(NodeId), G.n, f) != G.n) {
      std::cerr << "Error: cannot write labels" << std::endl;
      return 1;
    }
    std::fclose(f);
  }
  return 0;
}

// `LeList` command-line driver: flags and output lines of the reference's
// src/LeList.cpp:8-98 (-beta, -t, -seq, -check, -large, -nmmap) over
// include/psc/LeList.hpp.  Extra flag: -list <file> writes the triples.
#include <cstdio>
#include <iostream>

#include "cli_common.hpp"
#include "psc/LeList.hpp"
#include "psc/graph.hpp"

int main(int argc, char** argv) {
  CommandLine P{argc, argv};
  if (argc < 2) {
    std::cout << "usage: ./LeList fileName" << std::endl;
    return 0;
  }
  char* filename = argv[1];
  Graph G = P.getOption("-large") ? read_large_sym_graph(filename)
                                  : read_graph(filename, !P.getOption("-nmmap"));
  std::cout << "Graph: " << filename << std::endl;
  std::cout << "#vertices: " << G.n << " #edges: " << G.m << '\n';
  double beta = P.getOptionDouble("-beta", 1.5);
  LE_LIST LE_LIST_P(G);
  int repeat = (int)P.getOptionInt("-t", 3);
  if (P.getOption("-seq")) {
    LE_LIST_P.seq_le_list();
    double total = 0;
    for (int i = 0; i < repeat; i++) {
      double t = wall_seconds();
      LE_LIST_P.seq_le_list();
      double c = wall_seconds() - t;
      total += c;
      std::cout << "sequential LE-List cost: " << c << std::endl;
      std::cout << "LE-List size " << LE_LIST_P.list_offset << std::endl;
    }
    std::cout << "average sequential LE-List cost: " << total / repeat << std::endl;
  } else {
    LE_LIST_P.le_list(beta);
    double total = 0;
    for (int i = 0; i < repeat; i++) {
      double t = wall_seconds();
      LE_LIST_P.le_list(beta);
      double c = wall_seconds() - t;
      total += c;
      std::cout << "LE-List cost: " << c << std::endl;
    }
    std::cout << "# LE-List size: " << LE_LIST_P.list_offset << std::endl;
    std::cout << "average cost: " << total / repeat << std::endl;
  }
  if (const char* out = P.getOptionValue("-list")) {
    FILE* f = std::fopen(out, "wb");
    for (size_t i = 0; f && i < LE_LIST_P.list_offset; i++) {
      const uint32_t t[3] = {std::get<0>(LE_LIST_P.list[i]), std::get<1>(LE_LIST_P.list[i]),
                             std::get<2>(LE_LIST_P.list[i])};
      std::fwrite(t, 4, 3, f);
    }
    if (f) std::fclose(f);
  }
  if (P.getOption("-check")) {
    // src/LeList.cpp:59-97: the sequential definition against the batches
    LE_LIST_P.seq_le_list();
    const size_t seq_size = LE_LIST_P.list_offset;
    psc::sequence<std::tuple<NodeId, NodeId, NodeId>> seq(seq_size);
    for (size_t i = 0; i < seq_size; i++) seq[i] = LE_LIST_P.list[i];
    LE_LIST_P.le_list(beta);
    bool same = seq_size == LE_LIST_P.list_offset;
    for (size_t i = 0; same && i < seq_size; i++) same = seq[i] == LE_LIST_P.list[i];
    if (same) {
      std::cout << "pass check" << std::endl;
    } else {
      std::cout << "LeList_seq size " << seq_size << std::endl;
      std::cout << "LeList size " << LE_LIST_P.list_offset << std::endl;
    }
  }
  return 0;
}

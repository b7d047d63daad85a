// psc/graph.hpp — the reference's graph type and readers (src/graph.hpp),
// restated over libpsc_host.so.  Link with -lpsc_host.
//
//   struct Graph                    src/graph.hpp:35-43
//   read_graph(file, mmap, sym)     src/graph.hpp:248-277  (.bin and .adj;
//                                   a file name containing "sym" is symmetric)
//   read_large_graph(file)          src/graph.hpp:279-315  (CSR + transpose)
//   read_large_sym_graph(file)      src/graph.hpp:317-345
//   make_directed / make_symmetric  src/graph.hpp:222-245 / 187-220
// Errors print to stderr and abort(), as the reference does.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../psc_host.h"
#include "sequence.hpp"

using NodeId = uint32_t;  // src/utilities.h:17-27 (NodeId u32, EdgeId u64)
using EdgeId = uint64_t;
constexpr NodeId UINT_N_MAX = 0xFFFFFFFFu;

struct Graph {
  size_t n = 0;
  size_t m = 0;
  bool symmetric = false;
  psc::sequence<EdgeId> offset;
  psc::sequence<NodeId> E;
  psc::sequence<EdgeId> in_offset;
  psc::sequence<NodeId> in_E;
};

namespace psc_detail {

inline void die(const std::string& what) {
  std::fprintf(stderr, "Error: %s\n", what.c_str());
  std::abort();
}

inline void adopt_forward(Graph& g, psc_hgraph_t h) {
  g.n = psc_hgraph_n(h);
  g.m = psc_hgraph_m(h);
  g.offset = psc::sequence<EdgeId>::uninitialized(g.n + 1);
  g.E = psc::sequence<NodeId>::uninitialized(g.m);
  std::memcpy(g.offset.data(), psc_hgraph_off(h), (g.n + 1) * sizeof(EdgeId));
  if (g.m) std::memcpy(g.E.data(), psc_hgraph_E(h), g.m * sizeof(NodeId));
}

inline void adopt_transpose(Graph& g, psc_hgraph_t h) {
  g.in_offset = psc::sequence<EdgeId>::uninitialized(g.n + 1);
  g.in_E = psc::sequence<NodeId>::uninitialized(g.m);
  std::memcpy(g.in_offset.data(), psc_hgraph_in_off(h), (g.n + 1) * sizeof(EdgeId));
  if (g.m) std::memcpy(g.in_E.data(), psc_hgraph_in_E(h), g.m * sizeof(NodeId));
}

inline psc_hgraph_t handle_of(const Graph& g) {
  psc_hgraph_t h = psc_hgraph_from_csr(g.n, g.m, g.offset.data(), g.E.data());
  if (!h) die(psc_host_last_error());
  return h;
}

}  // namespace psc_detail

inline void make_directed(Graph& g) {
  psc_hgraph_t h = psc_detail::handle_of(g);
  if (psc_hgraph_build_transpose(h) != 0) psc_detail::die(psc_host_last_error());
  psc_detail::adopt_transpose(g, h);
  psc_hgraph_free(h);
}

inline void make_symmetric(Graph& g) {
  psc_hgraph_t h = psc_detail::handle_of(g);
  psc_hgraph_t s = psc_hgraph_symmetrize(h);
  psc_hgraph_free(h);
  if (!s) psc_detail::die(psc_host_last_error());
  psc_detail::adopt_forward(g, s);
  psc_hgraph_free(s);
  g.in_offset = g.offset;
  g.in_E = g.E;
}

inline Graph read_graph(const char* filename, bool enable_mmap = true, bool symmetric = false) {
  (void)enable_mmap;
  std::string f(filename);
  size_t dot = f.find_last_of('.');
  if (dot == std::string::npos) psc_detail::die("No graph extension provided");
  std::string ext = f.substr(dot + 1);
  psc_hgraph_t h = nullptr;
  if (ext == "bin")
    h = psc_hgraph_read_bin(filename);
  else if (ext == "adj")
    h = psc_hgraph_read_adj(filename);
  else
    psc_detail::die("Invalid graph extension");
  if (!h) psc_detail::die(psc_host_last_error());
  Graph g;
  psc_detail::adopt_forward(g, h);
  psc_hgraph_free(h);
  if (f.find("sym") != std::string::npos) {
    g.in_offset = g.offset;
    g.in_E = g.E;
    g.symmetric = true;
  } else if (symmetric) {
    make_symmetric(g);
    g.symmetric = true;
  } else {
    g.symmetric = false;
    make_directed(g);
  }
  return g;
}

inline Graph read_large_graph(const char* filename) {
  psc_hgraph_t h = psc_hgraph_read_large(filename);
  if (!h) psc_detail::die(psc_host_last_error());
  Graph g;
  psc_detail::adopt_forward(g, h);
  psc_detail::adopt_transpose(g, h);
  psc_hgraph_free(h);
  return g;
}

inline Graph read_large_sym_graph(const char* filename) {
  std::printf("read large sym graph %s\n", filename);
  psc_hgraph_t h = psc_hgraph_read_bin(filename);
  if (!h) psc_detail::die(psc_host_last_error());
  Graph g;
  psc_detail::adopt_forward(g, h);
  psc_hgraph_free(h);
  g.symmetric = true;
  g.in_offset = g.offset;
  g.in_E = g.E;
  return g;
}

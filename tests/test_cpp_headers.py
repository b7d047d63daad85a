"""The C++ drop-in headers (include/psc/*.hpp) compile as the reference's
interfaces are used, and the CLI driver links (CPU only)."""
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PROGRAM = r'''
#include "psc/graph.hpp"
#include "psc/scc.hpp"
#include "psc/reach.hpp"
#include "psc/bfs.hpp"
#include "psc/ldd.hpp"
#include "psc/Connectivity.h"
#include "psc/LeList.hpp"
int main(int argc, char** argv) {
  if (argc < 2) return 0;
  Graph graph = read_graph(argv[1]);
  tau = 64;
  _min_bag_size_ = 1024;
  SCC SCC_P(graph);
  parlay::sequence<size_t> label(graph.n);
  SCC_P.scc(label, 1.5, true, true);
  SCC_P.timer_reset();
  SCC_P.breakdown_report(1);
  REACH R(graph);
  parlay::sequence<bool> d1(graph.n), d2(graph.n);
  R.reach(0, d1, true);
  R.swap_graph();
  R.reach(0, d2, true);
  R.swap_graph();
  BFS B(graph);
  parlay::sequence<NodeId> dist(graph.n);
  B.bfs(0, dist);
  auto cc = Connectivity(graph, 0.2);
  auto cf = Connectivity(graph, 0.2, [](NodeId, NodeId) { return true; }, true);
  LDD L(graph);
  auto lp = L.ldd(0.2, true);
  LE_LIST LE(graph);
  LE.le_list(1.5);
  LE.seq_le_list();
  (void)cc; (void)cf; (void)lp;
  return (int)(label.size() != graph.n);
}
'''


def test_headers_compile(tmp_path):
    src = tmp_path / "use.cpp"
    src.write_text(PROGRAM)
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only",
                        f"-I{ROOT / 'include'}", str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_driver_built():
    from psc import _drivers

    exes = _drivers.build_drivers()
    for e in exes:
        assert e.exists()
        out = subprocess.run([str(e)], capture_output=True, text=True)
        assert f"usage: ./{e.name}" in out.stdout

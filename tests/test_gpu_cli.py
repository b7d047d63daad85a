"""The drop-in C++ interfaces on the GPU: the `scc` CLI driver (flags and
output lines of src/scc.cpp) and a program using SCC / REACH / swap_graph
through include/psc/*.hpp, compared with the oracle."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import psc
import pyoracle as O

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module", autouse=True)
def _dev(cuda_device):
    return cuda_device


def test_scc_driver(tmp_path):
    from psc import _drivers

    exe = _drivers.build_drivers()[0]
    g = psc.HostGraph.knn(30000, 5, seed=8)
    f = tmp_path / "knn.bin"
    g.write_bin(f)
    lab_file = tmp_path / "labels.u64"
    r = subprocess.run([str(exe), str(f), "-local_reach", "-local_scc", "-t", "2", "-status",
                        "-seed", "4", "-labels", str(lab_file)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    out = r.stdout
    assert re.search(r"^average cost [0-9.e-]+$", out, re.M)
    assert len(re.findall(r"^scc cost: ", out, re.M)) == 2
    for key in ("average init_time", "average first_round_time", "average multi_search time",
                "average hash table resize time"):
        assert key in out
    labels = np.fromfile(lab_file, dtype=np.uint64)
    ref = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=4)
    assert np.array_equal(labels, ref)
    tar, k = O.tarjan(g.n, g.off, g.E)
    assert f"n_scc = {k}" in out
    largest = np.bincount(O.canon(tar)).max()
    assert f"Largest StronglyConnectedComponents has {largest}" in out


def test_dropin_headers_program(tmp_path):
    prog = tmp_path / "prog.cpp"
    prog.write_text(r'''
#include <cstdio>
#include "psc/graph.hpp"
#include "psc/scc.hpp"
#include "psc/reach.hpp"
int main(int argc, char** argv) {
  Graph graph = read_graph(argv[1]);
  tau = 32;
  scc_seed = 6;
  SCC S(graph);
  parlay::sequence<size_t> label(graph.n);
  S.scc(label, 1.5, true, true);
  REACH R(graph);
  parlay::sequence<bool> f(graph.n), b(graph.n);
  R.reach(3, f, true);
  R.swap_graph();
  R.reach(3, b, false);
  R.swap_graph();
  FILE* o = std::fopen(argv[2], "wb");
  std::fwrite(label.data(), 8, graph.n, o);
  std::fwrite(f.data(), 1, graph.n, o);
  std::fwrite(b.data(), 1, graph.n, o);
  std::fclose(o);
  return 0;
}
''')
    build = ROOT / "parallel-strong-connectivity_gb300" / "_build"
    exe = tmp_path / "prog"
    r = subprocess.run(["g++", "-O2", "-std=c++17", f"-I{ROOT / 'include'}", str(prog), "-o", str(exe),
                        f"-L{build}", "-lpsc_cuda", "-lpsc_host", f"-Wl,-rpath,{build}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    g = psc.HostGraph.rmat(12, 1 << 16, seed=3)
    f = tmp_path / "g.bin"
    g.write_bin(f)
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(f), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    raw = out.read_bytes()
    labels = np.frombuffer(raw[: 8 * g.n], np.uint64)
    fw = np.frombuffer(raw[8 * g.n: 9 * g.n], np.uint8)
    bw = np.frombuffer(raw[9 * g.n:], np.uint8)
    assert np.array_equal(labels, O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=6))
    assert np.array_equal(fw, O.reach_seq(g.n, g.off, g.E, 3))
    assert np.array_equal(bw, O.reach_seq(g.n, g.in_off, g.in_E, 3))


def test_connectivity_and_lelist_drivers(tmp_path):
    from psc import _drivers

    exes = {e.name: e for e in _drivers.build_drivers()}
    g = psc.HostGraph.knn(20000, 5, seed=21).symmetrize()
    f = tmp_path / "knn_sym.bin"  # "sym" in the name: read as symmetric
    g.write_bin(f)
    lab_file = tmp_path / "cc.u32"
    r = subprocess.run([str(exes["Connectivity"]), str(f), "-t", "2", "-labels", str(lab_file)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert re.search(r"^average_time: [0-9.e-]+$", r.stdout, re.M)
    assert len(re.findall(r"^Connectivity time: ", r.stdout, re.M)) == 2
    labels = np.fromfile(lab_file, dtype=np.uint32)
    assert np.array_equal(O.canon(labels), O.canon(O.cc(g.n, g.off, g.E)))

    small = psc.HostGraph.grid(30, 30, 0.3, seed=4).symmetrize()
    f2 = tmp_path / "grid_sym.bin"
    small.write_bin(f2)
    out = tmp_path / "le.u32"
    r = subprocess.run([str(exes["LeList"]), str(f2), "-t", "1", "-check", "-list", str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "pass check" in r.stdout
    assert re.search(r"^average cost: [0-9.e-]+$", r.stdout, re.M)
    got = np.fromfile(out, dtype=np.uint32).reshape(-1, 3)
    perm = psc.random_permutation(small.n, 4)  # le_seed default
    assert np.array_equal(got, O.lelist_seq(small.n, small.off, small.E, perm))

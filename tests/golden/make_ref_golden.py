"""Generates tests/golden/ref_vectors.npz — outputs of the reference's own code.

The reference ships no test vectors.  Its headers (src/scc.hpp, reach.hpp,
bfs.hpp, graph.hpp, Connectivity.h, ldd.hpp, LeList.hpp and
baselines/tarjan_scc/tarjan_scc.hpp) are compiled unmodified against this
project's ParlayLib-API stand-in by oracle/ref.mk (oracle/_ref/libref_*.so),
and this script records what they compute on seeded inputs:

  scc_s{seed}     raw SCC labels (SCC::scc, beta 1.5, tau 512, lambda 1024,
                  VGC on; pivot order = the stand-in's random_shuffle, i.e.
                  the library's Feistel bijection keyed by seed)
  scc_plain_s1    the same with VGC off (-local_reach / -local_scc unset)
  tarjan          canonical partition of TARJAN_SCC
  reach_f / _b    REACH::reach from vertex 0, forward and backward
  in              the transpose of make_directed (src/graph.hpp:222-245)
  sym             make_symmetric (src/graph.hpp:187-220)
  cc              canonical partition of Connectivity(G_sym, 0.2)
  bfs             BFS::bfs distances from vertex 0 on G_sym
  le              LE_LIST::le_list(1.5) on G_sym under psc.random_permutation(n, 4)

Each output is stored as its SHA-256 (`{case}/{key}#sha`, over the array's
little-endian bytes) and, for graphs of at most 1024 vertices, also in full.
Graph inputs: the cases of graphs.npz (stored CSR) and seeded generator
outputs (`{case}/input#sha` pins the generator).

Run (from the repository root, with the reference checkout present and the
package built):  python tests/golden/make_ref_golden.py
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "parallel-strong-connectivity_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "tests"))

FULL_MAX_N = 1024
SEEDS = (1, 7)
LE_SEED = 4

# Seeded generator cases: (name, kind, size, seed) as in tests/_cases.py.
GEN = [
    ("rmat10_s1", "rmat", 10, 1), ("rmat13_s2", "rmat", 13, 2), ("rmat16_s1", "rmat", 16, 1),
    ("knn5000_s2", "knn", 5000, 2), ("knn60000_s3", "knn", 60000, 3),
    ("grid64_s2", "grid", 64, 2), ("grid256_s5", "grid", 256, 5),
]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def canon(lab: np.ndarray) -> np.ndarray:
    _, first, inv = np.unique(lab, return_index=True, return_inverse=True)
    return first[inv].astype(np.uint32)


def graph_cases():
    """(name, HostGraph) of every case, golden CSR first."""
    import _cases
    import psc

    out = []
    for name, c in _cases.golden().items():
        out.append((name, _cases.host_graph(c)))
    for name, kind, size, seed in GEN:
        out.append((name, _cases.generated(kind, size, seed)))
    return out


def outputs(g) -> dict:
    import psc
    import pyref as R

    n = g.n
    res = {}
    for s in SEEDS:
        res[f"scc_s{s}"] = R.scc(n, g.off, g.E, g.in_off, g.in_E, seed=s)
    res["scc_plain_s1"] = R.scc(n, g.off, g.E, g.in_off, g.in_E, seed=1, local_reach=False,
                                local_scc=False)
    t, _ = R.tarjan(n, g.off, g.E)
    res["tarjan"] = canon(t)
    res["reach_f"] = R.reach(n, g.off, g.E, g.in_off, g.in_E, 0, forward=True)
    res["reach_b"] = R.reach(n, g.off, g.E, g.in_off, g.in_E, 0, forward=False)
    io, iE = R.make_directed(n, g.off, g.E)
    res["in_off"], res["in_E"] = io, iE
    so, sE = R.make_symmetric(n, g.off, g.E)
    res["sym_off"], res["sym_E"] = so, sE
    res["cc"] = canon(R.cc(n, so, sE))
    res["bfs"] = R.bfs(n, so, sE, 0)
    if n >= 2:
        # LE_LIST's constructor sizes its bag by ceil(log n) * n
        # (src/LeList.hpp:62), which is 0 for n = 1: the reference's own
        # code reads outside that bag there, so one-vertex graphs have no
        # LE-list vector.
        perm = psc.random_permutation(n, LE_SEED)
        res["le"] = R.lelist(n, so, sE, perm)
    return res


def main():
    import pyref

    if not pyref.build():
        raise SystemExit("the reference-code oracle could not be built (no reference checkout?)")
    data = {}
    names = []
    for name, g in graph_cases():
        names.append(name)
        data[f"{name}/n"] = np.array([g.n], np.uint64)
        data[f"{name}/input#sha"] = np.array(sha(g.off) + sha(g.E))
        for k, v in outputs(g).items():
            data[f"{name}/{k}#sha"] = np.array(sha(v))
            if g.n <= FULL_MAX_N:
                data[f"{name}/{k}"] = v
        print(f"{name}: n={g.n} m={g.m}", flush=True)
    data["names"] = np.array(names)
    np.savez_compressed(HERE / "ref_vectors.npz", **data)
    print(f"wrote {len(names)} cases to {HERE / 'ref_vectors.npz'}")


if __name__ == "__main__":
    main()

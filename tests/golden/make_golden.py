"""Generates tests/golden/graphs.npz — known-answer fixtures for the parity tests.

The reference repository ships no test vectors and cannot be built here (its
ParlayLib submodule is empty), so the expected answers come from independent
implementations run in this container:

  scc   canonical strong components   scipy.sparse.csgraph.connected_components
  cc    canonical weak components of the symmetrised graph (make_symmetric
        semantics, src/graph.hpp:187-220: both directions, dedup, no
        self-loops)                    scipy.sparse.csgraph.connected_components
  le    LE-lists of the symmetrised graph for a stored permutation, from the
        definition (src/LeList.hpp:76-115): for priorities in order, record
        (target, source vertex, dist) whenever dist is strictly below every
        earlier priority's distance; sorted by (target, priority)
  reach forward reachable set from vertex 0   (plain BFS, this file)
  bfs   BFS distances from vertex 0            (plain BFS, this file)

"Canonical" = every vertex labelled with the smallest vertex id of its class.
Graphs are stored as CSR (off u64, E u32), duplicates and self-loops kept where
a case has them.  Three cases also pin the seeded generators of libpsc_host.so
(gen_* keys): the stored CSR is what those generators must keep producing.

Run:  python tests/golden/make_golden.py   (needs the built libpsc_host.so)
"""
from __future__ import annotations

import sys
from collections import deque
from pathlib import Path

import numpy as np
import scipy.sparse as sp
import scipy.sparse.csgraph as cg

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "parallel-strong-connectivity_gb300"))


def canon(lab: np.ndarray) -> np.ndarray:
    _, first, inv = np.unique(lab, return_index=True, return_inverse=True)
    return first[inv].astype(np.uint32)


def csr_from_edges(n, src, dst):
    src = np.asarray(src, np.int64)
    dst = np.asarray(dst, np.int64)
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    off = np.zeros(n + 1, np.uint64)
    np.add.at(off, src + 1, 1)
    off = np.cumsum(off).astype(np.uint64)
    return off, dst.astype(np.uint32)


def adj(off, E, n):
    return [E[off[u]:off[u + 1]].tolist() for u in range(n)]


def symmetric_csr(n, off, E):
    src = np.repeat(np.arange(n), np.diff(off).astype(np.int64))
    s = np.concatenate([src, E.astype(np.int64)])
    d = np.concatenate([E.astype(np.int64), src])
    keep = s != d
    pairs = np.unique(np.stack([s[keep], d[keep]], 1), axis=0) if keep.any() else np.zeros((0, 2), np.int64)
    return csr_from_edges(n, pairs[:, 0], pairs[:, 1])


def components(n, off, E, conn):
    A = sp.csr_matrix((np.ones(len(E), np.int8), E.astype(np.int64), off.astype(np.int64)), shape=(n, n))
    _, lab = cg.connected_components(A, directed=True, connection=conn)
    return canon(lab)


def bfs(n, off, E, s):
    d = np.full(n, 0xFFFFFFFF, np.uint32)
    d[s] = 0
    q = deque([s])
    A = adj(off, E, n)
    while q:
        u = q.popleft()
        for w in A[u]:
            if d[w] == 0xFFFFFFFF:
                d[w] = d[u] + 1
                q.append(w)
    return d


def lelist(n, off, E, perm):
    best = np.full(n, np.iinfo(np.int64).max, np.int64)
    out = []
    for i in range(n):
        d = bfs(n, off, E, int(perm[i])).astype(np.int64)
        d[d == 0xFFFFFFFF] = np.iinfo(np.int64).max
        better = np.nonzero(d < best)[0]
        for v in better:
            out.append((int(v), i, int(d[v])))
        best = np.minimum(best, d)
    out.sort()
    return np.array([(t, int(perm[p]), dd) for (t, p, dd) in out], np.uint32).reshape(-1, 3)


def hand_cases():
    cases = {}
    cases["single"] = (1, [], [])
    cases["isolated5"] = (5, [], [])
    cases["selfloops_dups"] = (4, [0, 0, 0, 1, 1, 2, 2, 3, 3], [0, 1, 1, 2, 0, 2, 3, 3, 3])
    cases["cycle8"] = (8, list(range(8)), [(i + 1) % 8 for i in range(8)])
    cases["two_cycles_bridge"] = (8, [0, 1, 2, 3, 4, 5, 6, 7, 3], [1, 2, 3, 0, 5, 6, 7, 4, 4])
    cases["chain10"] = (10, list(range(9)), list(range(1, 10)))
    k6 = [(u, v) for u in range(6) for v in range(6) if u != v]
    cases["complete6"] = (6, [a for a, _ in k6], [b for _, b in k6])
    # hub: 0 -> all, all -> 0 for even ids, plus a tail
    s, d = [], []
    for v in range(1, 40):
        s.append(0); d.append(v)
        if v % 2 == 0:
            s.append(v); d.append(0)
    s += [39, 38]; d += [38, 37]
    cases["hub40"] = (40, s, d)
    # nested SCCs: a ring of 3-cycles
    s, d = [], []
    for c in range(10):
        b = 3 * c
        s += [b, b + 1, b + 2]; d += [b + 1, b + 2, b]
        s.append(b + 2); d.append((b + 3) % 30)
    cases["ring_of_triangles"] = (30, s, d)
    # random multigraph with self-loops and duplicates (kept)
    rng = np.random.default_rng(20240601)
    n = 200
    s = rng.integers(0, n, 900); d = rng.integers(0, n, 900)
    s = np.concatenate([s, s[:50], np.arange(10)]); d = np.concatenate([d, d[:50], np.arange(10)])
    cases["random_multi200"] = (n, s.tolist(), d.tolist())
    # sparse random with many trivial SCCs
    s = rng.integers(0, 500, 600); d = rng.integers(0, 500, 600)
    cases["sparse500"] = (500, s.tolist(), d.tolist())
    return cases


def main():
    import psc

    data = {}
    names = []
    cases = hand_cases()
    for name, (n, s, d) in cases.items():
        off, E = csr_from_edges(n, s, d)
        cases[name] = (n, off, E)
    gens = {
        "gen_rmat8": psc.HostGraph.rmat(8, 1 << 11, seed=11),
        "gen_knn300": psc.HostGraph.knn(300, 5, seed=12),
        "gen_grid12": psc.HostGraph.grid(12, 12, 0.3, seed=13),
    }
    for name, g in gens.items():
        cases[name] = (g.n, g.off.astype(np.uint64), g.E.astype(np.uint32))
    perm_rng = np.random.default_rng(4)
    for name, (n, off, E) in cases.items():
        names.append(name)
        data[f"{name}/n"] = np.array([n], np.uint64)
        data[f"{name}/off"] = off
        data[f"{name}/E"] = E
        data[f"{name}/scc"] = components(n, off, E, "strong")
        soff, sE = symmetric_csr(n, off, E)
        data[f"{name}/cc"] = components(n, soff, sE, "weak")
        data[f"{name}/reach0"] = (bfs(n, off, E, 0) != 0xFFFFFFFF).astype(np.uint8)
        data[f"{name}/bfs0"] = bfs(n, off, E, 0)
        if n <= 400:
            perm = perm_rng.permutation(n).astype(np.uint32)
            data[f"{name}/perm"] = perm
            data[f"{name}/le"] = lelist(n, soff, sE, perm)
    data["names"] = np.array(names)
    np.savez_compressed(HERE / "graphs.npz", **data)
    print(f"wrote {len(names)} cases to {HERE / 'graphs.npz'}")


if __name__ == "__main__":
    main()

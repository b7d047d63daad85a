"""GPU parity for BFS distances and LE-lists: exact equality with the oracle's
sequential definitions and the golden fixtures."""
import numpy as np
import pytest

import psc
import pyoracle as O
from _cases import GEN_CASES, generated, golden, golden_names, host_graph

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _dev(cuda_device):
    return cuda_device


@pytest.mark.parametrize("name", golden_names())
def test_bfs_golden(name):
    c = golden()[name]
    g = host_graph(c)
    with psc.DeviceGraph(g) as dg:
        assert np.array_equal(dg.bfs(0), c["bfs0"])


@pytest.mark.parametrize("kind,size,seed", GEN_CASES)
def test_bfs_generated(kind, size, seed):
    g = generated(kind, size, seed)
    rng = np.random.default_rng(seed + 7)
    with psc.DeviceGraph(g) as dg:
        for src in rng.integers(0, g.n, 3).tolist():
            assert np.array_equal(dg.bfs(src), O.bfs_seq(g.n, g.off, g.E, src))


@pytest.mark.parametrize("name", [n for n in golden_names() if "perm" in golden()[n]])
def test_lelist_golden(name):
    c = golden()[name]
    s = host_graph(c).symmetrize()
    with psc.DeviceGraph(s) as dg:
        assert np.array_equal(dg.lelist(c["perm"]), c["le"])


@pytest.mark.parametrize("kind,size,seed", [("rmat", 10, 3), ("rmat", 12, 5), ("grid", 40, 4),
                                            ("knn", 3000, 5), ("knn", 400, 9)])
def test_lelist_generated(kind, size, seed):
    s = generated(kind, size, seed).symmetrize()
    perm = psc.random_permutation(s.n, seed + 4)
    ref = O.lelist_seq(s.n, s.off, s.E, perm)
    with psc.DeviceGraph(s) as dg:
        for beta in (1.5, 1.1, 4.0):
            assert np.array_equal(dg.lelist(perm, beta), ref)


def hub_graph(n, sizes, seed):
    """Symmetric graph: hubs 0..len(sizes) with the given numbers of random
    neighbours over a sparse random backbone."""
    rng = np.random.default_rng(seed)
    src, dst = [], []
    for h, size in enumerate(sizes):
        src.append(np.full(size, h))
        dst.append(rng.choice(np.arange(len(sizes), n), size, replace=False))
    src.append(rng.integers(0, n, 2 * n))
    dst.append(rng.integers(0, n, 2 * n))
    return psc.HostGraph.from_edges(n, np.concatenate(src), np.concatenate(dst)).symmetrize()


@pytest.mark.parametrize("sizes,seed", [((6000, 3000, 1000, 300, 257), 17),
                                        ((40000,), 3), (tuple([400] * 64), 8)])
def test_lelist_heavy_pairs(sizes, seed):
    """Vertices with hundreds to tens of thousands of edges (expanded by the
    balanced heavy-pair kernel) reached by many priorities at several levels;
    one frontier may hold many heavy pairs of the same hub."""
    s = hub_graph(50_000, sizes, seed)
    perm = psc.random_permutation(s.n, seed)
    ref = O.lelist_seq(s.n, s.off, s.E, perm)
    with psc.DeviceGraph(s) as dg:
        for beta in (1.5, 4.0):
            assert np.array_equal(dg.lelist(perm, beta), ref)


def test_lelist_directed_matches_definition():
    """Distances follow out-edges: the device result equals seq_le_list's
    definition on a directed graph too."""
    g = generated("rmat", 9, 11)
    perm = psc.random_permutation(g.n, 2)
    with psc.DeviceGraph(g) as dg:
        assert np.array_equal(dg.lelist(perm), O.lelist_seq(g.n, g.off, g.E, perm))


def test_lelist_capacity_status():
    s = generated("grid", 20, 3).symmetrize()
    perm = psc.random_permutation(s.n, 1)
    lib = psc.cuda()
    import ctypes as C
    with psc.DeviceGraph(s) as dg:
        out = np.empty(3, np.uint32)
        ln = C.c_uint64()
        st = lib.psc_lelist(dg.h, perm.ctypes.data, 1.5, out.ctypes.data, 1, C.byref(ln))
        assert st == psc._lib.PSC_ERR_CAPACITY and ln.value > 1

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


def test_lelist_caller_buffer():
    """Triples written into a caller array (what bench.py passes, page-locked),
    equal to the allocating call; a too-small array is refused with
    PSC_ERR_CAPACITY."""
    s = generated("rmat", 12, 5).symmetrize()
    perm = psc.random_permutation(s.n, 9)
    with psc.DeviceGraph(s) as dg:
        ref = dg.lelist(perm)
        buf = np.full(3 * len(ref) + 7, 0xFFFFFFFF, np.uint32)
        got = dg.lelist(perm, out=buf)
        assert np.array_equal(got, ref)
        assert np.all(buf[3 * len(ref):] == 0xFFFFFFFF)
        with pytest.raises(psc.PscError):
            dg.lelist(perm, out=np.empty(3 * (len(ref) - 1), np.uint32))


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


def test_lelist_table_retry():
    """A batch whose level inserts far more pairs than the previous batch's
    inserts per edge predict: the pair table overflows its estimate, inserts
    give up after their probe limit, and the level runs again on a table
    sized for the worst case.  With beta = 2 the batches are [2^k - 1,
    2^(k+1) - 1): priority 0 is a hub, priorities 1..254 its leaves (the batch
    [127, 255) inserts nothing, so the next estimate is the floor), and the
    batch [255, 511) is a 256-vertex clique that inserts 65,280 pairs at its
    first level."""
    leaves, clique, extra = 254, 256, 3000
    n = 1 + leaves + clique + extra
    hub = 0
    lv = np.arange(1, 1 + leaves)
    cq = np.arange(1 + leaves, 1 + leaves + clique)
    a, b = np.meshgrid(cq, cq)
    keep = a != b
    rng = np.random.default_rng(21)
    ex = np.arange(1 + leaves + clique, n)
    # leaves touch only the hub; the clique is its own component
    src = np.concatenate([np.full(leaves, hub), a[keep], ex, rng.choice(ex, 2000)])
    dst = np.concatenate([lv, b[keep], rng.choice(ex, len(ex)), rng.choice(ex, 2000)])
    s = psc.HostGraph.from_edges(n, src, dst).symmetrize()
    perm = np.concatenate([[hub], lv, cq, rng.permutation(ex)]).astype(np.uint32)
    ref = O.lelist_seq(s.n, s.off, s.E, perm)
    with psc.DeviceGraph(s) as dg:
        assert np.array_equal(dg.lelist(perm, 2.0), ref)
        assert dg.stats().table_grows >= 1


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

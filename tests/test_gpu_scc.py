"""GPU parity: SCC, reachability and the device transpose through the C ABI,
compared bit-exactly with the CPU oracle and the golden fixtures."""
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
def test_scc_golden(name):
    c = golden()[name]
    g = host_graph(c)
    with psc.DeviceGraph(g) as dg:
        for seed in (1, 2):
            lab = dg.scc(psc.default_params(seed=seed))
            ref = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=seed)
            assert np.array_equal(lab, ref), "raw labels differ from the oracle"
            assert np.array_equal(O.canon(lab), c["scc"]), "partition differs from scipy"


@pytest.mark.parametrize("kind,size,seed", GEN_CASES)
def test_scc_generated(kind, size, seed):
    g = generated(kind, size, seed)
    with psc.DeviceGraph(g) as dg:
        lab = dg.scc(psc.default_params(seed=seed))
    ref = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=seed)
    assert np.array_equal(lab, ref)
    tar, _ = O.tarjan(g.n, g.off, g.E)
    assert np.array_equal(O.canon(lab), O.canon(tar))


@pytest.mark.parametrize("params", [
    dict(local_reach=0, local_scc=0),
    dict(tau=1),
    dict(tau=64),
    dict(beta=1.1),
    dict(beta=2.0),
    dict(beta=8.0),
    dict(pull_div=1),       # push almost always
    dict(pull_div=100000),  # pull almost always
])
def test_scc_params(params):
    g = generated("rmat", 14, 7)
    with psc.DeviceGraph(g) as dg:
        lab = dg.scc(psc.default_params(seed=3, **params))
    ref = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=3,
                beta=params.get("beta", 1.5), tau=params.get("tau", 512))
    assert np.array_equal(lab, ref)


def test_scc_repeated_calls_reuse_state():
    g = generated("knn", 20000, 4)
    ref = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=9)
    with psc.DeviceGraph(g) as dg:
        for _ in range(3):
            assert np.array_equal(dg.scc(psc.default_params(seed=9)), ref)
        st = dg.stats()
        assert st.total_ms > 0 and st.batches > 0


def test_scc_symmetric_upload():
    s = generated("grid", 64, 3).symmetrize()
    with psc.DeviceGraph(s) as dg:
        lab = dg.scc(psc.default_params(seed=1))
    ref = O.scc(s.n, s.off, s.E, s.off, s.E, seed=1)
    assert np.array_equal(lab, ref)


def test_scc_table_growth_path():
    """A batch of ~100 pivots on a long chain: every pivot reaches the rest of
    the chain inside one subproblem, so the (v, pivot) closure (~6*10^4 pairs)
    outgrows the first table many times over.  Labels must not change."""
    n = 1200
    g = psc.HostGraph.from_edges(n, np.arange(n - 1), np.arange(1, n))
    with psc.DeviceGraph(g) as dg:
        lab = dg.scc(psc.default_params(seed=2, beta=100.0))
        assert dg.stats().table_grows > 0
    ref = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=2, beta=100.0)
    assert np.array_equal(lab, ref)


@pytest.mark.parametrize("name", golden_names())
def test_reach_golden(name):
    c = golden()[name]
    g = host_graph(c)
    with psc.DeviceGraph(g) as dg:
        assert np.array_equal(dg.reach(0), c["reach0"])
        assert np.array_equal(dg.reach(0, backward=True), O.reach_seq(g.n, g.in_off, g.in_E, 0))


@pytest.mark.parametrize("kind,size,seed", GEN_CASES)
def test_reach_generated(kind, size, seed):
    g = generated(kind, size, seed)
    rng = np.random.default_rng(seed)
    with psc.DeviceGraph(g) as dg:
        for src in rng.integers(0, g.n, 4).tolist():
            assert np.array_equal(dg.reach(src), O.reach_seq(g.n, g.off, g.E, src))
            assert np.array_equal(dg.reach(src, backward=True),
                                  O.reach_seq(g.n, g.in_off, g.in_E, src))


@pytest.mark.parametrize("kind,size,seed", GEN_CASES)
def test_device_transpose(kind, size, seed):
    g = generated(kind, size, seed)
    with psc.DeviceGraph.directed(g.off, g.E) as dg:
        in_off, in_E = dg.transpose()
        assert np.array_equal(in_off, g.in_off)
        assert np.array_equal(in_E, g.in_E)
        lab = dg.scc(psc.default_params(seed=5))
    assert np.array_equal(lab, O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=5))


def test_device_transpose_heavy_lists():
    # a star: one in-list of 20000 entries (global-memory sort path)
    n = 20001
    src = np.arange(1, n, dtype=np.uint32)
    dst = np.zeros(n - 1, dtype=np.uint32)
    g = psc.HostGraph.from_edges(n, np.concatenate([src, dst]), np.concatenate([dst, src]))
    with psc.DeviceGraph.directed(g.off, g.E) as dg:
        in_off, in_E = dg.transpose()
    assert np.array_equal(in_off, g.in_off) and np.array_equal(in_E, g.in_E)


@pytest.mark.parametrize("n,m,seed", [(1, 0, 1), (7, 0, 2), (100, 900, 3), (300, 50, 4),
                                      ((1 << 17) + 3, 600000, 5), (1 << 20, 40000, 6)])
def test_device_transpose_sizes(n, m, seed):
    """Radix passes 1 to 3 (target ids up to 8, 9, 18, 20 bits), edgeless
    graphs and long runs of vertices without in-edges."""
    rng = np.random.default_rng(seed)
    src = rng.integers(0, n, m).astype(np.uint32)
    dst = (rng.integers(0, max(1, n // 7), m) * 7 % n).astype(np.uint32)  # sparse targets
    g = psc.HostGraph.from_edges(n, src, dst)
    with psc.DeviceGraph.directed(g.off, g.E) as dg:
        in_off, in_E = dg.transpose()
    assert np.array_equal(in_off, g.in_off) and np.array_equal(in_E, g.in_E)


def test_invalid_source_rejected():
    g = generated("rmat", 10, 1)
    with psc.DeviceGraph(g) as dg:
        with pytest.raises(psc.PscError):
            dg.reach(g.n)

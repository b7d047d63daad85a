"""GPU parity on adversarial shapes: a long cycle (thousands of rounds), a
long chain (every vertex its own SCC, large multi-search closures), a dense
complete digraph, hubs above the heavy-vertex threshold in both directions,
and a union of many small cycles with cross links.  Raw labels against the
oracle, partitions against Tarjan."""
import numpy as np
import pytest

import psc
import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _dev(cuda_device):
    return cuda_device


def check(g, seeds=(1, 2), **kw):
    tar, _ = O.tarjan(g.n, g.off, g.E)
    with psc.DeviceGraph(g) as dg:
        for seed in seeds:
            lab = dg.scc(psc.default_params(seed=seed, **kw))
            assert np.array_equal(lab, O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=seed,
                                             beta=kw.get("beta", 1.5), tau=kw.get("tau", 512)))
            assert np.array_equal(O.canon(lab), O.canon(tar))


def test_long_cycle():
    n = 200_000
    g = psc.HostGraph.from_edges(n, np.arange(n), (np.arange(n) + 1) % n)
    check(g, seeds=(1,))


def test_long_chain():
    n = 50_000
    g = psc.HostGraph.from_edges(n, np.arange(n - 1), np.arange(1, n))
    check(g, seeds=(3,))


def test_complete_digraph():
    k = 300
    src, dst = np.meshgrid(np.arange(k), np.arange(k), indexing="ij")
    g = psc.HostGraph.from_edges(k, src.ravel(), dst.ravel())
    check(g)


@pytest.mark.parametrize("local", [0, 1])
def test_heavy_hubs(local):
    """Two hubs of 30000 spokes each way (above the 8192 heavy threshold),
    joined by one edge, plus a few one-way spokes."""
    s = 30_000
    hub_a, hub_b = 0, s + 1
    a = np.arange(1, s + 1)
    b = np.arange(s + 2, 2 * s + 2)
    src = np.concatenate([np.full(s, hub_a), a, np.full(s, hub_b), b, [hub_a],
                          np.full(100, hub_b)])
    dst = np.concatenate([a, np.full(s, hub_a), b, np.full(s, hub_b), [hub_b],
                          np.arange(2 * s + 2, 2 * s + 102)])
    g = psc.HostGraph.from_edges(2 * s + 102, src, dst)
    check(g, local_reach=local, local_scc=local)


def test_cycles_with_cross_links():
    rng = np.random.default_rng(5)
    src, dst, n = [], [], 0
    for size in rng.integers(1, 60, 2000).tolist():
        src += list(range(n, n + size))
        dst += [n + (i + 1) % size for i in range(size)]
        n += size
    cross = rng.integers(0, n, (3000, 2))
    g = psc.HostGraph.from_edges(n, src + cross[:, 0].tolist(), dst + cross[:, 1].tolist())
    check(g, seeds=(1, 7), beta=2.0, tau=64)

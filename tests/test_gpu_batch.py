"""GPU parity of batched SCC and connectivity: every graph of a packed batch
gets exactly the labels of a solve of that graph alone (the oracle's raw SCC
labels with the graph's own seed, the plain device call, and the connectivity
partition)."""
import numpy as np
import pytest

import psc
import pyoracle as O
from _cases import golden, golden_names, host_graph

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _dev(cuda_device):
    return cuda_device


def members_of(u, vbase):
    """Split a packed union back into its member graphs (local ids)."""
    return [u.member(vbase, k) for k in range(len(vbase) - 1)]


def check_scc_batch(graphs, params, seeds=None, plain=False):
    u, vb = psc.HostGraph.pack(graphs)
    with psc.DeviceGraph(u) as dg:
        dg.set_batch(vb)
        lab = dg.scc_batch(params, seeds)
    for k, g in enumerate(graphs):
        got = lab[int(vb[k]):int(vb[k + 1])]
        seed = int(seeds[k]) if seeds is not None else params.seed
        ref = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, beta=params.beta, tau=params.tau,
                    local_reach=params.local_reach, local_scc=params.local_scc, seed=seed)
        assert np.array_equal(got, ref), f"graph {k}: raw labels differ from a solo solve"
        if plain:
            p1 = psc.default_params(beta=params.beta, tau=params.tau, seed=seed,
                                    local_reach=params.local_reach, local_scc=params.local_scc)
            with psc.DeviceGraph(g) as d1:
                assert np.array_equal(d1.scc(p1), got)
    return u, vb, lab


def test_batch_golden_members():
    graphs = [host_graph(golden()[n]) for n in golden_names()]
    seeds = np.arange(len(graphs), dtype=np.uint64) * 7 + 3
    _, _, lab = check_scc_batch(graphs, psc.default_params(), seeds, plain=True)
    vb = np.concatenate([[0], np.cumsum([g.n for g in graphs])])
    for k, n in enumerate(golden_names()):
        assert np.array_equal(O.canon(lab[vb[k]:vb[k + 1]]), golden()[n]["scc"])


@pytest.mark.parametrize("count,lo,hi", [(40, 4, 11), (16, 8, 14)])
def test_batch_workload_members(count, lo, hi):
    u, vb = psc.batch_workload(count, 1000, lo, hi)
    graphs = members_of(u, vb)
    for k in (0, 1, count - 1):
        m = psc.batch_member(k, 1000, lo, hi)
        assert m.n == graphs[k].n and np.array_equal(m.E, graphs[k].E)
    seeds = 1000 + np.arange(count, dtype=np.uint64)
    _, _, lab = check_scc_batch(graphs, psc.default_params(), seeds)
    for k, g in enumerate(graphs):
        tar, _ = O.tarjan(g.n, g.off, g.E)
        assert np.array_equal(O.canon(lab[vb[k]:vb[k + 1]]), O.canon(tar))


@pytest.mark.parametrize("params", [
    dict(local_reach=0, local_scc=0),
    dict(beta=1.1, tau=16),
    dict(beta=4.0),
    dict(pull_div=1),
    dict(pull_div=100000),
])
def test_batch_params(params):
    u, vb = psc.batch_workload(12, 77, 5, 12)
    check_scc_batch(members_of(u, vb), psc.default_params(seed=5, **params))


def test_batch_edge_cases():
    """Single vertices, edgeless and fully trimmed graphs, one cycle and a
    chain long enough to grow the label tables, mixed in one batch."""
    one = psc.HostGraph.from_edges(1, [], [])
    empty = psc.HostGraph.from_edges(5, [], [])
    star = psc.HostGraph.from_edges(6, [0, 0, 0, 0, 0], [1, 2, 3, 4, 5])
    cyc = psc.HostGraph.from_edges(7, list(range(7)), [(i + 1) % 7 for i in range(7)])
    n = 1200
    chain = psc.HostGraph.from_edges(n, list(range(n - 1)), list(range(1, n)))
    graphs = [one, empty, star, cyc, chain, one, cyc]
    check_scc_batch(graphs, psc.default_params(beta=100.0), plain=True)
    check_scc_batch(graphs, psc.default_params(), np.arange(7, dtype=np.uint64))
    check_scc_batch([one], psc.default_params())


def test_batch_single_graph_equals_plain():
    g = psc.HostGraph.rmat(13, 16 << 13, seed=4)
    check_scc_batch([g], psc.default_params(seed=9), plain=True)


def test_batch_set_rejects_crossing_edges():
    a = psc.HostGraph.from_edges(4, [0, 1, 2], [1, 2, 3])
    with psc.DeviceGraph(a) as dg:
        with pytest.raises(psc.PscError):
            dg.set_batch(np.array([0, 2, 4], np.uint64))  # edge 1 -> 2 crosses
        with pytest.raises(psc.PscError):
            dg.set_batch(np.array([0, 3], np.uint64))     # does not end at n
        with pytest.raises(psc.PscError):
            dg.set_batch(np.array([0, 3, 2, 4], np.uint64))  # decreasing
        dg.set_batch(np.array([0, 4], np.uint64))
        assert psc.cuda().psc_batch_num_graphs(dg.h) == 1


def test_batch_repeated_and_reset():
    u, vb = psc.batch_workload(10, 5, 6, 12)
    graphs = members_of(u, vb)
    with psc.DeviceGraph(u) as dg:
        dg.set_batch(vb)
        a = dg.scc_batch(psc.default_params(seed=2))
        b = dg.scc_batch(psc.default_params(seed=2))
        assert np.array_equal(a, b)
        # a coarser table: first half / second half
        h = len(graphs) // 2
        dg.set_batch(np.array([0, vb[h], vb[-1]], np.uint64))
        c = dg.scc_batch(psc.default_params(seed=2))
    for part, (v0, v1) in enumerate([(0, int(vb[h])), (int(vb[h]), int(vb[-1]))]):
        gp, _ = psc.HostGraph.pack(graphs[:h] if part == 0 else graphs[h:])
        ref = O.scc(gp.n, gp.off, gp.E, gp.in_off, gp.in_E, seed=2)
        assert np.array_equal(c[v0:v1], ref)


def test_cc_batch():
    u, vb = psc.batch_workload(14, 31, 5, 12)
    graphs = [g.symmetrize() for g in members_of(u, vb)]
    s, svb = psc.HostGraph.pack(graphs)
    assert s.symmetric and np.array_equal(svb, vb)
    with psc.DeviceGraph(s) as dg:
        dg.set_batch(svb)
        lab = dg.cc_batch()
    for k, g in enumerate(graphs):
        got = lab[int(vb[k]):int(vb[k + 1])]
        assert (got < g.n).all()
        assert np.array_equal(O.canon(got), O.canon(O.cc(g.n, g.off, g.E)))

"""GPU parity for Connectivity (LDD + union-find): the partition must equal
the oracle's, scipy's (golden) and, with a spanning forest, the forest must
span every component without a cycle."""
import numpy as np
import pytest

import psc
import pyoracle as O
from _cases import GEN_CASES, generated, golden, golden_names, host_graph

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _dev(cuda_device):
    return cuda_device


def check_forest(n, labels_canon, forest):
    """forest: (k, 2) edges.  Acyclic, inside components, k = n - #components."""
    parent = np.arange(n)

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    for u, v in forest.tolist():
        assert labels_canon[u] == labels_canon[v], "forest edge crosses components"
        ru, rv = find(u), find(v)
        assert ru != rv, "forest has a cycle"
        parent[ru] = rv
    ncomp = len(np.unique(labels_canon))
    assert len(forest) == n - ncomp


@pytest.mark.parametrize("name", golden_names())
def test_cc_golden(name):
    c = golden()[name]
    s = host_graph(c).symmetrize()
    with psc.DeviceGraph(s) as dg:
        lab = dg.cc()
        lab2, forest = dg.cc(forest=True)
    assert np.array_equal(O.canon(lab), c["cc"])
    assert np.array_equal(O.canon(lab2), c["cc"])
    check_forest(s.n, c["cc"], forest)


@pytest.mark.parametrize("kind,size,seed", GEN_CASES)
def test_cc_generated(kind, size, seed):
    s = generated(kind, size, seed).symmetrize()
    ref = O.canon(O.cc(s.n, s.off, s.E))
    with psc.DeviceGraph(s) as dg:
        for beta in (0.2, 1.0):
            assert np.array_equal(O.canon(dg.cc(beta)), ref)
        lab, forest = dg.cc(forest=True)
    assert np.array_equal(O.canon(lab), ref)
    check_forest(s.n, ref, forest)


def test_cc_caller_buffer():
    """Labels written into a caller array equal the allocating call's."""
    s = generated("rmat", 12, 5).symmetrize()
    with psc.DeviceGraph(s) as dg:
        ref = dg.cc()
        buf = np.zeros(s.n, np.uint32)
        assert dg.cc(out=buf) is buf
        assert np.array_equal(buf, ref)


def test_cc_many_components():
    # disjoint cycles of various sizes plus isolated vertices
    src, dst = [], []
    n = 0
    rng = np.random.default_rng(3)
    for size in rng.integers(1, 40, 300).tolist():
        for i in range(size):
            src.append(n + i)
            dst.append(n + (i + 1) % size)
        n += size
    g = psc.HostGraph.from_edges(n + 50, src, dst)
    s = g.symmetrize()
    with psc.DeviceGraph(s) as dg:
        lab, forest = dg.cc(forest=True)
    ref = O.canon(O.cc(s.n, s.off, s.E))
    assert np.array_equal(O.canon(lab), ref)
    check_forest(s.n, ref, forest)


@pytest.mark.parametrize("kind,size,seed", [("knn", 20000, 3), ("rmat", 14, 2), ("grid", 128, 1)])
def test_ldd_properties(kind, size, seed):
    """LDD (src/ldd.hpp:325-417): every vertex carries a centre that labels
    itself, BFS parents are neighbours in the same cluster, and clusters never
    cross components."""
    s = generated(kind, size, seed).symmetrize()
    with psc.DeviceGraph(s) as dg:
        lab, par = dg.ldd(0.2)
    n = s.n
    assert (lab < n).all()
    assert (lab[lab] == lab).all(), "centres label themselves"
    centres = lab == np.arange(n)
    assert (par[centres] == np.arange(n)[centres]).all()
    v = np.nonzero(~centres)[0]
    assert (lab[par[v]] == lab[v]).all(), "parent in the same cluster"
    for x in v[:2000].tolist():
        assert par[x] in s.E[s.off[x]:s.off[x + 1]], "parent is a neighbour"
    comp = O.canon(O.cc(n, s.off, s.E))
    assert (comp[lab] == comp).all(), "clusters inside components"


def ldd_schedule(beta, rounds):
    """The reference's centre windows (src/ldd.hpp:343-373): round r offers
    the next floor(exp(r * beta)) of the 1024 sampled candidates."""
    import math
    out, sampled = [], 0
    for r in range(1, rounds + 1):
        work = min(int(math.floor(math.exp(r * beta))), 1024 - sampled)
        out.append((sampled, work))
        sampled += work
    return out


@pytest.mark.parametrize("kind,size,seed", [("knn", 20000, 3), ("rmat", 14, 2), ("grid", 128, 1)])
@pytest.mark.parametrize("beta", [0.2, 0.5])
def test_ldd_centre_schedule(kind, size, seed, beta):
    """LDD's centres, round by round: the candidates each round offers are the
    reference's (hash32(1024 + i) % n in windows of floor(exp(r * beta))),
    the first candidate is always a centre, the new centres the trace counts
    are exactly the candidates that label themselves in the output, and every
    other vertex is labelled by a candidate centre or (unreached) by itself."""
    s = generated(kind, size, seed).symmetrize()
    n = s.n
    with psc.DeviceGraph(s) as dg:
        lab, _ = dg.ldd(beta)
        rows = dg.ldd_rounds()
    assert len(rows) >= 1
    assert [tuple(r) for r in rows[:, :2].tolist()] == ldd_schedule(beta, len(rows))
    assert rows[:, 1].sum() == 1024
    cand = np.array([O.lib().orc_hash32_at(1024 + i) % n for i in range(1024)], np.uint32)
    assert lab[cand[0]] == cand[0], "the first candidate is a centre"
    cset = np.unique(cand)
    centres = cset[lab[cset] == cset]
    assert rows[:, 2].sum() == len(centres)
    assert (rows[:, 2] <= rows[:, 1]).all()
    other = lab != np.arange(n)
    assert np.isin(lab[other], centres).all(), "clusters belong to candidate centres"

"""Parity at the largest single-GPU sizes.

R-MAT n = 2^26 with 2^30 draws (0.57, 0.19, 0.19, 0.05), seed 3, deduplicated
(m = 1.06e9): SCC raw labels bit-exact with the oracle (src/scc.hpp:277-476),
the device transpose equal to the host's (src/graph.hpp:222-245); on its
symmetrisation (m = 2.1e9) the connectivity partition equal to the oracle's
(src/Connectivity.h:37-119) and the LE-lists for permutation seed 4 identical
to the oracle's parallel LE-lists (src/LeList.hpp:219-328).

The 4096-graph batch (vertex counts log-uniform in [2^8, 2^18), even members
R-MAT with 16 draws per vertex, odd members 2-D kNN k = 5, member k seeded
1000 + k; n = 1.56e8, m = 1.56e9): every member's labels from the batched
solve equal the oracle's solo solve of that member, on a stratified sample of
64 members."""
import os

import numpy as np
import pytest

import psc
import pyoracle as O

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module", autouse=True)
def _dev(cuda_device):
    return cuda_device


@pytest.fixture(scope="module")
def rmat26():
    return psc.HostGraph.rmat(26, 1 << 30, seed=3)


@pytest.fixture(scope="module")
def rmat26_sym(rmat26):
    return rmat26.symmetrize()


def test_scc_rmat26_labels(rmat26):
    g = rmat26
    with psc.DeviceGraph(g) as dg:
        lab = dg.scc(psc.default_params(seed=1))
    ref = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=1, nthreads=THREADS)
    assert np.array_equal(lab, ref)


def test_device_transpose_rmat26(rmat26):
    g = rmat26
    with psc.DeviceGraph.directed(g.off, g.E) as dg:
        in_off, in_E = dg.transpose()
    assert np.array_equal(in_off, g.in_off)
    assert np.array_equal(in_E, g.in_E)


def test_cc_rmat26_sym(rmat26_sym):
    s = rmat26_sym
    with psc.DeviceGraph(s) as dg:
        lab = dg.cc()
    ref = O.cc(s.n, s.off, s.E, nthreads=THREADS)
    assert np.array_equal(O.canon(lab), O.canon(ref))


def test_lelist_rmat26_sym(rmat26_sym):
    s = rmat26_sym
    perm = psc.random_permutation(s.n, 4)
    with psc.DeviceGraph(s) as dg:
        le = dg.lelist(perm)
    ref = O.lelist_par(s.n, s.off, s.E, perm, nthreads=THREADS)
    assert le.shape == ref.shape
    assert np.array_equal(le, ref)


def test_batch4096_sampled_members():
    count = 4096
    g, vb = psc.batch_workload(count)
    seeds = (1000 + np.arange(count)).astype(np.uint64)
    with psc.DeviceGraph(g) as dg:
        dg.set_batch(vb)
        lab = dg.scc_batch(psc.default_params(), seeds)
    sample = range(0, count, count // 64)
    for k in sample:
        mk = g.member(vb, k)
        ref = O.scc(mk.n, mk.off, mk.E, mk.in_off, mk.in_E, seed=1000 + k, nthreads=THREADS)
        assert np.array_equal(lab[int(vb[k]):int(vb[k + 1])], ref), f"member {k}"


def test_device_symmetrize_rmat26(rmat26, rmat26_sym):
    """make_symmetric on the device: 2.1e9 pairs sorted twice, 2.1e9 kept."""
    with psc.DeviceGraph.symmetrized(rmat26.off, rmat26.E) as dg:
        assert dg.m == rmat26_sym.m
        off, E = dg.download()
    assert np.array_equal(off, rmat26_sym.off)
    assert np.array_equal(E, rmat26_sym.E)

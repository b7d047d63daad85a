"""Parity at the benchmark sizes: the kNN 10^7 x 5 graph and the 4096^2 grid
(BASELINE config 2), SCC raw labels bit-exact with the oracle and the
partition equal to Tarjan's; connectivity of the symmetrised kNN graph equal
to the oracle's partition."""
import numpy as np
import pytest

import psc
import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _dev(cuda_device):
    return cuda_device


@pytest.fixture(scope="module")
def knn():
    return psc.HostGraph.knn(10_000_000, 5, seed=2)


def test_scc_knn_full(knn):
    g = knn
    with psc.DeviceGraph(g) as dg:
        lab = dg.scc(psc.default_params(seed=1))
    assert np.array_equal(lab, O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=1))
    tar, _ = O.tarjan(g.n, g.off, g.E)
    assert np.array_equal(O.canon(lab), O.canon(tar))


def test_device_transpose_knn_full(knn):
    """Three radix passes (ids of 24 bits) over 5 * 10^7 edges."""
    with psc.DeviceGraph.directed(knn.off, knn.E) as dg:
        in_off, in_E = dg.transpose()
    assert np.array_equal(in_off, knn.in_off) and np.array_equal(in_E, knn.in_E)


def test_scc_grid_full():
    g = psc.HostGraph.grid(4096, 4096, 0.3, seed=2)
    with psc.DeviceGraph(g) as dg:
        lab = dg.scc(psc.default_params(seed=1))
    assert np.array_equal(lab, O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=1))


def test_cc_knn_full(knn):
    s = knn.symmetrize()
    with psc.DeviceGraph(s) as dg:
        lab = dg.cc()
    assert np.array_equal(O.canon(lab), O.canon(O.cc(s.n, s.off, s.E)))


def test_device_symmetrize_knn_full(knn):
    """make_symmetric on the device (two radix sorts of 10^8 pairs) equals
    the host library's, bit for bit."""
    s = knn.symmetrize()
    with psc.DeviceGraph.symmetrized(knn.off, knn.E) as dg:
        assert dg.m == s.m
        off, E = dg.download()
    assert np.array_equal(off, s.off) and np.array_equal(E, s.E)

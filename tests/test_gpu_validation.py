"""Malformed graphs are refused before any traversal kernel reads them: a
target outside [0, n), offsets that decrease, offsets that do not start at 0
(device arrays), at upload (host and device arrays, with or without a host
transpose) and in a server batch.  The checks read only the arrays
themselves, so these inputs are safe to hand to the device."""
import ctypes as C

import numpy as np
import pytest

import psc
from psc import _lib
from psc.server import CC, SCC

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _dev(cuda_device):
    return cuda_device


def good():
    return psc.HostGraph.rmat(8, 1 << 10, seed=3)


def upload(off, E, in_off, in_E, n, m):
    lib = psc.cuda()
    h = C.c_void_p()
    st = lib.psc_graph_upload(off.ctypes.data, E.ctypes.data,
                              None if in_off is None else in_off.ctypes.data,
                              None if in_E is None else in_E.ctypes.data, n, m, C.byref(h))
    if st == 0:
        lib.psc_graph_free(h)
    return st


def decreasing(off, m):
    """A copy of off with one interior offset above its successor (ends kept)."""
    off = off.copy()
    k = next(i for i in range(1, len(off) - 1) if off[i + 1] < m)
    off[k] = off[k + 1] + 1
    return off


def test_upload_rejects_a_target_outside_the_graph():
    g = good()
    E = g.E.copy()
    E[len(E) // 2] = g.n
    assert upload(g.off, E, g.in_off, g.in_E, g.n, g.m) == _lib.PSC_ERR_INVALID
    in_E = g.in_E.copy()
    in_E[0] = g.n + 5
    assert upload(g.off, g.E, g.in_off, in_E, g.n, g.m) == _lib.PSC_ERR_INVALID
    assert upload(g.off, E, None, None, g.n, g.m) == _lib.PSC_ERR_INVALID
    assert upload(g.off, g.E, g.in_off, g.in_E, g.n, g.m) == 0


def test_upload_rejects_decreasing_offsets():
    g = good()
    assert upload(decreasing(g.off, g.m), g.E, g.in_off, g.in_E, g.n, g.m) == _lib.PSC_ERR_INVALID
    assert upload(g.off, g.E, decreasing(g.in_off, g.m), g.in_E, g.n, g.m) == _lib.PSC_ERR_INVALID


def test_directed_upload_checks_before_building_the_transpose():
    g = good()
    lib = psc.cuda()
    E = g.E.copy()
    E[-1] = 0xFFFFFFFF
    h = C.c_void_p()
    assert lib.psc_graph_upload_directed(g.off.ctypes.data, E.ctypes.data, g.n, g.m,
                                         C.byref(h)) == _lib.PSC_ERR_INVALID
    assert lib.psc_graph_upload_directed(g.off.ctypes.data, g.E.ctypes.data, g.n, g.m,
                                         C.byref(h)) == 0
    lib.psc_graph_free(h)


def test_device_upload_checks_the_offset_ends():
    g = good()
    lib = psc.cuda()
    bad = g.off.copy()
    bad[0] = 1
    ptrs = []
    try:
        for a in (bad, g.E):
            p = C.c_void_p()
            assert lib.psc_device_alloc(a.nbytes, C.byref(p)) == 0
            ptrs.append(p)
            assert lib.psc_copy(p, a.ctypes.data, a.nbytes) == 0
        h = C.c_void_p()
        assert lib.psc_graph_upload_device(ptrs[0], ptrs[1], None, None, g.n, g.m,
                                           C.byref(h)) == _lib.PSC_ERR_INVALID
    finally:
        for p in ptrs:
            lib.psc_device_free(p)


@pytest.mark.parametrize("kind", [SCC, CC])
def test_server_fails_a_batch_with_a_malformed_request(kind):
    g = good() if kind == SCC else good().symmetrize()
    E = g.E.copy()
    E[3] = g.n  # a vertex id of the next request once packed: still caught
    bad = psc.HostGraph(g.n, g.m, g.off, E, symmetric=g.symmetric)
    with psc.Server(workers=1, max_batch=1) as srv:
        with pytest.raises(psc.PscError) as err:
            srv.wait(srv.submit(bad, kind, 1))
        assert err.value.status == _lib.PSC_ERR_INVALID
        lab, info = srv.wait(srv.submit(g, kind, 1))  # the server keeps serving
        assert info.status == 0 and len(lab) == g.n


@pytest.mark.parametrize("kind", [SCC, CC])
def test_server_malformed_request_fails_alone_in_its_batch(kind):
    """A malformed request packed beside good ones fails alone: the others
    are solved (the batch runs again without it) and equal their solo
    solves."""
    def sym(g):
        return g if kind == SCC else g.symmetrize()

    goods = [sym(psc.HostGraph.rmat(8, 1 << 10, seed=s)) for s in (3, 4)]
    b = sym(psc.HostGraph.rmat(8, 1 << 10, seed=5))
    E = b.E.copy()
    E[7] = b.n + 2
    bad = psc.HostGraph(b.n, b.m, b.off, E, symmetric=b.symmetric)
    blocker = sym(psc.HostGraph.knn(1_000_000, 5, seed=9))
    n, m = blocker.n, blocker.m
    # the server's footprint estimate of one blocker (SCC: transpose built on
    # the device, as submit sends none here)
    x = 16 * (n + 1) + 22 * m + 168 * n if kind == SCC else 8 * (n + 1) + 4 * m + 64 * n
    # room for one blocker and a half: the second blocker waits until the
    # first is done, the three small requests queue behind it, and all four
    # are taken as one batch (whichever worker thread takes them)
    with psc.Server(workers=1, max_batch=8, hbm_budget=int(1.5 * x)) as srv:
        r0 = srv.submit(blocker, kind, 1)
        r1 = srv.submit(blocker, kind, 2)
        ids = [srv.submit(goods[0], kind, 11), srv.submit(bad, kind, 12),
               srv.submit(goods[1], kind, 13)]
        srv.wait(r0)
        srv.wait(r1)
        outs = []
        for rid in (ids[0], ids[2]):
            lab, info = srv.wait(rid)
            assert info.status == 0
            outs.append((lab, info))
        with pytest.raises(psc.PscError) as err:
            srv.wait(ids[1])
        assert err.value.status == _lib.PSC_ERR_INVALID
    assert max(info.batch_size for _, info in outs) >= 2, "the requests were not batched"
    for g, (lab, _), seed in zip(goods, outs, (11, 13)):
        with psc.DeviceGraph(g) as dg:
            if kind == SCC:
                assert np.array_equal(lab, dg.scc(psc.default_params(seed=seed)))
            else:
                import pyoracle as O
                assert np.array_equal(O.canon(lab), O.canon(dg.cc()))


def test_symmetrize_upload_rejects_a_malformed_graph():
    g = good()
    E = g.E.copy()
    E[-1] = g.n
    lib = psc.cuda()
    h = C.c_void_p()
    assert lib.psc_graph_upload_symmetrize(g.off.ctypes.data, E.ctypes.data, g.n, g.m,
                                           C.byref(h)) == _lib.PSC_ERR_INVALID
    off = decreasing(g.off, g.m)
    assert lib.psc_graph_upload_symmetrize(off.ctypes.data, g.E.ctypes.data, g.n, g.m,
                                           C.byref(h)) == _lib.PSC_ERR_INVALID

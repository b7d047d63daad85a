"""psc_reach_noalloc — reachability for callers that may not allocate device
memory (an engine that owns the GPU's memory budget and hands out every
buffer itself, or latency-critical code that cannot pay for the
synchronisation cudaMalloc / cudaFree may imply).

The test plays such a caller: it owns the graph and output buffers, passes
them in, and checks that two calls in a row give exactly what the allocating
entry point psc_reach gives (exact equality: the output is a 0/1 flag per
vertex).  It also checks that graphs above the fixed scratch limit are
refused before any device work, that a graph of exactly the limit (which
fills the fixed bitmaps, queues and heavy list) gives the same sets, that a
malformed graph is refused, and that a call takes no device memory (the
device's free memory is the same before and after it).  This file is
collected last so that a
failure here cannot hide the other tests; it passes alone in a fresh process
as well as after them.
"""
import ctypes as C

import numpy as np
import pytest

import psc
import pyoracle as O
from psc import _lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _dev(cuda_device):
    return cuda_device


class DeviceArrays:
    """The caller's own device copies of a graph (allocated by the test)."""

    def __init__(self, g):
        self.lib = psc.cuda()
        self.ptrs = []
        self.off = self.put(g.off)
        self.E = self.put(g.E)
        self.in_off = self.put(g.in_off)
        self.in_E = self.put(g.in_E)
        self.dst = self.alloc(g.n)
        self.n, self.m = g.n, g.m

    def alloc(self, nbytes):
        p = C.c_void_p()
        _lib.check(self.lib.psc_device_alloc(max(1, nbytes), C.byref(p)), "psc_device_alloc")
        self.ptrs.append(p.value)
        return p.value

    def put(self, a):
        a = np.ascontiguousarray(a)
        p = self.alloc(a.nbytes)
        _lib.check(self.lib.psc_copy(p, a.ctypes.data, a.nbytes), "psc_copy")
        return p

    def reach(self, src, backward):
        r = C.c_uint32()
        st = self.lib.psc_reach_noalloc(self.off, self.E, self.in_off, self.in_E, self.n, self.m,
                                        src, int(backward), self.dst, None, C.byref(r))
        _lib.check(st, "psc_reach_noalloc")
        out = np.empty(self.n, np.uint8)
        _lib.check(self.lib.psc_copy(out.ctypes.data, self.dst, self.n), "psc_copy")
        return out

    def free(self):
        for p in self.ptrs:
            self.lib.psc_device_free(p)


@pytest.mark.parametrize("kind", ["rmat", "knn", "grid"])
def test_noalloc_matches_allocating_reach(kind):
    if kind == "rmat":
        g = psc.HostGraph.rmat(15, 1 << 19, seed=21)
    elif kind == "knn":
        g = psc.HostGraph.knn(200000, 5, seed=22)
    else:
        g = psc.HostGraph.grid(400, 400, 0.3, seed=23)
    arrays = DeviceArrays(g)
    try:
        with psc.DeviceGraph(g) as dg:
            rng = np.random.default_rng(7)
            srcs = rng.integers(0, g.n, 2).tolist()
            for backward in (False, True):
                # two calls in a row: the second must not see the first's state
                for src in srcs:
                    got = arrays.reach(src, backward)
                    want = dg.reach(src, backward=backward)
                    assert np.array_equal(got, want)
            ref = O.reach_seq(g.n, g.off, g.E, srcs[0])
            assert np.array_equal(arrays.reach(srcs[0], False), ref)
    finally:
        arrays.free()


def test_noalloc_symmetric_graph():
    s = psc.HostGraph.knn(50000, 5, seed=24).symmetrize()
    arrays = DeviceArrays(s)
    try:
        r = C.c_uint32()
        for src in (0, 4242):
            st = arrays.lib.psc_reach_noalloc(arrays.off, arrays.E, None, None, s.n, s.m, src, 0,
                                              arrays.dst, None, C.byref(r))
            _lib.check(st, "psc_reach_noalloc")
            out = np.empty(s.n, np.uint8)
            _lib.check(arrays.lib.psc_copy(out.ctypes.data, arrays.dst, s.n), "psc_copy")
            assert np.array_equal(out, O.reach_seq(s.n, s.off, s.E, src))
    finally:
        arrays.free()


def test_noalloc_rejects_graphs_above_the_limit():
    lib = psc.cuda()
    limit = 1 << 21
    small = DeviceArrays(psc.HostGraph.rmat(8, 1 << 10, seed=1))
    try:
        st = lib.psc_reach_noalloc(small.off, small.E, small.in_off, small.in_E, limit + 1,
                                   small.m, 0, 0, small.dst, None, None)
        assert st == _lib.PSC_ERR_TOO_LARGE
        assert b"psc_reach_noalloc" in lib.psc_strerror(st)
    finally:
        small.free()


def test_noalloc_at_the_vertex_limit():
    """n = 2^21 exactly (R-MAT, 16 draws per vertex): from the hub the search
    expands a vertex of the heavy list, switches to pull rounds and back to
    push rounds; from a second source the previous call's state must not
    leak."""
    g = psc.HostGraph.rmat(21, 16 << 21, seed=25)
    assert g.n == 1 << 21
    arrays = DeviceArrays(g)
    try:
        with psc.DeviceGraph(g) as dg:
            for src in (0, 12345):
                for backward in (False, True):
                    got = arrays.reach(src, backward)
                    assert np.array_equal(got, dg.reach(src, backward=backward))
        ref = O.reach_seq(g.n, g.off, g.E, 0)
        got = arrays.reach(0, False)
        assert np.array_equal(got, ref)
        assert got.sum() > g.n // 4
    finally:
        arrays.free()


def test_noalloc_refuses_a_malformed_graph():
    g = psc.HostGraph.rmat(10, 1 << 13, seed=26)
    E = g.E.copy()
    E[len(E) // 3] = g.n + 1
    bad = psc.HostGraph(g.n, g.m, g.off, E, g.in_off, g.in_E)
    arrays = DeviceArrays(bad)
    try:
        r = C.c_uint32()
        st = arrays.lib.psc_reach_noalloc(arrays.off, arrays.E, arrays.in_off, arrays.in_E, g.n,
                                          g.m, 0, 0, arrays.dst, None, C.byref(r))
        assert st == _lib.PSC_ERR_INVALID
    finally:
        arrays.free()
    good = DeviceArrays(g)  # the next call on a good graph is unaffected
    try:
        assert np.array_equal(good.reach(0, False), O.reach_seq(g.n, g.off, g.E, 0))
    finally:
        good.free()


def test_noalloc_takes_no_device_memory():
    """Free device memory (cudaMemGetInfo, through torch) is unchanged across
    calls, once a first pass of the same calls has loaded the kernels they
    use (lazy module loading takes device memory for code)."""
    torch = pytest.importorskip("torch")
    g = psc.HostGraph.rmat(16, 1 << 20, seed=27)
    arrays = DeviceArrays(g)
    calls = [(0, False), (0, True), (99, True), (4321, False)]
    try:
        for src, backward in calls:
            arrays.reach(src, backward)
        torch.cuda.synchronize()
        before = torch.cuda.mem_get_info(0)[0]
        for src, backward in calls:
            arrays.reach(src, backward)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info(0)[0] == before
    finally:
        arrays.free()

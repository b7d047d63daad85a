"""Python-side graph objects over the native libraries.

HostGraph   — CSR + transpose in numpy arrays (the reference's struct Graph,
              src/graph.hpp:35-43), built by libpsc_host.so's seeded
              generators or read from GBBS .bin files.
DeviceGraph — a psc_graph_t handle: the same graph resident in HBM, with the
              SCC / reach / connectivity / LE-list / BFS calls of
              libpsc_cuda.so.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import Params, Stats, check


def _ptr(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data


@dataclass
class HostGraph:
    n: int
    m: int
    off: np.ndarray              # u64[n+1]
    E: np.ndarray                # u32[m]
    in_off: np.ndarray | None = None
    in_E: np.ndarray | None = None
    symmetric: bool = False

    # -- construction through libpsc_host.so -------------------------------
    @staticmethod
    def _adopt(h: int, what: str) -> "HostGraph":
        lib = _lib.host()
        if not h:
            raise RuntimeError(f"{what}: {lib.psc_host_last_error().decode()}")
        try:
            n = lib.psc_hgraph_n(h)
            m = lib.psc_hgraph_m(h)
            off = np.ctypeslib.as_array(C.cast(lib.psc_hgraph_off(h), C.POINTER(C.c_uint64)),
                                        shape=(n + 1,)).copy()
            E = (np.ctypeslib.as_array(C.cast(lib.psc_hgraph_E(h), C.POINTER(C.c_uint32)),
                                       shape=(m,)).copy() if m else np.zeros(0, np.uint32))
            g = HostGraph(int(n), int(m), off, E)
            ip = lib.psc_hgraph_in_off(h)
            if ip:
                g.in_off = np.ctypeslib.as_array(C.cast(ip, C.POINTER(C.c_uint64)),
                                                 shape=(n + 1,)).copy()
                g.in_E = (np.ctypeslib.as_array(C.cast(lib.psc_hgraph_in_E(h),
                                                       C.POINTER(C.c_uint32)), shape=(m,)).copy()
                          if m else np.zeros(0, np.uint32))
            return g
        finally:
            lib.psc_hgraph_free(h)

    def _handle(self) -> int:
        lib = _lib.host()
        h = lib.psc_hgraph_from_csr(self.n, self.m, _ptr(self.off), _ptr(self.E))
        if not h:
            raise RuntimeError(lib.psc_host_last_error().decode())
        return h

    @staticmethod
    def rmat(log2n: int, draws: int, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             seed: int = 1) -> "HostGraph":
        g = HostGraph._adopt(_lib.host().psc_hgraph_rmat(log2n, draws, a, b, c, seed), "rmat")
        return g.with_transpose()

    @staticmethod
    def knn(npts: int, k: int = 5, seed: int = 2) -> "HostGraph":
        return HostGraph._adopt(_lib.host().psc_hgraph_knn(npts, k, seed), "knn").with_transpose()

    @staticmethod
    def grid(rows: int, cols: int, p_bidir: float = 0.3, seed: int = 2) -> "HostGraph":
        return HostGraph._adopt(_lib.host().psc_hgraph_grid(rows, cols, p_bidir, seed),
                                "grid").with_transpose()

    @staticmethod
    def from_edges(n: int, src, dst, drop_self: bool = True) -> "HostGraph":
        src = np.ascontiguousarray(src, dtype=np.uint32)
        dst = np.ascontiguousarray(dst, dtype=np.uint32)
        h = _lib.host().psc_hgraph_from_edges(n, len(src), _ptr(src), _ptr(dst), int(drop_self))
        return HostGraph._adopt(h, "from_edges").with_transpose()

    @staticmethod
    def read_bin(path: str, large: bool = False) -> "HostGraph":
        lib = _lib.host()
        h = (lib.psc_hgraph_read_large if large else lib.psc_hgraph_read_bin)(str(path).encode())
        g = HostGraph._adopt(h, "read_bin")
        return g if g.in_off is not None else g.with_transpose()

    def write_bin(self, path: str) -> None:
        lib = _lib.host()
        h = self._handle()
        try:
            if lib.psc_hgraph_write_bin(h, str(path).encode()) != 0:
                raise RuntimeError(lib.psc_host_last_error().decode())
        finally:
            lib.psc_hgraph_free(h)

    def with_transpose(self) -> "HostGraph":
        if self.in_off is not None:
            return self
        lib = _lib.host()
        h = self._handle()
        try:
            if lib.psc_hgraph_build_transpose(h) != 0:
                raise RuntimeError(lib.psc_host_last_error().decode())
            n, m = self.n, self.m
            self.in_off = np.ctypeslib.as_array(C.cast(lib.psc_hgraph_in_off(h),
                                                       C.POINTER(C.c_uint64)), shape=(n + 1,)).copy()
            self.in_E = (np.ctypeslib.as_array(C.cast(lib.psc_hgraph_in_E(h), C.POINTER(C.c_uint32)),
                                               shape=(m,)).copy() if m else np.zeros(0, np.uint32))
        finally:
            lib.psc_hgraph_free(h)
        return self

    def symmetrize(self) -> "HostGraph":
        lib = _lib.host()
        h = self._handle()
        try:
            s = lib.psc_hgraph_symmetrize(h)
        finally:
            lib.psc_hgraph_free(h)
        g = HostGraph._adopt(s, "symmetrize")
        g.symmetric = True
        g.in_off, g.in_E = g.off, g.E
        return g

    @staticmethod
    def pack(graphs: list["HostGraph"]) -> tuple["HostGraph", np.ndarray]:
        """Disjoint union of graphs for a batch: graph k's vertex i becomes
        vbase[k] + i.  Returns (union, vbase u64[len(graphs)+1])."""
        gs = [g.with_transpose() if not g.symmetric else g for g in graphs]
        vb = np.zeros(len(gs) + 1, np.uint64)
        eb = np.zeros(len(gs) + 1, np.uint64)
        vb[1:] = np.cumsum([g.n for g in gs])
        eb[1:] = np.cumsum([g.m for g in gs])

        def cat(field_off, field_E):
            off = np.concatenate([getattr(g, field_off)[:-1] + eb[k] for k, g in enumerate(gs)]
                                 + [eb[-1:]]).astype(np.uint64)
            E = np.concatenate([getattr(g, field_E).astype(np.uint64) + vb[k]
                                for k, g in enumerate(gs)]).astype(np.uint32)
            return off, E

        off, E = cat("off", "E")
        u = HostGraph(int(vb[-1]), int(eb[-1]), off, E)
        if all(g.symmetric for g in gs):
            u.symmetric = True
            u.in_off, u.in_E = u.off, u.E
        else:
            u.in_off, u.in_E = cat("in_off", "in_E")
        return u, vb

    def member(self, vbase: np.ndarray, k: int) -> "HostGraph":
        """Graph k of a packed batch, with local vertex ids."""
        v0, v1 = int(vbase[k]), int(vbase[k + 1])
        e0, e1 = int(self.off[v0]), int(self.off[v1])
        off = (self.off[v0:v1 + 1] - e0).astype(np.uint64)
        E = (self.E[e0:e1].astype(np.int64) - v0).astype(np.uint32)
        g = HostGraph(v1 - v0, e1 - e0, off, E)
        if self.symmetric:
            g.symmetric = True
            g.in_off, g.in_E = g.off, g.E
        elif self.in_off is not None:
            f0, f1 = int(self.in_off[v0]), int(self.in_off[v1])
            g.in_off = (self.in_off[v0:v1 + 1] - f0).astype(np.uint64)
            g.in_E = (self.in_E[f0:f1].astype(np.int64) - v0).astype(np.uint32)
        return g

    def edge_list(self) -> tuple[np.ndarray, np.ndarray]:
        src = np.repeat(np.arange(self.n, dtype=np.uint32), np.diff(self.off).astype(np.int64))
        return src, self.E


def random_permutation(n: int, seed: int) -> np.ndarray:
    """perm[i] = Feistel bijection of i on [0, n) (stands in for
    parlay::random_permutation, src/LeList.hpp:67)."""
    out = np.empty(n, dtype=np.uint32)
    _lib.host().psc_random_permutation(n, seed, _ptr(out))
    return out


def batch_member_spec(k: int, seed0: int = 1000, log2_min: float = 8,
                      log2_max: float = 18) -> tuple[str, int]:
    """('rmat', log2 n) or ('knn', points) of member k of the batch workload."""
    kind, size = C.c_uint32(), C.c_uint64()
    if _lib.host().psc_batch_member_spec(k, seed0, log2_min, log2_max, C.byref(kind),
                                         C.byref(size)) != 0:
        raise ValueError("log2 range must lie in [1, 31]")
    return ("rmat" if kind.value == 0 else "knn"), int(size.value)


def batch_member(k: int, seed0: int = 1000, log2_min: float = 8,
                 log2_max: float = 18) -> HostGraph:
    """Member k of the seeded batch workload (with its transpose)."""
    return HostGraph._adopt(_lib.host().psc_hgraph_batch_member(k, seed0, log2_min, log2_max),
                            "batch_member")


def batch_workload(count: int, seed0: int = 1000, log2_min: float = 8,
                   log2_max: float = 18) -> tuple[HostGraph, np.ndarray]:
    """Members 0..count-1 of the batch workload, generated in parallel and
    packed: (union, vbase)."""
    vb = np.zeros(count + 1, np.uint64)
    h = _lib.host().psc_hgraph_batch(count, seed0, log2_min, log2_max, _ptr(vb))
    return HostGraph._adopt(h, "batch_workload"), vb


def default_params(**kw) -> Params:
    p = Params()
    _lib.cuda().psc_params_default(C.byref(p))
    for k, v in kw.items():
        setattr(p, "lambda_" if k == "lambda" else k, v)
    return p


class DeviceGraph:
    """A graph resident on the current CUDA device (psc_graph_t)."""

    def __init__(self, g: HostGraph | None = None, *, handle: int | None = None):
        self._lib = _lib.cuda()
        if handle is not None:
            self.h = handle
        else:
            assert g is not None
            h = C.c_void_p()
            if g.symmetric:
                st = self._lib.psc_graph_upload(_ptr(g.off), _ptr(g.E), None, None, g.n, g.m,
                                                C.byref(h))
            else:
                gt = g.with_transpose()
                st = self._lib.psc_graph_upload(_ptr(gt.off), _ptr(gt.E), _ptr(gt.in_off),
                                                _ptr(gt.in_E), g.n, g.m, C.byref(h))
            check(st, "psc_graph_upload")
            self.h = h.value
        self.n = int(self._lib.psc_graph_num_vertices(self.h))
        self.m = int(self._lib.psc_graph_num_edges(self.h))

    @staticmethod
    def directed(off: np.ndarray, E: np.ndarray) -> "DeviceGraph":
        """Upload a CSR and build its transpose on the device."""
        lib = _lib.cuda()
        off = np.ascontiguousarray(off, dtype=np.uint64)
        E = np.ascontiguousarray(E, dtype=np.uint32)
        h = C.c_void_p()
        check(lib.psc_graph_upload_directed(_ptr(off), _ptr(E), len(off) - 1, len(E), C.byref(h)),
              "psc_graph_upload_directed")
        return DeviceGraph(handle=h.value)

    @staticmethod
    def symmetrized(off: np.ndarray, E: np.ndarray) -> "DeviceGraph":
        """Upload a directed CSR and symmetrise it on the device
        (make_symmetric semantics, src/graph.hpp:187-220)."""
        lib = _lib.cuda()
        off = np.ascontiguousarray(off, dtype=np.uint64)
        E = np.ascontiguousarray(E, dtype=np.uint32)
        h = C.c_void_p()
        check(lib.psc_graph_upload_symmetrize(_ptr(off), _ptr(E) if len(E) else None,
                                              len(off) - 1, len(E), C.byref(h)),
              "psc_graph_upload_symmetrize")
        return DeviceGraph(handle=h.value)

    def download(self) -> tuple[np.ndarray, np.ndarray]:
        """The handle's CSR (off u64[n+1], E u32[m]) in host memory."""
        off = np.empty(self.n + 1, np.uint64)
        E = np.empty(max(self.m, 1), np.uint32)
        check(self._lib.psc_graph_download(self.h, _ptr(off), _ptr(E)), "psc_graph_download")
        return off, E[: self.m]

    def free(self) -> None:
        if getattr(self, "h", None):
            self._lib.psc_graph_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.free()

    def transpose(self) -> tuple[np.ndarray, np.ndarray]:
        in_off = np.empty(self.n + 1, np.uint64)
        in_E = np.empty(max(self.m, 1), np.uint32)
        check(self._lib.psc_graph_download_transpose(self.h, _ptr(in_off), _ptr(in_E)),
              "psc_graph_download_transpose")
        return in_off, in_E[: self.m]

    def scc(self, params: Params | None = None, out: np.ndarray | None = None) -> np.ndarray:
        p = params or default_params()
        labels = out if out is not None else np.empty(self.n, np.uint64)
        check(self._lib.psc_scc(self.h, C.byref(p), _ptr(labels)), "psc_scc")
        return labels

    # -- batches of disjoint graphs -----------------------------------------
    def set_batch(self, vbase: np.ndarray) -> None:
        """Attach the graph-offset table of a packed batch (HostGraph.pack)."""
        vb = np.ascontiguousarray(vbase, dtype=np.uint64)
        check(self._lib.psc_batch_set(self.h, _ptr(vb), len(vb) - 1), "psc_batch_set")
        self.vbase = vb

    def scc_batch(self, params: Params | None = None, seeds=None,
                  out: np.ndarray | None = None) -> np.ndarray:
        """SCC labels of every graph of the batch, local to each graph."""
        p = params or default_params()
        sd = None if seeds is None else np.ascontiguousarray(seeds, dtype=np.uint64)
        labels = out if out is not None else np.empty(self.n, np.uint64)
        check(self._lib.psc_scc_batch(self.h, C.byref(p), _ptr(sd), _ptr(labels)), "psc_scc_batch")
        return labels

    def scc_batch_device(self, d_labels: int, params: Params | None = None, seeds=None) -> None:
        p = params or default_params()
        sd = None if seeds is None else np.ascontiguousarray(seeds, dtype=np.uint64)
        check(self._lib.psc_scc_batch_device(self.h, C.byref(p), _ptr(sd), d_labels),
              "psc_scc_batch_device")

    def tune(self, params: Params | None = None, seeds=None, reps: int = 2):
        """Autotuned SCC parameters for this graph or batch: (params, report)."""
        p = params or default_params()
        q = Params()
        C.memmove(C.byref(q), C.byref(p), C.sizeof(Params))
        sd = None if seeds is None else np.ascontiguousarray(seeds, dtype=np.uint64)
        rep = _lib.TuneReport()
        check(self._lib.psc_tune_scc(self.h, _ptr(sd), reps, C.byref(q), C.byref(rep)),
              "psc_tune_scc")
        return q, rep

    def cc_batch(self, beta: float = 0.2) -> np.ndarray:
        """Connectivity roots of every graph of a symmetric batch, local ids."""
        labels = np.empty(self.n, np.uint32)
        check(self._lib.psc_cc_batch(self.h, beta, _ptr(labels)), "psc_cc_batch")
        return labels

    def scc_device(self, d_labels: int, params: Params | None = None) -> None:
        p = params or default_params()
        check(self._lib.psc_scc_device(self.h, C.byref(p), d_labels), "psc_scc_device")

    def reach(self, src: int, backward: bool = False, local: bool = True,
              tau: int = 512) -> np.ndarray:
        dst = np.empty(self.n, np.uint8)
        r = C.c_uint32()
        check(self._lib.psc_reach(self.h, src, int(backward), int(local), tau, _ptr(dst),
                                  C.byref(r)), "psc_reach")
        self.last_rounds = r.value
        return dst

    def cc(self, beta: float = 0.2, forest: bool = False, out: np.ndarray | None = None):
        """Connected components of a symmetric graph: u32 root per vertex, and
        with forest=True also a spanning forest as a (k, 2) u32 edge array.
        out: optional u32[n] array (e.g. page-locked) that receives the labels."""
        labels = out if out is not None else np.empty(self.n, np.uint32)
        if forest:
            fo = np.empty(2 * max(self.n, 1), np.uint32)
            k = C.c_uint64()
            check(self._lib.psc_cc(self.h, beta, _ptr(labels), _ptr(fo), C.byref(k)), "psc_cc")
            return labels, fo[: 2 * k.value].reshape(-1, 2)
        check(self._lib.psc_cc(self.h, beta, _ptr(labels), None, None), "psc_cc")
        return labels

    def ldd(self, beta: float = 0.2) -> tuple[np.ndarray, np.ndarray]:
        """Low-diameter decomposition: (centre label, BFS parent) per vertex."""
        lab = np.empty(self.n, np.uint32)
        par = np.empty(self.n, np.uint32)
        check(self._lib.psc_ldd(self.h, beta, _ptr(lab), _ptr(par)), "psc_ldd")
        return lab, par

    def ldd_rounds(self) -> np.ndarray:
        """The last LDD's centre schedule: (k, 3) u32 rows (first candidate
        index, candidates offered, new centres), one per round."""
        r = C.c_uint32()
        cap = 256
        while True:
            out = np.empty(3 * cap, np.uint32)
            st = self._lib.psc_ldd_rounds(self.h, _ptr(out), cap, C.byref(r))
            if st == _lib.PSC_ERR_CAPACITY:
                cap = r.value
                continue
            check(st, "psc_ldd_rounds")
            return out[: 3 * r.value].reshape(-1, 3)

    def bfs(self, src: int) -> np.ndarray:
        """Hop distances from src (UINT32_MAX = unreached)."""
        d = np.empty(self.n, np.uint32)
        r = C.c_uint32()
        check(self._lib.psc_bfs(self.h, src, _ptr(d), C.byref(r)), "psc_bfs")
        self.last_rounds = r.value
        return d

    def lelist(self, perm: np.ndarray, beta: float = 1.5,
               out: np.ndarray | None = None) -> np.ndarray:
        """LE-lists for priority order perm: (k, 3) u32 triples (target,
        source vertex, distance) sorted by (target, priority).  out: optional
        u32 array of 3 * capacity entries (e.g. page-locked) that receives the
        triples; a list longer than its capacity raises PscError."""
        perm = np.ascontiguousarray(perm, dtype=np.uint32)
        if out is not None:
            ln = C.c_uint64()
            check(self._lib.psc_lelist(self.h, _ptr(perm), beta, _ptr(out), len(out) // 3,
                                       C.byref(ln)), "psc_lelist")
            return out[: 3 * ln.value].reshape(-1, 3)
        cap = max(16, 8 * self.n)
        while True:
            out = np.empty(3 * cap, np.uint32)
            ln = C.c_uint64()
            st = self._lib.psc_lelist(self.h, _ptr(perm), beta, _ptr(out), cap, C.byref(ln))
            if st == _lib.PSC_ERR_CAPACITY:
                cap = ln.value
                continue
            check(st, "psc_lelist")
            return out[: 3 * ln.value].reshape(-1, 3)

    def stats(self) -> Stats:
        s = Stats()
        check(self._lib.psc_last_stats(self.h, C.byref(s)), "psc_last_stats")
        return s

    def set_profiling(self, on: bool) -> None:
        check(self._lib.psc_set_profiling(self.h, int(on)), "psc_set_profiling")

    def profile(self) -> dict[str, dict]:
        out = {}
        for k in range(self._lib.psc_profile_count()):
            name = C.c_char_p()
            la, ms, by = C.c_uint64(), C.c_double(), C.c_double()
            check(self._lib.psc_profile_get(self.h, k, C.byref(name), C.byref(la), C.byref(ms),
                                            C.byref(by)), "psc_profile_get")
            out[name.value.decode()] = {"launches": la.value, "ms": ms.value, "bytes": by.value}
        return out

    def profile_reset(self) -> None:
        check(self._lib.psc_profile_reset(self.h), "psc_profile_reset")

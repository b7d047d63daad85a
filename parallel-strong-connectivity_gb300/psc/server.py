"""Python side of the request server (psc_server_* in include/psc.h):
continuous batching of SCC and connectivity solves under a device-memory
budget."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import RequestInfo, ServerConfig, ServerStats, check
from .graph import HostGraph, default_params

SCC = 0
CC = 1


def server_config(**kw) -> ServerConfig:
    c = ServerConfig()
    _lib.cuda().psc_server_config_default(C.byref(c))
    for k, v in kw.items():
        if k == "scc":
            c.scc = v
        else:
            setattr(c, k, v)
    return c


class Server:
    """psc_server_t: submit(graph) returns an id; wait(id) returns
    (labels, info).  SCC requests take a directed HostGraph (labels u64 as
    DeviceGraph.scc), connectivity requests a symmetric one (labels u32 roots
    local to the graph)."""

    def __init__(self, config: ServerConfig | None = None, **kw):
        self._lib = _lib.cuda()
        cfg = config or server_config(**kw)
        h = C.c_void_p()
        check(self._lib.psc_server_create(C.byref(cfg), C.byref(h)), "psc_server_create")
        self.h = h.value
        self._live = {}  # id -> (arrays kept alive, labels)

    def submit(self, g: HostGraph, kind: int = SCC, seed: int = 1,
               with_transpose: bool = False) -> int:
        """with_transpose: send g's host transpose along (SCC requests),
        else the server builds it on the device."""
        off = np.ascontiguousarray(g.off, dtype=np.uint64)
        E = np.ascontiguousarray(g.E, dtype=np.uint32)
        tin = (None, None)
        if with_transpose and kind == SCC:
            gt = g.with_transpose()
            tin = (np.ascontiguousarray(gt.in_off, dtype=np.uint64),
                   np.ascontiguousarray(gt.in_E, dtype=np.uint32))
        out = np.empty(g.n, np.uint64 if kind == SCC else np.uint32)
        rid = C.c_uint64()
        check(self._lib.psc_server_submit(
            self.h, kind, off.ctypes.data, E.ctypes.data if g.m else None,
            tin[0].ctypes.data if tin[0] is not None else None,
            tin[1].ctypes.data if tin[1] is not None and g.m else None,
            g.n, g.m, seed, out.ctypes.data, C.byref(rid)), "psc_server_submit")
        self._live[rid.value] = (off, E, out, tin)
        return rid.value

    def wait(self, rid: int) -> tuple[np.ndarray, RequestInfo]:
        info = RequestInfo()
        st = self._lib.psc_server_wait(self.h, rid, C.byref(info))
        kept = self._live.pop(rid, None)
        check(st, "psc_server_wait")
        return kept[2], info

    def drain(self) -> None:
        check(self._lib.psc_server_drain(self.h), "psc_server_drain")

    def stats(self) -> ServerStats:
        s = ServerStats()
        check(self._lib.psc_server_stats(self.h, C.byref(s)), "psc_server_stats")
        return s

    def close(self) -> None:
        if getattr(self, "h", None):
            self._lib.psc_server_destroy(self.h)
            self.h = None
            self._live.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


__all__ = ["Server", "server_config", "SCC", "CC", "default_params"]

"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the
checker and by bench.py's CPU-baseline / reference arm.  See oracle.h for the
restatement and its parity pins.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
SRCS = ["util.c", "scc.c", "cc.c", "lelist.c"]

_lib = None


def build(force: bool = False) -> Path:
    deps = [HERE / s for s in SRCS] + [HERE / "oracle.h", HERE / "common.h"]
    if force or not LIB.exists() or any(d.stat().st_mtime > LIB.stat().st_mtime for d in deps):
        LIB.parent.mkdir(parents=True, exist_ok=True)
        cmd = [os.environ.get("CC", "gcc"), "-O3", "-std=c11", "-fopenmp", "-fPIC", "-shared",
               "-Wall", "-Wextra", *[str(HERE / s) for s in SRCS], "-o", str(LIB), "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    return LIB


P = C.c_void_p
U64 = C.c_uint64
U32 = C.c_uint32
I32 = C.c_int
D = C.c_double

_SIGS = {
    "orc_transpose": (None, [U64, U64, P, P, P, P]),
    "orc_pivot_order": (U64, [U64, P, P, U64, P, C.POINTER(U64)]),
    "orc_reach_seq": (None, [U64, P, P, U32, P]),
    "orc_reach": (I32, [U64, U64, P, P, P, P, U32, P, I32, U32, I32]),
    "orc_scc": (I32, [U64, U64, P, P, P, P, D, U32, I32, I32, U64, P, I32]),
    "orc_tarjan": (U32, [U64, P, P, P]),
    "orc_canon_u64": (None, [U64, P, P]),
    "orc_canon_u32": (None, [U64, P, P]),
    "orc_bfs_seq": (None, [U64, P, P, U32, P]),
    "orc_cc": (I32, [U64, U64, P, P, D, P, I32]),
    "orc_lelist_seq": (I32, [U64, P, P, P, P, U64, C.POINTER(U64)]),
    "orc_lelist_par": (I32, [U64, P, P, P, D, P, U64, C.POINTER(U64), I32]),
    "orc_perm_at": (U64, [U64, U64, U64]),
    "orc_hash32_at": (U32, [U32]),
    "orc_hash64_at": (U64, [U64]),
}


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB))
        for k, (r, a) in _SIGS.items():
            f = getattr(_lib, k)
            f.restype = r
            f.argtypes = a
    return _lib


def _p(a):
    return a.ctypes.data


def _u64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def transpose(n, off, E):
    off, E = _u64(off), _u32(E)
    m = len(E)
    in_off = np.empty(n + 1, np.uint64)
    in_E = np.empty(max(m, 1), np.uint32)
    lib().orc_transpose(n, m, _p(off), _p(E), _p(in_off), _p(in_E))
    return in_off, in_E[:m]


def pivot_order(n, off, in_off, seed):
    off, in_off = _u64(off), _u64(in_off)
    P = np.empty(max(n, 1), np.uint32)
    nz = C.c_uint64()
    k = lib().orc_pivot_order(n, _p(off), _p(in_off), seed, _p(P), C.byref(nz))
    return P[:k], nz.value


def scc(n, off, E, in_off, in_E, beta=1.5, tau=512, local_reach=True, local_scc=True, seed=1,
        nthreads=0):
    off, E, in_off, in_E = _u64(off), _u32(E), _u64(in_off), _u32(in_E)
    labels = np.empty(max(n, 1), np.uint64)
    rc = lib().orc_scc(n, len(E), _p(off), _p(E if len(E) else np.zeros(1, np.uint32)), _p(in_off),
                       _p(in_E if len(in_E) else np.zeros(1, np.uint32)), beta, tau,
                       int(local_reach), int(local_scc), seed, _p(labels), nthreads)
    assert rc == 0
    return labels[:n]


def reach(n, off, E, in_off, in_E, src, local=True, tau=512, nthreads=0):
    off, E, in_off, in_E = _u64(off), _u32(E), _u64(in_off), _u32(in_E)
    dst = np.empty(max(n, 1), np.uint8)
    lib().orc_reach(n, len(E), _p(off), _p(E), _p(in_off), _p(in_E), src, _p(dst), int(local),
                    tau, nthreads)
    return dst[:n]


def reach_seq(n, off, E, src):
    off, E = _u64(off), _u32(E)
    dst = np.empty(max(n, 1), np.uint8)
    lib().orc_reach_seq(n, _p(off), _p(E if len(E) else np.zeros(1, np.uint32)), src, _p(dst))
    return dst[:n]


def tarjan(n, off, E):
    off, E = _u64(off), _u32(E)
    out = np.empty(max(n, 1), np.uint32)
    k = lib().orc_tarjan(n, _p(off), _p(E if len(E) else np.zeros(1, np.uint32)), _p(out))
    return out[:n], int(k)


def canon(labels):
    labels = np.ascontiguousarray(labels)
    n = len(labels)
    out = np.empty(max(n, 1), np.uint32)
    if labels.dtype == np.uint64:
        lib().orc_canon_u64(n, _p(labels), _p(out))
    else:
        labels = _u32(labels)
        lib().orc_canon_u32(n, _p(labels), _p(out))
    return out[:n]


def bfs_seq(n, off, E, src):
    off, E = _u64(off), _u32(E)
    d = np.empty(max(n, 1), np.uint32)
    lib().orc_bfs_seq(n, _p(off), _p(E if len(E) else np.zeros(1, np.uint32)), src, _p(d))
    return d[:n]


def cc(n, off, E, beta=0.2, nthreads=0):
    off, E = _u64(off), _u32(E)
    out = np.empty(max(n, 1), np.uint32)
    lib().orc_cc(n, len(E), _p(off), _p(E if len(E) else np.zeros(1, np.uint32)), beta, _p(out),
                 nthreads)
    return out[:n]


def _lelist(fn, n, off, E, perm, *extra):
    off, E, perm = _u64(off), _u32(E), _u32(perm)
    Eb = E if len(E) else np.zeros(1, np.uint32)
    cap = max(16, 8 * n)
    while True:
        out = np.empty(3 * cap, np.uint32)
        ln = C.c_uint64()
        if fn is lib().orc_lelist_seq:
            rc = fn(n, _p(off), _p(Eb), _p(perm), _p(out), cap, C.byref(ln))
        else:
            rc = fn(n, _p(off), _p(Eb), _p(perm), extra[0], _p(out), cap, C.byref(ln), extra[1])
        if rc == 0:
            return out[: 3 * ln.value].reshape(-1, 3)
        cap = ln.value


def lelist_seq(n, off, E, perm):
    return _lelist(lib().orc_lelist_seq, n, off, E, perm)


def lelist_par(n, off, E, perm, beta=1.5, nthreads=0):
    return _lelist(lib().orc_lelist_par, n, off, E, perm, beta, nthreads)

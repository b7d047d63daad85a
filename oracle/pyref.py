"""ctypes binding of the reference-built oracle (oracle/_ref/libref_*.so).

TEST INFRASTRUCTURE ONLY: imported by tests/ and by the fixture generator
tests/golden/make_ref_golden.py.  The libraries hold the reference's own
src/scc.hpp, reach.hpp, bfs.hpp, graph.hpp, Connectivity.h, ldd.hpp,
LeList.hpp and baselines/tarjan_scc/tarjan_scc.hpp, compiled unmodified from
the reference checkout against this project's ParlayLib-API stand-in
(oracle/ref_shim/) by oracle/ref.mk.  They can be built only where the
reference checkout is present; `available()` says whether they are.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
OUT = HERE / "_ref"
DEFAULT_REF = Path(os.environ.get("PSC_REFERENCE_SRC", "/root/reference"))
NAMES = ("scc", "cc", "lelist")

P = C.c_void_p
U64 = C.c_uint64
U32 = C.c_uint32
I32 = C.c_int
I64 = C.c_int64
D = C.c_double

_SIGS = {
    "scc": {
        "ref_scc": (I32, [U64, U64, P, P, P, P, D, U64, U64, I32, I32, U64, P]),
        "ref_reach": (I32, [U64, U64, P, P, P, P, U32, I32, U64, I32, P]),
        "ref_bfs": (I32, [U64, U64, P, P, U32, P]),
        "ref_make_directed": (I32, [U64, U64, P, P, P, P]),
        "ref_make_symmetric": (I64, [U64, U64, P, P, P, P]),
        "ref_tarjan": (I64, [U64, U64, P, P, P]),
        "ref_set_threads": (None, [I32]),
    },
    "cc": {
        "ref_cc": (I64, [U64, U64, P, P, D, P, P]),
        "ref_ldd": (I64, [U64, U64, P, P, D, P, P]),
        "ref_set_threads": (None, [I32]),
    },
    "lelist": {
        "ref_lelist": (I64, [U64, U64, P, P, P, D, I32, P, U64]),
        "ref_set_threads": (None, [I32]),
    },
}

_libs: dict[str, C.CDLL] = {}


def lib_path(name: str) -> Path:
    return OUT / f"libref_{name}.so"


def build(ref: Path = DEFAULT_REF, force: bool = False) -> bool:
    """Build the libraries with oracle/ref.mk when the reference checkout is
    present; returns whether all of them exist afterwards."""
    if (ref / "src" / "scc.hpp").exists():
        cmd = ["make", "-s", "-f", str(HERE / "ref.mk"), f"REF={ref}", "-j3"]
        if force:
            cmd.append("-B")
        r = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"reference oracle build failed:\n{r.stdout}\n{r.stderr}")
    return available()


def available() -> bool:
    return all(lib_path(n).exists() for n in NAMES)


def lib(name: str) -> C.CDLL:
    if name not in _libs:
        if not lib_path(name).exists():
            raise FileNotFoundError(f"{lib_path(name)} is not built (needs the reference checkout)")
        L = C.CDLL(str(lib_path(name)))
        for k, (r, a) in _SIGS[name].items():
            f = getattr(L, k)
            f.restype = r
            f.argtypes = a
        _libs[name] = L
    return _libs[name]


def set_threads(t: int) -> None:
    for n in NAMES:
        lib(n).ref_set_threads(t)


def _p(a):
    return a.ctypes.data


def _u64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)


def _u32(a):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    return a if len(a) else np.zeros(1, np.uint32)


def scc(n, off, E, in_off, in_E, beta=1.5, tau=512, lam=1024, local_reach=True, local_scc=True,
        seed=1):
    """SCC::scc's raw labels (src/scc.hpp:277-476)."""
    m = len(E)
    out = np.empty(max(n, 1), np.uint64)
    rc = lib("scc").ref_scc(n, m, _p(_u64(off)), _p(_u32(E)), _p(_u64(in_off)), _p(_u32(in_E)),
                            beta, tau, lam, int(local_reach), int(local_scc), seed, _p(out))
    assert rc == 0
    return out[:n]


def reach(n, off, E, in_off, in_E, src, forward=True, tau=512, local=True):
    out = np.empty(max(n, 1), np.uint8)
    lib("scc").ref_reach(n, len(E), _p(_u64(off)), _p(_u32(E)), _p(_u64(in_off)),
                         _p(_u32(in_E)), src, int(forward), tau, int(local), _p(out))
    return out[:n]


def bfs(n, off, E, src):
    out = np.empty(max(n, 1), np.uint32)
    lib("scc").ref_bfs(n, len(E), _p(_u64(off)), _p(_u32(E)), src, _p(out))
    return out[:n]


def make_directed(n, off, E):
    m = len(E)
    in_off = np.empty(n + 1, np.uint64)
    in_E = np.empty(max(m, 1), np.uint32)
    lib("scc").ref_make_directed(n, m, _p(_u64(off)), _p(_u32(E)), _p(in_off), _p(in_E))
    return in_off, in_E[:m]


def make_symmetric(n, off, E):
    m = len(E)
    so = np.empty(n + 1, np.uint64)
    sE = np.empty(max(2 * m, 1), np.uint32)
    ms = lib("scc").ref_make_symmetric(n, m, _p(_u64(off)), _p(_u32(E)), _p(so), _p(sE))
    return so, sE[:ms].copy()


def tarjan(n, off, E):
    out = np.empty(max(n, 1), np.uint32)
    k = lib("scc").ref_tarjan(n, len(E), _p(_u64(off)), _p(_u32(E)), _p(out))
    return out[:n], int(k)


def cc(n, off, E, beta=0.2, forest=False):
    """Connectivity's labels (src/Connectivity.h:37-119); with forest=True
    also its spanning forest as an (k, 2) array."""
    out = np.empty(max(n, 1), np.uint32)
    fo = np.empty(2 * max(n, 1), np.uint32) if forest else None
    k = lib("cc").ref_cc(n, len(E), _p(_u64(off)), _p(_u32(E)), beta, _p(out),
                         _p(fo) if forest else None)
    if forest:
        return out[:n], fo[: 2 * k].reshape(-1, 2)
    return out[:n]


def ldd(n, off, E, beta=0.2):
    out = np.empty(max(n, 1), np.uint32)
    rounds = lib("cc").ref_ldd(n, len(E), _p(_u64(off)), _p(_u32(E)), beta, _p(out), None)
    return out[:n], int(rounds)


def lelist(n, off, E, perm, beta=1.5, sequential=False):
    """LE_LIST::le_list (or seq_le_list) under the permutation perm, as an
    (k, 3) array of (target, source, distance)."""
    perm = _u32(perm)
    cap = max(16, 8 * n)
    while True:
        out = np.empty(3 * cap, np.uint32)
        k = lib("lelist").ref_lelist(n, len(E), _p(_u64(off)), _p(_u32(E)), _p(perm), beta,
                                     int(sequential), _p(out), cap)
        if k <= cap:
            return out[: 3 * k].reshape(-1, 3)
        cap = k

"""ctypes bindings of the two native libraries.

libpsc_cuda.so  — the GB300 kernels behind the C ABI of include/psc.h
libpsc_host.so  — host graph construction of include/psc_host.h

Both are loaded from parallel-strong-connectivity_gb300/_build/.  There is no
fallback: a missing library raises, so nothing silently runs elsewhere.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_BUILD = Path(__file__).resolve().parent.parent / "_build"
CUDA_LIB_PATH = _BUILD / "libpsc_cuda.so"
HOST_LIB_PATH = _BUILD / "libpsc_host.so"

PSC_OK = 0
PSC_ERR_INVALID = 1
PSC_ERR_OOM = 2
PSC_ERR_CUDA = 3
PSC_ERR_ITER_LIMIT = 4
PSC_ERR_TABLE_FULL = 5
PSC_ERR_NO_DEVICE = 6
PSC_ERR_CAPACITY = 7
PSC_ERR_TOO_LARGE = 8


class PscError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: {strerror(status)} (status {status})")


class Params(C.Structure):
    """psc_params_t (include/psc.h)."""
    _fields_ = [
        ("beta", C.c_double),
        ("tau", C.c_uint32),
        ("lambda_", C.c_uint32),
        ("local_reach", C.c_int32),
        ("local_scc", C.c_int32),
        ("seed", C.c_uint64),
        ("block", C.c_uint32),
        ("pull_div", C.c_uint32),
    ]


class Stats(C.Structure):
    """psc_stats_t (include/psc.h)."""
    _fields_ = [
        ("total_ms", C.c_double),
        ("reach_rounds", C.c_uint64),
        ("batches", C.c_uint64),
        ("subrounds", C.c_uint64),
        ("table_grows", C.c_uint64),
        ("kernel_launches", C.c_uint64),
        ("phase_ms", C.c_double * 4),
    ]


class ServerConfig(C.Structure):
    """psc_server_config_t (include/psc.h)."""
    _fields_ = [
        ("hbm_budget", C.c_uint64),
        ("workers", C.c_uint32),
        ("max_batch", C.c_uint32),
        ("cc_beta", C.c_double),
        ("scc", Params),
        ("max_batch_edges", C.c_uint64),
    ]


class ServerStats(C.Structure):
    """psc_server_stats_t (include/psc.h)."""
    _fields_ = [(f, C.c_uint64) for f in ("submitted", "completed", "failed", "rejected", "batches",
                                          "peak_bytes", "max_running", "queued", "bytes_in_use",
                                          "kernel_launches")] + \
        [("busy_ms", C.c_double)]


class RequestInfo(C.Structure):
    """psc_request_info_t (include/psc.h)."""
    _fields_ = [
        ("status", C.c_int32),
        ("batch_size", C.c_uint32),
        ("queue_ms", C.c_double),
        ("latency_ms", C.c_double),
    ]


class TuneReport(C.Structure):
    """psc_tune_report_t (include/psc.h)."""
    _fields_ = [("start_ms", C.c_double), ("best_ms", C.c_double), ("trials", C.c_uint32)]


P = C.c_void_p
U64 = C.c_uint64
U32 = C.c_uint32
I32 = C.c_int
D = C.c_double

# name -> (restype, argtypes); the exported surface of include/psc.h
CUDA_SIGNATURES = {
    "psc_params_default": (None, [C.POINTER(Params)]),
    "psc_graph_upload": (I32, [P, P, P, P, U64, U64, C.POINTER(P)]),
    "psc_graph_upload_directed": (I32, [P, P, U64, U64, C.POINTER(P)]),
    "psc_graph_upload_device": (I32, [P, P, P, P, U64, U64, C.POINTER(P)]),
    "psc_graph_free": (I32, [P]),
    "psc_graph_num_vertices": (U64, [P]),
    "psc_graph_num_edges": (U64, [P]),
    "psc_graph_download_transpose": (I32, [P, P, P]),
    "psc_graph_upload_symmetrize": (I32, [P, P, U64, U64, C.POINTER(P)]),
    "psc_graph_download": (I32, [P, P, P]),
    "psc_scc": (I32, [P, C.POINTER(Params), P]),
    "psc_scc_device": (I32, [P, C.POINTER(Params), P]),
    "psc_reach": (I32, [P, U32, I32, I32, U32, P, C.POINTER(U32)]),
    "psc_cc": (I32, [P, D, P, P, C.POINTER(U64)]),
    "psc_bfs": (I32, [P, U32, P, C.POINTER(U32)]),
    "psc_ldd": (I32, [P, D, P, P]),
    "psc_ldd_rounds": (I32, [P, P, U32, C.POINTER(U32)]),
    "psc_lelist": (I32, [P, P, D, P, U64, C.POINTER(U64)]),
    "psc_reach_noalloc": (I32, [P, P, P, P, U64, U64, U32, I32, P, P, C.POINTER(U32)]),
    "psc_batch_set": (I32, [P, P, U32]),
    "psc_batch_num_graphs": (U32, [P]),
    "psc_scc_batch": (I32, [P, C.POINTER(Params), P, P]),
    "psc_scc_batch_device": (I32, [P, C.POINTER(Params), P, P]),
    "psc_cc_batch": (I32, [P, D, P]),
    "psc_tune_scc": (I32, [P, P, U32, C.POINTER(Params), C.POINTER(TuneReport)]),
    "psc_server_config_default": (None, [C.POINTER(ServerConfig)]),
    "psc_server_create": (I32, [C.POINTER(ServerConfig), C.POINTER(P)]),
    "psc_server_submit": (I32, [P, I32, P, P, P, P, U64, U64, U64, P, C.POINTER(U64)]),
    "psc_server_wait": (I32, [P, U64, C.POINTER(RequestInfo)]),
    "psc_server_drain": (I32, [P]),
    "psc_server_stats": (I32, [P, C.POINTER(ServerStats)]),
    "psc_server_destroy": (I32, [P]),
    "psc_last_stats": (I32, [P, C.POINTER(Stats)]),
    "psc_set_profiling": (I32, [P, I32]),
    "psc_profile_count": (I32, []),
    "psc_profile_get": (I32, [P, I32, C.POINTER(C.c_char_p), C.POINTER(U64), C.POINTER(D),
                              C.POINTER(D)]),
    "psc_profile_reset": (I32, [P]),
    "psc_host_alloc": (I32, [C.c_size_t, C.POINTER(P)]),
    "psc_host_free": (I32, [P]),
    "psc_device_alloc": (I32, [C.c_size_t, C.POINTER(P)]),
    "psc_device_free": (I32, [P]),
    "psc_copy": (I32, [P, P, C.c_size_t]),
    "psc_timer_start": (I32, [P]),
    "psc_timer_stop": (I32, [P, C.POINTER(D)]),
    "psc_set_device": (I32, [I32]),
    "psc_device_count": (I32, []),
    "psc_strerror": (C.c_char_p, [I32]),
    "psc_version": (C.c_char_p, []),
}

HOST_SIGNATURES = {
    "psc_hgraph_rmat": (P, [U32, U64, D, D, D, U64]),
    "psc_hgraph_knn": (P, [U64, U32, U64]),
    "psc_hgraph_grid": (P, [U32, U32, D, U64]),
    "psc_hgraph_from_edges": (P, [U64, U64, P, P, I32]),
    "psc_hgraph_from_csr": (P, [U64, U64, P, P]),
    "psc_hgraph_read_bin": (P, [C.c_char_p]),
    "psc_hgraph_write_bin": (I32, [P, C.c_char_p]),
    "psc_hgraph_read_large": (P, [C.c_char_p]),
    "psc_hgraph_read_adj": (P, [C.c_char_p]),
    "psc_hgraph_build_transpose": (I32, [P]),
    "psc_hgraph_symmetrize": (P, [P]),
    "psc_hgraph_n": (U64, [P]),
    "psc_hgraph_m": (U64, [P]),
    "psc_hgraph_off": (P, [P]),
    "psc_hgraph_E": (P, [P]),
    "psc_hgraph_in_off": (P, [P]),
    "psc_hgraph_in_E": (P, [P]),
    "psc_hgraph_free": (None, [P]),
    "psc_hgraph_pack": (P, [P, U32, P]),
    "psc_batch_member_spec": (I32, [U32, U64, D, D, C.POINTER(U32), C.POINTER(U64)]),
    "psc_hgraph_batch_member": (P, [U32, U64, D, D]),
    "psc_hgraph_batch": (P, [U32, U64, D, D, P]),
    "psc_random_permutation": (None, [U64, U64, P]),
    "psc_host_last_error": (C.c_char_p, []),
}

_cuda: C.CDLL | None = None
_host: C.CDLL | None = None


def _bind(lib: C.CDLL, sigs: dict) -> C.CDLL:
    for name, (res, args) in sigs.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


def cuda() -> C.CDLL:
    """The CUDA library.  Raises if it has not been built."""
    global _cuda
    if _cuda is None:
        if not CUDA_LIB_PATH.exists():
            raise RuntimeError(f"{CUDA_LIB_PATH} is missing: build it first "
                               "(python -c 'import __graft_entry__ as g; g.build()')")
        _cuda = _bind(C.CDLL(str(CUDA_LIB_PATH)), CUDA_SIGNATURES)
    return _cuda


def host() -> C.CDLL:
    global _host
    if _host is None:
        if not HOST_LIB_PATH.exists():
            raise RuntimeError(f"{HOST_LIB_PATH} is missing: build it first")
        _host = _bind(C.CDLL(str(HOST_LIB_PATH)), HOST_SIGNATURES)
    return _host


def strerror(status: int) -> str:
    try:
        return cuda().psc_strerror(status).decode()
    except Exception:  # library not loadable: still name the status
        return {0: "ok", 1: "invalid argument", 2: "device out of memory", 3: "CUDA error",
                4: "iteration limit", 5: "table full", 6: "no device",
                7: "buffer too small"}.get(status, "unknown")


def check(status: int, what: str) -> None:
    if status != PSC_OK:
        raise PscError(status, what)

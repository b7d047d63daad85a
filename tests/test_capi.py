"""The C-ABI libraries load and export every function their headers declare
(CPU only: no compute call needs a GPU here)."""
import ctypes as C
import re
from pathlib import Path

import pytest

import psc
from psc import _lib

INCLUDE = Path(__file__).resolve().parent.parent / "include"
DECL = re.compile(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(psc_\w+)\s*\(", re.M)


def declared(header: str) -> list[str]:
    text = (INCLUDE / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = sorted(set(DECL.findall(text)))
    assert names, header
    return names


@pytest.mark.parametrize("name", declared("psc.h"))
def test_cuda_lib_exports(name):
    lib = C.CDLL(str(_lib.CUDA_LIB_PATH))
    assert hasattr(lib, name), name
    assert name in _lib.CUDA_SIGNATURES, f"{name} has no ctypes signature"


@pytest.mark.parametrize("name", declared("psc_host.h"))
def test_host_lib_exports(name):
    lib = C.CDLL(str(_lib.HOST_LIB_PATH))
    assert hasattr(lib, name), name
    assert name in _lib.HOST_SIGNATURES, f"{name} has no ctypes signature"


def test_every_binding_is_declared():
    assert set(_lib.CUDA_SIGNATURES) == set(declared("psc.h"))
    assert set(_lib.HOST_SIGNATURES) == set(declared("psc_host.h"))


def test_defaults_and_strings():
    p = psc.default_params()
    assert (p.beta, p.tau, p.lambda_, p.local_reach, p.local_scc) == (1.5, 512, 1024, 1, 1)
    lib = psc.cuda()
    assert lib.psc_strerror(0) == b"ok"
    assert b"invalid" in lib.psc_strerror(1)
    assert lib.psc_version().startswith(b"psc-gb300")
    assert lib.psc_profile_count() > 0
    assert lib.psc_device_count() >= 0


def test_invalid_arguments_rejected_before_device_use():
    lib = psc.cuda()
    h = C.c_void_p()
    assert lib.psc_graph_upload(None, None, None, None, 4, 0, C.byref(h)) == _lib.PSC_ERR_INVALID
    assert lib.psc_graph_upload(None, None, None, None, 0, 0, C.byref(h)) == _lib.PSC_ERR_INVALID
    import numpy as np
    off = np.array([0, 1, 2], np.uint64)
    E = np.array([1, 0], np.uint32)
    bad = np.array([0, 1, 3], np.uint64)  # off[n] != m
    assert lib.psc_graph_upload(off.ctypes.data, E.ctypes.data, bad.ctypes.data, E.ctypes.data,
                                2, 2, C.byref(h)) == _lib.PSC_ERR_INVALID
    assert lib.psc_graph_upload(off.ctypes.data, E.ctypes.data, off.ctypes.data, None, 2, 2,
                                C.byref(h)) == _lib.PSC_ERR_INVALID
    assert lib.psc_scc(None, None, None) == _lib.PSC_ERR_INVALID
    assert lib.psc_graph_free(None) == 0

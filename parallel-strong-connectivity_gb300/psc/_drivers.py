"""Builds the command-line drivers (g++ against include/psc/*.hpp, linked to
the in-tree libpsc_cuda.so and libpsc_host.so with an $ORIGIN rpath)."""
from __future__ import annotations

from pathlib import Path

from ._build import BUILD, CUDA_LIB, CXX, HOST_LIB, INCLUDE, PKG, _run, _stale

DRIVERS = {
    "scc": PKG / "drivers" / "scc_main.cpp",
    "Connectivity": PKG / "drivers" / "connectivity_main.cpp",
    "LeList": PKG / "drivers" / "lelist_main.cpp",
}


def build_drivers(force: bool = False) -> list[Path]:
    out = []
    headers = (list((INCLUDE / "psc").glob("*.hpp")) + list((INCLUDE / "psc").glob("*.h"))
               + list(INCLUDE.glob("*.h")) + list((PKG / "drivers").glob("*.hpp")))
    for name, src in DRIVERS.items():
        exe = BUILD / name
        if force or _stale(exe, [src, CUDA_LIB, HOST_LIB, *headers]):
            _run([CXX, "-O3", "-std=c++17", "-Wall", "-Wextra", f"-I{INCLUDE}",
                  f"-I{PKG / 'drivers'}", str(src),
                  "-o", str(exe), f"-L{BUILD}", "-lpsc_cuda", "-lpsc_host",
                  "-Wl,-rpath,$ORIGIN", "-lpthread", "-ldl"])
        out.append(exe)
    return out

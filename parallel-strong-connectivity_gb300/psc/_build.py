"""Native build of the library (no cmake): nvcc for the sm_103a CUDA library,
g++ for the host graph library and the command-line drivers.  Everything is
built in-tree under parallel-strong-connectivity_gb300/_build/."""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent.parent
REPO = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = REPO / "include"

NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]

CUDA_LIB = BUILD / "libpsc_cuda.so"
HOST_LIB = BUILD / "libpsc_host.so"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def cuda_sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def build_cuda(force: bool = False, jobs: int | None = None) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    srcs = cuda_sources()
    objs = [BUILD / (s.stem + ".o") for s in srcs]
    todo = [(s, o) for s, o in zip(srcs, objs) if force or _stale(o, [s] + headers)]
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(_run, [NVCC, *ARCH, *NVCC_FLAGS, "-c", str(s), "-o", str(o)])
                    for s, o in todo]
            for f in futs:
                f.result()
    if force or todo or _stale(CUDA_LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-o", str(CUDA_LIB), *map(str, objs)])
    return CUDA_LIB


def build_host(force: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    src = CSRC / "host_graph.cpp"
    deps = [src, CSRC / "psc_hash.h", INCLUDE / "psc_host.h"]
    if force or _stale(HOST_LIB, deps):
        _run([CXX, "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-Wall", "-Wextra",
              str(src), "-o", str(HOST_LIB)])
    return HOST_LIB


def build_all(force: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_cuda, force)
        b = ex.submit(build_host, force)
        a.result()
        b.result()
    from . import _drivers

    _drivers.build_drivers(force)


if __name__ == "__main__":
    build_all(force=True)

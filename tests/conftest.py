"""Shared test setup: import paths, the `gpu` marker and native builds.

CPU tests (-m "not gpu") need the oracle and libpsc_host.so, plus
libpsc_cuda.so for the export check; they are built here if missing (nvcc
cross-compiles without a GPU).  GPU tests call libpsc_cuda.so through its C
ABI and compare with the oracle.
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT / "parallel-strong-connectivity_gb300", ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session", autouse=True)
def native_builds():
    import pyoracle
    from psc import _build

    pyoracle.build()
    _build.build_host()
    _build.build_cuda()
    yield


@pytest.fixture(scope="session")
def cuda_device():
    import psc

    if psc.cuda().psc_device_count() < 1:
        pytest.skip("no CUDA device")
    return 0

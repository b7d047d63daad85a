"""Test helpers: golden fixtures and seeded graph cases."""
from __future__ import annotations

from functools import lru_cache
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden" / "graphs.npz"


@lru_cache(maxsize=1)
def golden() -> dict:
    z = np.load(GOLDEN)
    out = {}
    for name in z["names"].tolist():
        c = {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")}
        c["n"] = int(c["n"][0])
        out[name] = c
    return out


def golden_names() -> list[str]:
    return list(golden().keys())


def host_graph(case: dict):
    """HostGraph (with transpose) of a golden case, duplicates/self-loops kept."""
    import psc
    import pyoracle

    n = case["n"]
    off = case["off"].astype(np.uint64)
    E = case["E"].astype(np.uint32)
    in_off, in_E = pyoracle.transpose(n, off, E)
    return psc.HostGraph(n, len(E), off, E, in_off, in_E)


def generated(kind: str, size: int, seed: int):
    import psc

    if kind == "rmat":
        return psc.HostGraph.rmat(size, 16 << size, seed=seed)
    if kind == "knn":
        return psc.HostGraph.knn(size, 5, seed=seed)
    if kind == "grid":
        return psc.HostGraph.grid(size, size, 0.3, seed=seed)
    raise ValueError(kind)


GEN_CASES = [
    ("rmat", 10, 1), ("rmat", 13, 2), ("rmat", 16, 1),
    ("knn", 5000, 2), ("knn", 60000, 3),
    ("grid", 64, 2), ("grid", 256, 5),
]


# ---------------------------------------------------------------- outputs of
# the reference's own code (tests/golden/make_ref_golden.py)
REF_VECTORS = Path(__file__).resolve().parent / "golden" / "ref_vectors.npz"

# (kind, size, seed) of the generated cases of ref_vectors.npz by name.
REF_GEN = {
    "rmat10_s1": ("rmat", 10, 1), "rmat13_s2": ("rmat", 13, 2), "rmat16_s1": ("rmat", 16, 1),
    "knn5000_s2": ("knn", 5000, 2), "knn60000_s3": ("knn", 60000, 3),
    "grid64_s2": ("grid", 64, 2), "grid256_s5": ("grid", 256, 5),
}
REF_SCC_SEEDS = (1, 7)
REF_LE_SEED = 4


@lru_cache(maxsize=1)
def ref_vectors() -> dict:
    z = np.load(REF_VECTORS)
    out = {}
    for name in z["names"].tolist():
        c = {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")}
        c["n"] = int(c["n"][0])
        out[name] = c
    return out


def ref_names() -> list[str]:
    return list(ref_vectors().keys())


def ref_graph(name: str):
    """HostGraph (with transpose) of a ref_vectors case."""
    if name in REF_GEN:
        return generated(*REF_GEN[name])
    return host_graph(golden()[name])


def sha(a: np.ndarray) -> str:
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def canon(lab: np.ndarray) -> np.ndarray:
    """Every vertex labelled with the smallest vertex id of its class (u32)."""
    _, first, inv = np.unique(lab, return_index=True, return_inverse=True)
    return first[inv].astype(np.uint32)


def ref_check(case: dict, key: str, got: np.ndarray) -> None:
    """Asserts got equals the reference's output `key` of a case (in full
    where stored, else by SHA-256)."""
    if key in case:
        want = case[key]
        assert got.shape == want.shape and np.array_equal(got, want), \
            f"{key}: differs from the reference's code"
    assert sha(got) == str(case[key + "#sha"]), f"{key}: differs from the reference's code (sha)"

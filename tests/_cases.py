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

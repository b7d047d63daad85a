"""The CPU baseline of bench.py: the OpenMP oracle timed on the host with its
labels compared to a given labelling, the single-thread Tarjan baseline with
its partition checked, and the size bound above which Tarjan is skipped.  No
GPU: the labelling compared against is the oracle's own, or a planted wrong
one."""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402
import psc  # noqa: E402
import pyoracle as O  # noqa: E402


def small_graph():
    return psc.HostGraph.rmat(12, 1 << 16, seed=5)


def test_cpu_baseline_fields_and_checks():
    g = small_graph()
    lab = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=1)
    r = bench.cpu_baseline(g, "rmat12", gpu_labels=lab, budget_s=0.2, max_runs=2)
    assert r["kind"] == "port" and r["unit"] == "edges/s" and r["value"] > 0
    assert r["labels_equal_gpu"] is True
    t = r["tarjan_1thread"]
    assert t["threads"] == 1 and t["partition_equal_gpu"] is True
    assert t["sccs"] == len(np.unique(lab))


def test_cpu_baseline_flags_a_wrong_labelling():
    g = small_graph()
    lab = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=1).copy()
    # merge two different components: labels and partition both disagree
    a = int(np.flatnonzero(lab != lab[0])[0])
    lab[a] = lab[0]
    r = bench.cpu_baseline(g, "rmat12", gpu_labels=lab, budget_s=0.1, max_runs=1)
    assert r["labels_equal_gpu"] is False
    assert r["tarjan_1thread"]["partition_equal_gpu"] is False


def test_cpu_baseline_skips_tarjan_above_the_bound(monkeypatch):
    g = small_graph()
    monkeypatch.setattr(bench, "TARJAN_MAX_EDGES", g.m - 1)
    r = bench.cpu_baseline(g, "rmat12", budget_s=0.1, max_runs=1)
    assert "skipped" in r["tarjan_1thread"] and r["labels_equal_gpu"] is None

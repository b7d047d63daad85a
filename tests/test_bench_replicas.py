"""The replica plumbing of bench.py (N > 1 under torchrun): each rank
initialises gloo from the environment, the timing is the maximum over ranks,
and the reference arm runs on rank 0 only.  Two CPU processes, no GPU."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
ROOT = Path(__file__).resolve().parent.parent

WORKER = r"""
import os, sys, json
sys.path.insert(0, sys.argv[1])
import bench
world, rank, local, dist = bench.dist_setup()
assert world == 2 and dist is not None
t = bench.max_over_ranks(dist, 1.0 + rank)    # rank 1 is slower
bench.barrier(dist)
print(json.dumps({"rank": rank, "local": local, "max": t}), flush=True)
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_max_and_barrier(tmp_path):
    script = tmp_path / "worker.py"
    script.write_text(WORKER)
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, str(script), str(ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err
    import json
    res = sorted((json.loads(o.strip().splitlines()[-1]) for o, _ in outs), key=lambda r: r["rank"])
    assert [r["rank"] for r in res] == [0, 1]
    assert all(r["max"] == 2.0 for r in res)


def test_reference_arm_only_on_rank_zero(tmp_path):
    """run_reference returns at once on rank != 0 (prints nothing)."""
    sys.path.insert(0, str(ROOT))
    import bench

    class A:
        workload = "rmat16"
        steps = 1
        warmup = 0
        gpus = 2
        batch_count = 4

    assert bench.run_reference(A(), 2, 1, None) is None

#!/usr/bin/env python3
"""Benchmark of the GB300 strong-connectivity path.

One step = one full SCC solve (trim -> first-pivot reach -> prefix-doubling
multi-search -> partition -> finalise) of a seeded synthetic graph, the scope
of the reference's `scc cost` (src/scc.cpp:62-66: graph load and transpose
excluded).

Default workload (the headline line): directed R-MAT, n = 2^26 vertices,
2^30 draws with (a, b, c, d) = (0.57, 0.19, 0.19, 0.05), seed 3, duplicates
and self-loops removed (m = 1.06e9), beta 1.5, tau 512, VGC on: the largest
single-GPU configuration.  The graph (9.6 GB with its transpose) is far larger
than the 129 MB L2, so no flush is needed between steps.

  value   edges/s with the graph resident in HBM (psc_scc_device), timed by
          CUDA events on the library's stream around exactly K steps
  e2e     edges/s through the C ABI with pinned host buffers: every step
          uploads CSR + transpose (H2D), solves, and reads the labels (D2H)
  roofline  the dominant kernel family of a profiled pass of the same
          workload: algorithmic bytes / its event-timed duration vs the
          measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (an OpenMP restatement of the reference's
          SCC, pinned to the reference's own code) on the same graph, with
          its labels compared to the GPU's
  connectivity, lelist  the rest of the configuration on the symmetrised
          graph (m = 2.1e9): GPU time, roofline, the oracle's time and the
          equality of partition / LE-lists
  configs  the other configurations measured in the same run (--extras):
          R-MAT 2^16 (C1), kNN 10^7 x 5 and the 4096^2 grid (C2), the
          4096-graph batch against per-graph plain solves (C4) and the served
          stream with p50/p99 per arrival rate against plain solves (C5)

`--workload` runs one configuration alone (knn, grid, rmat16, rmat22, rmat26,
batch, serve).  `--impl reference` times the CPU implementation alone as the
reference arm.  Under torchrun (N > 1) each rank runs an independent replica on
its own GPU (replicas only: a solve does not shard); rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "parallel-strong-connectivity_gb300"))

WORKLOADS = {
    "knn": dict(desc="directed 2-D kNN, 10^7 points in the unit square (seed 2), k=5",
                make=lambda psc: psc.HostGraph.knn(10_000_000, 5, seed=2)),
    "grid": dict(desc="directed 4096x4096 grid, fair-coin orientation, bidirectional p=0.3 (seed 2)",
                 make=lambda psc: psc.HostGraph.grid(4096, 4096, 0.3, seed=2)),
    "rmat16": dict(desc="directed R-MAT n=2^16, 2^20 draws (0.57,0.19,0.19,0.05), seed 1, dedup",
                   make=lambda psc: psc.HostGraph.rmat(16, 1 << 20, seed=1)),
    "rmat26": dict(desc="directed R-MAT n=2^26, 2^30 draws (0.57,0.19,0.19,0.05), seed 3, dedup",
                   make=lambda psc: psc.HostGraph.rmat(26, 1 << 30, seed=3)),
    "rmat22": dict(desc="directed R-MAT n=2^22, 2^26 draws (0.57,0.19,0.19,0.05), seed 3, dedup "
                        "(a profiling size of the 2^26 configuration)",
                   make=lambda psc: psc.HostGraph.rmat(22, 1 << 26, seed=3)),
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"psc_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
        if not self.proc or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        try:
            self.path.unlink()
        except Exception:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


class Pinned:
    """numpy views over page-locked host memory from the library."""

    def __init__(self, lib):
        self.lib = lib
        self.ptrs = []

    def empty(self, n, dtype):
        dt = np.dtype(dtype)
        p = C.c_void_p()
        st = self.lib.psc_host_alloc(max(1, n * dt.itemsize), C.byref(p))
        if st:
            raise RuntimeError("pinned alloc failed")
        self.ptrs.append(p.value)
        buf = (C.c_byte * max(1, n * dt.itemsize)).from_address(p.value)
        return np.frombuffer(buf, dtype=dt, count=n)

    def copy(self, a):
        out = self.empty(len(a), a.dtype)
        out[:] = a
        return out

    def free(self):
        for p in self.ptrs:
            self.lib.psc_host_free(p)
        self.ptrs = []


# Largest graph the single-thread Tarjan baseline is timed on (a few seconds).
TARJAN_MAX_EDGES = 2e8


def cpu_baseline(g, workload: str, gpu_labels=None, budget_s: float = 15.0,
                 max_runs: int = 20) -> dict:
    """The oracle timed on the host cores; its labels of the first run are
    compared with the GPU's (raw u64 labels, same seed)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle

    threads = os.cpu_count() or 1
    runs, t_total, same = 0, 0.0, None
    while runs < max_runs and (runs == 0 or t_total < budget_s):
        t = time.perf_counter()
        lab = pyoracle.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=1, nthreads=threads)
        t_total += time.perf_counter() - t
        if runs == 0 and gpu_labels is not None:
            same = bool(np.array_equal(lab, gpu_labels))
        runs += 1
    # the reference's sequential baseline (baselines/tarjan_scc), one thread,
    # as an independent check of the partition
    if g.m <= TARJAN_MAX_EDGES:
        t = time.perf_counter()
        tl, k = pyoracle.tarjan(g.n, g.off, g.E)
        tarjan = {"ms": (time.perf_counter() - t) * 1e3, "threads": 1, "sccs": k,
                  "partition_equal_gpu": None if gpu_labels is None else
                  bool(np.array_equal(pyoracle.canon(tl), pyoracle.canon(gpu_labels)))}
    else:
        tarjan = {"skipped": f"m > {TARJAN_MAX_EDGES:.0e} edges (bounded CPU sample)"}
    return {"value": g.m * runs / t_total, "unit": "edges/s", "cores": threads, "kind": "port",
            "sample": f"{runs} full SCC solve(s) of the {workload} workload, "
                      f"{t_total / runs * 1e3:.1f} ms each (OpenMP restatement of src/scc.hpp)",
            "labels_equal_gpu": same, "tarjan_1thread": tarjan}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811
        dist.init_process_group("gloo")
    return world, rank, local, dist


def max_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def run_reference_batch(args) -> None:
    """Reference arm of the batch workload: the CPU restatement solves member
    graphs one by one (as the reference's scc binary would, one graph per
    run); each step is a stratified sample of 64 members."""
    import psc

    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle

    count = args.batch_count
    stride = max(1, count // 64)
    sample = list(range(0, count, stride))
    members = [psc.batch_member(k, **BATCH) for k in sample]
    threads = os.cpu_count() or 1

    def step():
        for k, mk in zip(sample, members):
            pyoracle.scc(mk.n, mk.off, mk.E, mk.in_off, mk.in_E, seed=BATCH["seed0"] + k,
                         nthreads=threads)

    for _ in range(args.warmup):
        step()
    t = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t
    value = len(sample) * args.steps / dt
    line = {
        "impl": "reference", "metric": "batched SCC graphs/s", "value": value, "unit": "graphs/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": f"scc_batch{count}", "graph": batch_desc(count), "graphs": count,
                   "beta": 1.5, "tau": 512, "vgc": True},
        "cpu_baseline": {"value": value, "unit": "graphs/s", "cores": threads, "kind": "port",
                         "sample": f"each step: {len(sample)} members (every {stride}th) solved "
                                   "one by one by the OpenMP restatement of src/scc.hpp"},
        "e2e": {"value": value, "unit": "graphs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference(args, world, rank, dist) -> None:
    if rank != 0:
        return
    if args.workload == "batch":
        run_reference_batch(args)
        return
    import psc

    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle

    wl = WORKLOADS[args.workload]
    g = wl["make"](psc)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        pyoracle.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=1, nthreads=threads)
    t = time.perf_counter()
    for _ in range(args.steps):
        pyoracle.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=1, nthreads=threads)
    dt = time.perf_counter() - t
    value = g.m * args.steps / dt
    line = {
        "impl": "reference", "metric": "SCC edges/s", "value": value, "unit": "edges/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": f"scc_{args.workload}", "graph": wl["desc"], "n": g.n, "m": g.m,
                   "beta": 1.5, "tau": 512, "vgc": True},
        "cpu_baseline": {"value": value, "unit": "edges/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full SCC solves (OpenMP restatement of "
                                   "src/scc.hpp; the reference needs the absent ParlayLib)"},
        "e2e": {"value": value, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ncu_step(args) -> None:
    """Profiling target: build the workload, upload it, run one warm-up solve
    and one solve, and nothing else (no CPU baseline, no end-to-end pass)."""
    import psc

    if args.workload == "batch":
        g, vb = psc.batch_workload(args.batch_count, **BATCH)
        seeds = (BATCH["seed0"] + np.arange(args.batch_count)).astype(np.uint64)
        with psc.DeviceGraph(g) as dg:
            dg.set_batch(vb)
            for _ in range(2):
                dg.scc_batch(psc.default_params(), seeds)
            st = dg.stats()
            log(f"ncu step: batch of {args.batch_count} n={g.n} m={g.m} {st.total_ms:.2f} ms, "
                f"{st.kernel_launches} launches")
        return
    wl = WORKLOADS[args.workload]
    g = wl["make"](psc)
    if args.ncu_op == "scc":
        with psc.DeviceGraph(g) as dg:
            params = psc.default_params(seed=1)
            for _ in range(2):
                dg.scc(params)
            st = dg.stats()
    elif args.ncu_op == "transpose":
        for _ in range(2):
            with psc.DeviceGraph.directed(g.off, g.E) as dg:
                st = dg.stats()
    else:
        s = g.symmetrize()
        with psc.DeviceGraph(s) as dg:
            for _ in range(2):
                if args.ncu_op == "cc":
                    dg.cc()
                else:
                    dg.lelist(psc.random_permutation(s.n, 4))
            st = dg.stats()
    log(f"ncu step: {args.ncu_op} on {args.workload} n={g.n} m={g.m} {st.total_ms:.2f} ms, "
        f"{st.kernel_launches} launches")


BATCH = dict(seed0=1000, log2_min=8.0, log2_max=18.0)


def batch_desc(count: int) -> str:
    return (f"{count} directed graphs, vertex counts log-uniform in [2^8, 2^18); even members "
            "R-MAT (16 draws per vertex, 0.57/0.19/0.19/0.05, dedup), odd members 2-D kNN k=5; "
            "member k seeded 1000+k; packed into one CSR + transpose with a graph-offset table")


def run_batch(args, world, rank, local, dist) -> dict | None:
    """Batched SCC: every step solves all graphs of the batch in one lockstep
    call (psc_scc_batch_device); compared with per-graph plain solves of a
    stratified sample of the same graphs on the same GPU."""
    import psc
    from psc import _lib

    lib = psc.cuda()
    if world > 1:
        _lib.check(lib.psc_set_device(local), "psc_set_device")
    if lib.psc_device_count() < 1:
        raise SystemExit("no CUDA device")
    count = args.batch_count
    t = time.perf_counter()
    g, vb = psc.batch_workload(count, **BATCH)
    log(f"[rank {rank}] generated batch of {count}: n={g.n} m={g.m} in {time.perf_counter() - t:.1f}s")
    n, m = g.n, g.m
    seeds = (BATCH["seed0"] + np.arange(count)).astype(np.uint64)
    params = psc.default_params()
    tune = None

    pin = Pinned(lib)
    h_off, h_E = pin.copy(g.off), pin.copy(g.E)
    h_in_off, h_in_E = pin.copy(g.in_off), pin.copy(g.in_E)
    h_labels = pin.empty(n, np.uint64)

    dg = psc.DeviceGraph(g)
    dg.set_batch(vb)
    d_labels = C.c_void_p()
    _lib.check(lib.psc_device_alloc(n * 8, C.byref(d_labels)), "psc_device_alloc")
    if not args.no_tune:
        # the autotuner picks tau / pull threshold / block / beta on this
        # batch before the timed region; every comparison below uses them
        params, rep = dg.tune(params, seeds, reps=1)
        tune = {"tau": params.tau, "pull_div": params.pull_div, "block": params.block,
                "beta": params.beta, "start_ms": rep.start_ms, "best_ms": rep.best_ms,
                "trials": rep.trials}
        log(f"[rank {rank}] tuned: {tune}")
    for _ in range(args.warmup):
        dg.scc_batch_device(d_labels.value, params, seeds)
    ref_labels = dg.scc_batch(params, seeds)
    chk = pin.empty(n, np.uint64)
    _lib.check(lib.psc_copy(chk.ctypes.data, d_labels.value, n * 8), "psc_copy")
    if not np.array_equal(chk, ref_labels):
        raise SystemExit("device and host batched SCC outputs disagree")

    barrier(dist)
    launches = 0
    with ClockSampler(local) as clk:
        _lib.check(lib.psc_timer_start(dg.h), "psc_timer_start")
        for _ in range(args.steps):
            dg.scc_batch_device(d_labels.value, params, seeds)
            launches += dg.stats().kernel_launches
        ms = C.c_double()
        _lib.check(lib.psc_timer_stop(dg.h, C.byref(ms)), "psc_timer_stop")
    barrier(dist)
    total_ms = max_over_ranks(dist, ms.value)
    clocks = clk.summary()
    value = count * args.steps * world / (total_ms / 1e3)
    last = dg.stats()

    dg.set_profiling(True)
    dg.profile_reset()
    for _ in range(args.profile_steps):
        dg.scc_batch_device(d_labels.value, params, seeds)
    prof = dg.profile()
    dg.set_profiling(False)
    roofline = roofline_of(prof, args.profile_steps)

    # per-graph plain solves of a stratified sample (every stride-th member),
    # each timed by CUDA events on its own handle, labels checked against the
    # batch's
    stride = max(1, count // args.plain_sample)
    sample = list(range(0, count, stride))
    plain_ms, plain_launches = 0.0, 0
    mismatched = 0
    for k in sample:
        mk = g.member(vb, k)
        pk = psc.default_params(seed=int(seeds[k]), tau=params.tau, pull_div=params.pull_div,
                                block=params.block, beta=params.beta)
        with psc.DeviceGraph(mk) as d1:
            lab1 = d1.scc(pk)  # warm-up and check
            if not np.array_equal(lab1, ref_labels[int(vb[k]):int(vb[k + 1])]):
                mismatched += 1
            d_l1 = C.c_void_p()
            _lib.check(lib.psc_device_alloc(mk.n * 8, C.byref(d_l1)), "psc_device_alloc")
            _lib.check(lib.psc_timer_start(d1.h), "psc_timer_start")
            d1.scc_device(d_l1.value, pk)
            t1 = C.c_double()
            _lib.check(lib.psc_timer_stop(d1.h, C.byref(t1)), "psc_timer_stop")
            plain_launches += d1.stats().kernel_launches
            lib.psc_device_free(d_l1.value)
        plain_ms += t1.value
    if mismatched:
        raise SystemExit(f"{mismatched} sampled graphs differ between batched and plain solves")
    plain_rate = len(sample) / (plain_ms / 1e3)

    # end to end: upload the packed batch from pinned memory, attach the
    # graph-offset table, solve, read the labels back
    h2d = h_off.nbytes + h_E.nbytes + h_in_off.nbytes + h_in_E.nbytes + vb.nbytes
    d2h = n * 8
    P = C.c_void_p
    sd = np.ascontiguousarray(seeds)

    def e2e_step():
        h = P()
        _lib.check(lib.psc_graph_upload(h_off.ctypes.data, h_E.ctypes.data, h_in_off.ctypes.data,
                                        h_in_E.ctypes.data, n, m, C.byref(h)), "psc_graph_upload")
        try:
            _lib.check(lib.psc_batch_set(h, vb.ctypes.data, count), "psc_batch_set")
            _lib.check(lib.psc_scc_batch(h, C.byref(params), sd.ctypes.data, h_labels.ctypes.data),
                       "psc_scc_batch")
        finally:
            lib.psc_graph_free(h)

    e2e_step()
    if not np.array_equal(h_labels, ref_labels):
        raise SystemExit("end-to-end batched SCC labels disagree")
    barrier(dist)
    t = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = max_over_ranks(dist, time.perf_counter() - t)
    e2e_value = count * args.steps * world / e2e_s

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_batch(g, vb, seeds, sample, budget_s=args.cpu_budget)

    lib.psc_device_free(d_labels.value)
    dg.free()
    pin.free()
    if rank != 0:
        return None
    line = {
        "metric": "batched SCC graphs/s", "value": value, "unit": "graphs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic",
        "config": {"workload": f"scc_batch{count}", "graph": batch_desc(count), "graphs": count,
                   "n": n, "m": m, "beta": params.beta, "tau": params.tau,
                   "pull_div": params.pull_div, "block": params.block, "vgc": True,
                   "autotune": tune,
                   "parallelism": f"replicas{world}", "l2": "inputs larger than L2 (no flush)",
                   "edges_per_s": m * args.steps * world / (total_ms / 1e3),
                   "batches": last.batches, "subrounds": last.subrounds,
                   "reach_rounds": last.reach_rounds,
                   "phase_ms": {"trim": last.phase_ms[0], "first_pivot": last.phase_ms[1],
                                "multi_search": last.phase_ms[2], "table_resize": last.phase_ms[3]}},
        "plain": {"value": plain_rate, "unit": "graphs/s", "sample": len(sample),
                  "ms_per_graph": plain_ms / len(sample),
                  "launches_per_graph": plain_launches / len(sample),
                  "how": f"psc_scc_device on each of {len(sample)} members (every {stride}th), "
                         "graph resident, CUDA events per call; labels equal to the batch's"},
        "speedup_vs_plain": value / plain_rate,
        "e2e": {"value": e2e_value, "unit": "graphs/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s / args.steps * 1e3},
        "roofline": roofline,
        "profile": {k: {"launches": v["launches"] // max(1, args.profile_steps),
                        "ms": v["ms"] / max(1, args.profile_steps)}
                    for k, v in prof.items() if v["launches"]},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "gpu_launches": launches,
    }
    return line


SERVE = dict(pool=48, seed0=5000, log10_min=3.0, log10_max=7.0, cc_share=0.2,
             rates=(200, 1000, 5000), requests=240, budget=120 << 30)


def serve_pool(psc, count: int, seed0: int):
    """Seeded request pool: member i has n = floor(10^u) vertices, u uniform
    in [3, 7) drawn from seed0 + i; even members R-MAT (2^round(log2 n)
    vertices, 16 draws per vertex), odd members 2-D kNN (k = 5)."""
    import math
    out = []
    for i in range(count):
        u = SERVE["log10_min"] + (SERVE["log10_max"] - SERVE["log10_min"]) * _unit(seed0 + i)
        n = int(10 ** u)
        if i % 2 == 0:
            log2n = max(8, round(math.log2(n)))
            out.append(psc.HostGraph.rmat(log2n, 16 << log2n, seed=seed0 + i))
        else:
            out.append(psc.HostGraph.knn(max(n, 16), 5, seed=seed0 + i))
    return out


def _unit(seed: int) -> float:
    """Uniform [0, 1) draw of a seed (SplitMix64 finaliser of the seed)."""
    x = (seed + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    x ^= x >> 30
    x = (x * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    x ^= x >> 27
    x = (x * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    x ^= x >> 31
    return (x >> 11) / float(1 << 53)


def run_serve(args, world, rank, local, dist) -> dict | None:
    """Served stream: Poisson arrivals of SCC (80 %) and connectivity (20 %)
    requests drawn from a seeded pool, through the request server
    (continuous batching, 120 GiB admission budget); latency p50/p99 and
    graphs/s per arrival rate, against the same requests solved one by one
    with plain calls."""
    import threading
    import psc
    from psc import _lib
    from psc.server import CC, SCC

    lib = psc.cuda()
    if world > 1:
        _lib.check(lib.psc_set_device(local), "psc_set_device")
    t = time.perf_counter()
    pool = serve_pool(psc, SERVE["pool"], SERVE["seed0"])
    rng = np.random.default_rng(SERVE["seed0"])
    nreq = args.serve_requests
    picks = rng.integers(0, len(pool), nreq)
    kinds = np.where(rng.random(nreq) < SERVE["cc_share"], CC, SCC)
    sym = {}
    for i in sorted(set(picks[kinds == CC].tolist())):
        sym[i] = pool[i].symmetrize()
    # pinned copies of the request arrays (what a serving front end holds)
    pin = Pinned(lib)
    parr = {}
    for i in set(picks.tolist()):
        for kind in (SCC, CC):
            if kind == CC and i not in sym:
                continue
            g = pool[i] if kind == SCC else sym[i]
            parr[(i, kind)] = (g, pin.copy(g.off), pin.copy(g.E) if g.m else g.E)
    ptr_t = {i: (pool[i], pin.copy(pool[i].in_off), pin.copy(pool[i].in_E) if pool[i].m else
                 pool[i].in_E) for i in set(picks[kinds == SCC].tolist())}
    log(f"[rank {rank}] serve pool of {len(pool)} graphs (n {min(g.n for g in pool)}.."
        f"{max(g.n for g in pool)}) built in {time.perf_counter() - t:.1f}s")
    seeds = (1000 + np.arange(nreq)).astype(np.uint64)

    def request(j):
        g, off, E = parr[(int(picks[j]), int(kinds[j]))]
        return g, off, E, int(kinds[j]), int(seeds[j])

    def submit(srv, j, out):
        # requests carry the graph as struct Graph does: CSR and, for SCC,
        # its transpose
        g, off, E, kind, seed = request(j)
        tin = (ptr_t[int(picks[j])][1].ctypes.data, ptr_t[int(picks[j])][2].ctypes.data) \
            if kind == SCC else (None, None)
        rid = C.c_uint64()
        _lib.check(lib.psc_server_submit(srv, kind, off.ctypes.data, E.ctypes.data, tin[0], tin[1],
                                         g.n, g.m, seed, out.ctypes.data, C.byref(rid)),
                   "psc_server_submit")
        return rid.value

    outs = [pin.empty(request(j)[0].n, np.uint64 if kinds[j] == SCC else np.uint32)
            for j in range(nreq)]

    def serve(rate: float | None) -> dict:
        cfg = psc.server_config(hbm_budget=SERVE["budget"], workers=args.serve_workers)
        if args.serve_batch_edges is not None:
            cfg.max_batch_edges = args.serve_batch_edges
        h = C.c_void_p()
        _lib.check(lib.psc_server_create(C.byref(cfg), C.byref(h)), "psc_server_create")
        arr = np.cumsum(rng.exponential(1.0 / rate, nreq)) if rate else np.zeros(nreq)
        ids = [None] * nreq
        lat = np.zeros(nreq)
        done_t = np.zeros(nreq)
        ready = threading.Event()

        def waiter():
            ready.wait()
            for j in range(nreq):
                while ids[j] is None:
                    time.sleep(0.0002)
                info = _lib.RequestInfo()
                _lib.check(lib.psc_server_wait(h, ids[j], C.byref(info)), "psc_server_wait")
                lat[j] = info.latency_ms
                done_t[j] = time.perf_counter()

        wt = threading.Thread(target=waiter)
        wt.start()
        t0 = time.perf_counter()
        ready.set()
        for j in range(nreq):
            d = t0 + arr[j] - time.perf_counter()
            if d > 0:
                time.sleep(d)
            ids[j] = submit(h, j, outs[j])
        wt.join()
        st = _lib.ServerStats()
        lib.psc_server_stats(h, C.byref(st))
        lib.psc_server_destroy(h)
        span = done_t.max() - t0
        return {"rate": rate, "graphs_per_s": nreq / span, "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "batches": int(st.batches),
                "max_in_flight": int(st.max_running), "peak_gb": st.peak_bytes / 1e9,
                "launches": int(st.kernel_launches)}

    serve(None)  # warm-up (pool allocations, module load)
    # reference results of the mixed stream for the equality check
    sweep = []
    with ClockSampler(local) as clk:
        for rate in SERVE["rates"]:
            sweep.append(serve(float(rate)))
            log(f"  rate {rate}/s: {sweep[-1]}")
        sat = serve(None)
    clocks = clk.summary()
    mixed = [o.copy() for o in outs]

    # plain sequential solves of the same stream
    t = time.perf_counter()
    for j in range(nreq):
        g, off, E, kind, seed = request(j)
        h = C.c_void_p()
        if kind == SCC:
            # the host-built transpose is uploaded too (not timed to build)
            _, in_off, in_E = ptr_t[int(picks[j])]
            _lib.check(lib.psc_graph_upload(off.ctypes.data, E.ctypes.data, in_off.ctypes.data,
                                            in_E.ctypes.data, g.n, g.m, C.byref(h)), "upload")
            p = psc.default_params(seed=seed)
            _lib.check(lib.psc_scc(h, C.byref(p), outs[j].ctypes.data), "psc_scc")
        else:
            _lib.check(lib.psc_graph_upload(off.ctypes.data, E.ctypes.data, None, None, g.n, g.m,
                                            C.byref(h)), "upload")
            _lib.check(lib.psc_cc(h, 0.2, outs[j].ctypes.data, None, None), "psc_cc")
        lib.psc_graph_free(h)
    plain_s = time.perf_counter() - t
    bad = 0
    for j in range(nreq):
        if kinds[j] == SCC:
            bad += not np.array_equal(outs[j], mixed[j])
        else:
            sys.path.insert(0, str(ROOT / "oracle"))
            import pyoracle
            bad += not np.array_equal(pyoracle.canon(outs[j]), pyoracle.canon(mixed[j]))
    if bad:
        raise SystemExit(f"{bad} served results differ from plain solves")
    plain_rate = nreq / plain_s
    pin.free()
    if rank != 0:
        return None
    top = sweep[-1]
    line = {
        "metric": "served SCC/CC graphs/s", "value": sat["graphs_per_s"], "unit": "graphs/s",
        "n_gpus": world, "steps": len(SERVE["rates"]) + 1, "warmup": 1,
        "ms_per_step": 1e3 * nreq / sat["graphs_per_s"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": "serve", "requests_per_rate": nreq,
                   "graph": "pool of 48 seeded graphs, n = floor(10^u), u uniform in [3, 7); even "
                            "R-MAT (16 draws per vertex), odd 2-D kNN k=5; 80 % SCC (directed), "
                            "20 % connectivity (symmetrised); Poisson arrivals",
                   "hbm_budget_gb": SERVE["budget"] / 2**30, "workers": args.serve_workers,
                   "max_batch_edges": int(psc.server_config().max_batch_edges
                                          if args.serve_batch_edges is None
                                          else args.serve_batch_edges),
                   "parallelism": f"replicas{world}"},
        "sweep": sweep, "saturated": sat,
        "latency_ms": {"p50": top["p50_ms"], "p99": top["p99_ms"], "rate": top["rate"]},
        "plain": {"value": plain_rate, "unit": "graphs/s",
                  "how": "the same requests one by one from pinned memory: upload (SCC: CSR and "
                         "its host-built transpose), psc_scc or psc_cc, labels to host, free; "
                         "results equal the served ones"},
        "speedup_vs_plain": sat["graphs_per_s"] / plain_rate,
        "e2e": {"value": sat["graphs_per_s"], "unit": "graphs/s",
                "h2d_bytes_per_step": int(sum((2 if kinds[j] == SCC else 1) *
                                              (request(j)[0].off.nbytes + request(j)[0].E.nbytes)
                                              for j in range(nreq))),
                "d2h_bytes_per_step": int(sum(o.nbytes for o in outs))},
        "roofline": None, "cpu_baseline": None, "clocks": clocks,
        "gpu_launches": sat["launches"],
    }
    return line


def cpu_baseline_batch(g, vb, seeds, sample, budget_s: float = 15.0) -> dict:
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle

    threads = os.cpu_count() or 1
    done, t_total = 0, 0.0
    for k in sample:
        mk = g.member(vb, k)
        t = time.perf_counter()
        pyoracle.scc(mk.n, mk.off, mk.E, mk.in_off, mk.in_E, seed=int(seeds[k]), nthreads=threads)
        t_total += time.perf_counter() - t
        done += 1
        if t_total > budget_s:
            break
    return {"value": done / t_total, "unit": "graphs/s", "cores": threads, "kind": "port",
            "sample": f"{done} member graphs (every {sample[1] - sample[0] if len(sample) > 1 else 1}"
                      f"th) solved one by one, {t_total / done * 1e3:.1f} ms each (OpenMP "
                      "restatement of src/scc.hpp)"}


# DRAM bytes (read + write) per launch of a workload's dominant kernel family:
# dram__bytes_read.sum + dram__bytes_write.sum of the family's kernels in one
# ncu capture (a single pass) of `python bench.py --ncu-step --workload W`,
# divided by the family's profiled scopes (the launches counted in the
# roofline entry).  A workload without a capture of its current dominant
# kernels reports null.
#   scc_rmat26 / reach_pull: k_reach_pull_staged, k_reach_pull,
#     k_pull_out_edges and k_queue_to_bitmap, 6,605 MB over 2 solves x 6 scopes
#   scc_knn / reach_vgc: k_reach_vgc, 10,912 MB over 185 launches
NCU_TRAFFIC: dict = {
    ("scc_rmat26", "reach_pull"): 550.4e6,
    ("scc_knn", "reach_vgc"): 59.0e6,
}


def roofline_of(prof: dict, steps: int, workload: str = "") -> dict:
    fam, top = max(prof.items(), key=lambda kv: kv[1]["ms"])
    peak, peak_kind = peaks()
    achieved = (top["bytes"] / top["launches"]) / (top["ms"] / top["launches"] / 1e3) / 1e9 \
        if top["launches"] and top["ms"] > 0 else 0.0
    prof_total = sum(v["ms"] for v in prof.values())
    return {
        "bound": "hbm", "kernel": fam, "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak, "peak_source": peak_kind,
        "traffic": NCU_TRAFFIC.get((workload, fam)),
        "launches": top["launches"] // max(1, steps),
        "share": top["ms"] / prof_total if prof_total else None,
        "bytes_per_launch": top["bytes"] / max(1, top["launches"]),
    }


def run_gpu(args, world, rank, local, dist) -> dict | None:
    import psc
    from psc import _lib

    lib = psc.cuda()
    if world > 1:
        _lib.check(lib.psc_set_device(local), "psc_set_device")
    if lib.psc_device_count() < 1:
        raise SystemExit("no CUDA device")
    wl = WORKLOADS[args.workload]
    t = time.perf_counter()
    g = wl["make"](psc)
    log(f"[rank {rank}] generated {args.workload}: n={g.n} m={g.m} in {time.perf_counter() - t:.1f}s")
    params = psc.default_params(seed=1)
    n, m = g.n, g.m

    pin = Pinned(lib)
    h_off, h_E = pin.copy(g.off), pin.copy(g.E)
    h_in_off, h_in_E = pin.copy(g.in_off), pin.copy(g.in_E)
    h_labels = pin.empty(n, np.uint64)

    dg = psc.DeviceGraph(g)
    d_labels = C.c_void_p()
    _lib.check(lib.psc_device_alloc(n * 8, C.byref(d_labels)), "psc_device_alloc")

    # warm-up
    for _ in range(args.warmup):
        dg.scc_device(d_labels.value, params)
    # correctness guard: device labels == host-call labels
    ref_labels = dg.scc(params)
    chk = pin.empty(n, np.uint64)
    _lib.check(lib.psc_copy(chk.ctypes.data, d_labels.value, n * 8), "psc_copy")
    if not np.array_equal(chk, ref_labels):
        raise SystemExit("device and host SCC outputs disagree")

    # timed region: exactly K steps, CUDA events on the library's stream
    barrier(dist)
    _lib.check(lib.psc_copy(None, None, 0), "sync")
    launches = 0
    with ClockSampler(local) as clk:
        _lib.check(lib.psc_timer_start(dg.h), "psc_timer_start")
        for _ in range(args.steps):
            dg.scc_device(d_labels.value, params)
            launches += dg.stats().kernel_launches
        ms = C.c_double()
        _lib.check(lib.psc_timer_stop(dg.h, C.byref(ms)), "psc_timer_stop")
    barrier(dist)
    total_ms = max_over_ranks(dist, ms.value)
    clocks = clk.summary()
    value = m * args.steps * world / (total_ms / 1e3)
    last = dg.stats()

    # profiled pass (same workload, after the timed region)
    dg.set_profiling(True)
    dg.profile_reset()
    for _ in range(args.profile_steps):
        dg.scc_device(d_labels.value, params)
    prof = dg.profile()
    dg.set_profiling(False)
    roofline = roofline_of(prof, args.profile_steps, f"scc_{args.workload}")

    # end to end through the C ABI with pinned host buffers
    h2d = h_off.nbytes + h_E.nbytes + h_in_off.nbytes + h_in_E.nbytes
    d2h = n * 8
    P = C.c_void_p

    def e2e_step():
        h = P()
        _lib.check(lib.psc_graph_upload(h_off.ctypes.data, h_E.ctypes.data, h_in_off.ctypes.data,
                                        h_in_E.ctypes.data, n, m, C.byref(h)), "psc_graph_upload")
        try:
            _lib.check(lib.psc_scc(h, C.byref(params), h_labels.ctypes.data), "psc_scc")
        finally:
            lib.psc_graph_free(h)

    e2e_step()
    if not np.array_equal(h_labels, ref_labels):
        raise SystemExit("end-to-end SCC labels disagree")
    barrier(dist)
    t = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = max_over_ranks(dist, time.perf_counter() - t)
    e2e_value = m * args.steps * world / e2e_s

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(g, args.workload, ref_labels, budget_s=args.cpu_budget)
        if cpu["labels_equal_gpu"] is False:
            raise SystemExit("GPU labels differ from the oracle's")

    lib.psc_device_free(d_labels.value)
    dg.free()
    pin.free()
    extra = cc_le_extra(psc, g, rank, world, args) if args.workload == "rmat26" else {}
    if rank != 0:
        return None
    line = {
        "metric": "SCC edges/s", "value": value, "unit": "edges/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic",
        "config": {"workload": f"scc_{args.workload}", "graph": wl["desc"], "n": n, "m": m,
                   "beta": 1.5, "tau": 512, "vgc": True, "parallelism": f"replicas{world}",
                   "l2": "inputs larger than L2 (no flush)" if (h2d > 129e6) else "L2-resident",
                   "batches": last.batches, "subrounds": last.subrounds,
                   "reach_rounds": last.reach_rounds,
                   "phase_ms": {"trim": last.phase_ms[0], "first_pivot": last.phase_ms[1],
                                "multi_search": last.phase_ms[2], "table_resize": last.phase_ms[3]}},
        "e2e": {"value": e2e_value, "unit": "edges/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s / args.steps * 1e3},
        "roofline": roofline,
        "profile": {k: {"launches": v["launches"] // max(1, args.profile_steps),
                        "ms": v["ms"] / max(1, args.profile_steps)}
                    for k, v in prof.items() if v["launches"]},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "gpu_launches": launches,
    }
    line.update(extra)
    return line


def cc_le_extra(psc, g, rank, world, args) -> dict:
    """The rest of the R-MAT 2^26 configuration: connectivity and LE-lists
    (permutation seed 4) on the symmetrised graph, resident on the device,
    each with the roofline of its dominant kernel family, and (rank 0, one
    replica) the oracle's connectivity and parallel LE-lists on the host
    cores: their time as the CPU baseline and their output as the check."""
    t = time.perf_counter()
    s = g.symmetrize()
    log(f"[rank {rank}] symmetrised: m = {s.m} in {time.perf_counter() - t:.1f}s")
    out = {}
    # the timed calls read the permutation from and write their output to
    # page-locked host memory, as the SCC end-to-end pass does
    pin = Pinned(psc.cuda())
    perm = pin.copy(psc.random_permutation(s.n, 4))
    with psc.DeviceGraph(s) as dg:
        lab = dg.cc()
        lab_pin = pin.empty(s.n, np.uint32)
        cc_ms = min((dg.cc(out=lab_pin), dg.stats().total_ms)[1] for _ in range(3))
        dg.set_profiling(True)
        dg.profile_reset()
        dg.cc()
        cc_roof = roofline_of(dg.profile(), 1)
        dg.set_profiling(False)
        le = dg.lelist(perm)
        le_pin = pin.empty(3 * len(le), np.uint32)
        le_ms = min((dg.lelist(perm, out=le_pin), dg.stats().total_ms)[1] for _ in range(2))
        dg.set_profiling(True)
        dg.profile_reset()
        dg.lelist(perm)
        le_roof = roofline_of(dg.profile(), 1)
        dg.set_profiling(False)
    out["connectivity"] = {"ms": cc_ms, "edges_per_s": s.m / (cc_ms / 1e3), "m_sym": s.m,
                           "components": int(len(np.unique(lab))), "roofline": cc_roof,
                           "scope": "graph resident; labels copied to page-locked host memory"}
    out["lelist"] = {"ms": le_ms, "triples": int(len(le)), "perm_seed": 4, "roofline": le_roof,
                     "scope": "graph resident; permutation from and triples to page-locked "
                              "host memory"}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sys.path.insert(0, str(ROOT / "oracle"))
        import pyoracle
        threads = os.cpu_count() or 1
        t = time.perf_counter()
        ref = pyoracle.cc(s.n, s.off, s.E, nthreads=threads)
        cpu_ms = (time.perf_counter() - t) * 1e3
        out["connectivity"]["cpu_baseline"] = {
            "ms": cpu_ms, "cores": threads, "kind": "port",
            "sample": "one connectivity solve (OpenMP restatement of src/Connectivity.h)"}
        out["connectivity"]["partition_equal_oracle"] = bool(
            np.array_equal(pyoracle.canon(ref), pyoracle.canon(lab)))
        del ref
        if not args.no_le_check:
            t = time.perf_counter()
            ref_le = pyoracle.lelist_par(s.n, s.off, s.E, perm, nthreads=threads)
            cpu_ms = (time.perf_counter() - t) * 1e3
            out["lelist"]["cpu_baseline"] = {
                "ms": cpu_ms, "cores": threads, "kind": "port",
                "sample": "one LE-list solve (OpenMP restatement of src/LeList.hpp:219-328)"}
            out["lelist"]["equal_oracle"] = bool(ref_le.shape == le.shape and
                                                 np.array_equal(ref_le, le))
            if not out["lelist"]["equal_oracle"]:
                raise SystemExit("GPU LE-lists differ from the oracle's")
        if not out["connectivity"]["partition_equal_oracle"]:
            raise SystemExit("GPU connectivity partition differs from the oracle's")
    pin.free()
    return out


# Keys of a workload's line kept when it rides on the headline line.
EXTRA_KEYS = ("metric", "value", "unit", "ms_per_step", "speedup_vs_plain", "plain", "e2e",
              "roofline", "cpu_baseline", "latency_ms", "sweep", "saturated", "clocks",
              "gpu_launches")


def run_extras(args, world, rank, local, dist) -> dict:
    """The other configurations, each measured as its own workload would be
    (fewer CPU-baseline seconds) and summarised under the headline line."""
    out = {}
    for name in [x for x in args.extras.split(",") if x and x != "none"]:
        sub = argparse.Namespace(**vars(args))
        sub.workload = name
        sub.cpu_budget = min(args.cpu_budget, 5.0)
        t = time.perf_counter()
        if name == "batch":
            line = run_batch(sub, world, rank, local, dist)
        elif name == "serve":
            line = run_serve(sub, world, rank, local, dist)
        else:
            line = run_gpu(sub, world, rank, local, dist)
        log(f"[rank {rank}] extra {name}: {time.perf_counter() - t:.1f}s")
        if line is not None:
            cfg = line.get("config", {})
            key = cfg.get("workload", name)
            out[key] = {k: line[k] for k in EXTRA_KEYS if k in line}
            out[key]["config"] = {k: v for k, v in cfg.items() if k not in ("phase_ms",)}
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["psc", "reference"], default="psc")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["batch", "serve"], default="rmat26",
                    help="headline workload (default: R-MAT 2^26, the largest single-GPU "
                         "configuration, with its connectivity and LE-lists)")
    ap.add_argument("--extras", default="rmat16,knn,grid,batch,serve",
                    help="with the rmat26 headline: other configurations measured in the same "
                         "run and summarised under its line ('none' for the headline alone)")
    ap.add_argument("--cpu-budget", type=float, default=15.0,
                    help="seconds of CPU-baseline solves on the host cores")
    ap.add_argument("--no-le-check", action="store_true",
                    help="rmat26: skip the oracle's LE-lists (check and CPU baseline)")
    ap.add_argument("--serve-requests", type=int, default=SERVE["requests"],
                    help="requests per arrival rate of the serve workload")
    ap.add_argument("--serve-workers", type=int, default=4)
    ap.add_argument("--serve-batch-edges", type=int, default=None,
                    help="serve workload: edge cap of one server batch (library default if unset)")
    ap.add_argument("--no-tune", action="store_true",
                    help="batch workload: keep the default parameters")
    ap.add_argument("--batch-count", type=int, default=4096,
                    help="graphs in the batch workload")
    ap.add_argument("--plain-sample", type=int, default=256,
                    help="batch members solved one by one for the plain comparison")
    ap.add_argument("--profile-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ncu-step", action="store_true",
                    help="profiling target: one warm-up solve and one solve only")
    ap.add_argument("--ncu-op", choices=["scc", "cc", "lelist", "transpose"], default="scc",
                    help="operation of --ncu-step (cc and lelist on the symmetrised graph)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "psc":
        log("note: fewer than 3 warm-up steps")
    world, rank, local, dist = dist_setup()
    if args.ncu_step:
        run_ncu_step(args)
        return
    try:
        if args.impl == "reference":
            run_reference(args, world, rank, dist)
            return
        if args.workload == "batch":
            line = run_batch(args, world, rank, local, dist)
        elif args.workload == "serve":
            line = run_serve(args, world, rank, local, dist)
        else:
            line = run_gpu(args, world, rank, local, dist)
        if args.workload == "rmat26":
            extras = run_extras(args, world, rank, local, dist)
            if line is not None:
                line["configs"] = extras
        if line is not None:
            print(json.dumps(line), flush=True)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()

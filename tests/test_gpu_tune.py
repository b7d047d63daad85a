"""GPU tests of the autotuner and of the block-size knob it turns: tuned
parameters are valid, and solves with them keep the oracle's labels (raw
labels for the same beta and tau, the partition always)."""
import numpy as np
import pytest

import psc
import pyoracle as O

pytestmark = pytest.mark.gpu

TAUS = {32, 64, 128, 256, 512}
PULLS = {5, 10, 20, 40, 80}
BLOCKS = {128, 256, 512}
BETAS = {1.5, 2.0, 3.0, 4.0}


@pytest.fixture(scope="module", autouse=True)
def _dev(cuda_device):
    return cuda_device


def check_params(q):
    assert q.tau in TAUS and q.pull_div in PULLS and q.block in BLOCKS and q.beta in BETAS


@pytest.mark.parametrize("block", [128, 256, 512])
def test_block_sizes_keep_labels(block):
    g = psc.HostGraph.rmat(14, 16 << 14, seed=7)
    ref = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=3)
    with psc.DeviceGraph(g) as dg:
        for pull_div in (1, 20, 100000):  # push-heavy, default, pull-heavy
            lab = dg.scc(psc.default_params(seed=3, block=block, pull_div=pull_div,
                                            local_reach=0, local_scc=0))
            assert np.array_equal(lab, ref)
            assert np.array_equal(dg.scc(psc.default_params(seed=3, block=block)), ref)


def test_tune_plain_graph():
    g = psc.HostGraph.knn(40000, 5, seed=4)
    with psc.DeviceGraph(g) as dg:
        q, rep = dg.tune(psc.default_params(seed=2))
        check_params(q)
        assert rep.trials >= 1 + 4 + 4 + 2 + 3
        assert rep.best_ms <= rep.start_ms
        lab = dg.scc(q)
    ref = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=2, beta=q.beta, tau=q.tau)
    assert np.array_equal(lab, ref)


def test_tune_batch():
    u, vb = psc.batch_workload(24, 1000, 5, 12)
    seeds = 1000 + np.arange(24, dtype=np.uint64)
    with psc.DeviceGraph(u) as dg:
        dg.set_batch(vb)
        base = dg.scc_batch(psc.default_params(), seeds)
        q, rep = dg.tune(psc.default_params(), seeds, reps=1)
        check_params(q)
        lab = dg.scc_batch(q, seeds)
    for k in range(24):
        a, b = base[vb[k]:vb[k + 1]], lab[vb[k]:vb[k + 1]]
        assert np.array_equal(O.canon(a), O.canon(b))
        m = u.member(vb, k)
        ref = O.scc(m.n, m.off, m.E, m.in_off, m.in_E, seed=int(seeds[k]), beta=q.beta, tau=q.tau)
        assert np.array_equal(b, ref)

"""The CPU oracle pinned against the golden fixtures and against its own
baselines (Tarjan, sequential reach/BFS/LE-list).  CPU only."""
import numpy as np
import pytest

import pyoracle as O
from _cases import GEN_CASES, generated, golden, golden_names, host_graph


@pytest.mark.parametrize("name", golden_names())
def test_golden_scc(name):
    c = golden()[name]
    g = host_graph(c)
    lab = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=3)
    assert np.array_equal(O.canon(lab), c["scc"])
    tar, _ = O.tarjan(g.n, g.off, g.E)
    assert np.array_equal(O.canon(tar), c["scc"])


@pytest.mark.parametrize("name", golden_names())
def test_golden_cc(name):
    c = golden()[name]
    s = host_graph(c).symmetrize()
    assert np.array_equal(O.canon(O.cc(s.n, s.off, s.E)), c["cc"])


@pytest.mark.parametrize("name", [n for n in golden_names() if "perm" in golden()[n]])
def test_golden_lelist(name):
    c = golden()[name]
    s = host_graph(c).symmetrize()
    assert np.array_equal(O.lelist_seq(s.n, s.off, s.E, c["perm"]), c["le"])
    assert np.array_equal(O.lelist_par(s.n, s.off, s.E, c["perm"]), c["le"])


@pytest.mark.parametrize("name", golden_names())
def test_golden_reach_bfs(name):
    c = golden()[name]
    g = host_graph(c)
    assert np.array_equal(O.reach_seq(g.n, g.off, g.E, 0), c["reach0"])
    assert np.array_equal(O.bfs_seq(g.n, g.off, g.E, 0), c["bfs0"])
    for local in (False, True):
        assert np.array_equal(O.reach(g.n, g.off, g.E, g.in_off, g.in_E, 0, local=local, tau=4),
                              c["reach0"])


@pytest.mark.parametrize("kind,size,seed", GEN_CASES)
def test_scc_restatement_vs_tarjan(kind, size, seed):
    g = generated(kind, size, seed)
    lab = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=seed)
    tar, _ = O.tarjan(g.n, g.off, g.E)
    assert np.array_equal(O.canon(lab), O.canon(tar))


@pytest.mark.parametrize("kind,size,seed", GEN_CASES[:4])
def test_scc_raw_labels_independent_of_schedule(kind, size, seed):
    """Raw labels depend only on (graph, pivot order, beta): VGC on/off, tau
    and the thread count do not change them (the closure is unique)."""
    g = generated(kind, size, seed)
    a = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=5)
    b = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=5, local_reach=False, local_scc=False,
              nthreads=1)
    c = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=5, tau=3, nthreads=3)
    assert np.array_equal(a, b) and np.array_equal(a, c)
    # another beta changes the batches, never the partition
    d = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=5, beta=2.5)
    assert np.array_equal(O.canon(a), O.canon(d))


def test_scc_label_encoding():
    """Trimmed vertices get 0..|ZEROS|-1 in id order; the rest get pivot labels
    >= |ZEROS| (src/scc.hpp:304-305, 314, 475-476)."""
    g = generated("rmat", 12, 4)
    lab = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=1)
    deg_out = np.diff(g.off)
    deg_in = np.diff(g.in_off)
    zeros = np.nonzero((deg_out == 0) | (deg_in == 0))[0]
    assert np.array_equal(lab[zeros], np.arange(len(zeros), dtype=np.uint64))
    rest = np.setdiff1d(np.arange(g.n), zeros)
    assert (lab[rest] >= len(zeros)).all()


@pytest.mark.parametrize("kind,size,seed", GEN_CASES[:5])
def test_reach_parallel_equals_sequential(kind, size, seed):
    g = generated(kind, size, seed)
    for src in (0, g.n // 2, g.n - 1):
        ref = O.reach_seq(g.n, g.off, g.E, src)
        assert np.array_equal(O.reach(g.n, g.off, g.E, g.in_off, g.in_E, src), ref)
        back = O.reach_seq(g.n, g.in_off, g.in_E, src)
        assert np.array_equal(O.reach(g.n, g.in_off, g.in_E, g.off, g.E, src, local=False), back)


@pytest.mark.parametrize("kind,size,seed", [("rmat", 9, 3), ("grid", 20, 4), ("knn", 400, 5)])
def test_lelist_par_equals_seq(kind, size, seed):
    import psc

    s = generated(kind, size, seed).symmetrize()
    perm = psc.random_permutation(s.n, 4)
    assert np.array_equal(O.lelist_seq(s.n, s.off, s.E, perm),
                          O.lelist_par(s.n, s.off, s.E, perm, beta=1.5))
    assert np.array_equal(O.lelist_seq(s.n, s.off, s.E, perm),
                          O.lelist_par(s.n, s.off, s.E, perm, beta=3.0))


def test_permutation_is_a_bijection_and_matches_library():
    import psc

    for k in (1, 2, 3, 5, 17, 1000, 4097, 65536, 100003):
        p = np.array([O.lib().orc_perm_at(i, k, 9) for i in range(k)], np.uint64)
        assert np.array_equal(np.sort(p), np.arange(k, dtype=np.uint64))
        assert np.array_equal(p.astype(np.uint32), psc.random_permutation(k, 9))


def _lowbias32(x):
    M = 0xFFFFFFFF
    x ^= x >> 16
    x = (x * 0x7FEB352D) & M
    x ^= x >> 15
    x = (x * 0x846CA68B) & M
    return x ^ (x >> 16)


def _splitmix64_mix(x):
    M = (1 << 64) - 1
    x ^= x >> 30
    x = (x * 0xBF58476D1CE4E5B9) & M
    x ^= x >> 27
    x = (x * 0x94D049BB133111EB) & M
    return x ^ (x >> 31)


def test_hash_spec_known_answers():
    """The oracle's hashes are exactly the published lowbias32 and
    SplitMix64 finaliser (restated here in Python)."""
    for x in [0, 1, 2, 3, 1023, 1024, 0xDEADBEEF, 0xFFFFFFFF, 123456789]:
        assert O.lib().orc_hash32_at(x) == _lowbias32(x)
    for x in [0, 1, 2, 1 << 40, 0x9E3779B97F4A7C15, (1 << 64) - 1]:
        assert O.lib().orc_hash64_at(x) == _splitmix64_mix(x)

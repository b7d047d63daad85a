"""The C oracle and the host graph library pinned to the reference's own code.

tests/golden/ref_vectors.npz holds what the reference's headers compute
(compiled unmodified against the ParlayLib-API stand-in, oracle/ref.mk) on the
golden and seeded graphs: raw SCC labels (src/scc.hpp:277-476), REACH sets,
Tarjan, make_directed / make_symmetric (src/graph.hpp:187-245), Connectivity
partitions (src/Connectivity.h:37-119), BFS distances and LE-lists
(src/LeList.hpp:219-328).  These tests hold the oracle's restatement and the
host graph library to them; where the reference build itself is present
(oracle/_ref, built only where the reference checkout is), the live tests
compare on more inputs and parameters."""
import numpy as np
import pytest

import psc
import pyoracle as O
import pyref
from _cases import (REF_LE_SEED, REF_SCC_SEEDS, canon, generated, ref_check, ref_graph,
                    ref_names, ref_vectors, sha)


@pytest.mark.parametrize("name", ref_names())
def test_inputs_reproduce(name):
    """The stored CSR and the seeded generators still give the graphs the
    vectors were computed on."""
    g = ref_graph(name)
    assert g.n == ref_vectors()[name]["n"]
    assert sha(g.off) + sha(g.E) == str(ref_vectors()[name]["input#sha"])


@pytest.mark.parametrize("name", ref_names())
def test_oracle_scc_equals_reference(name):
    c, g = ref_vectors()[name], ref_graph(name)
    for s in REF_SCC_SEEDS:
        ref_check(c, f"scc_s{s}", O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=s))
    ref_check(c, "scc_plain_s1", O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=1,
                                       local_reach=False, local_scc=False))
    t, _ = O.tarjan(g.n, g.off, g.E)
    ref_check(c, "tarjan", canon(t))


@pytest.mark.parametrize("name", ref_names())
def test_oracle_reach_equals_reference(name):
    c, g = ref_vectors()[name], ref_graph(name)
    ref_check(c, "reach_f", O.reach_seq(g.n, g.off, g.E, 0))
    ref_check(c, "reach_b", O.reach_seq(g.n, g.in_off, g.in_E, 0))
    ref_check(c, "reach_f", O.reach(g.n, g.off, g.E, g.in_off, g.in_E, 0))


@pytest.mark.parametrize("name", ref_names())
def test_host_transpose_and_symmetrize_equal_reference(name):
    c, g = ref_vectors()[name], ref_graph(name)
    io, iE = O.transpose(g.n, g.off, g.E)
    ref_check(c, "in_off", io)
    ref_check(c, "in_E", iE)
    h = psc.HostGraph(g.n, g.m, g.off, g.E).with_transpose()  # libpsc_host.so
    ref_check(c, "in_off", h.in_off.astype(np.uint64))
    ref_check(c, "in_E", h.in_E.astype(np.uint32))
    s = g.symmetrize()
    ref_check(c, "sym_off", s.off.astype(np.uint64))
    ref_check(c, "sym_E", s.E.astype(np.uint32))


@pytest.mark.parametrize("name", ref_names())
def test_oracle_cc_bfs_lelist_equal_reference(name):
    c, g = ref_vectors()[name], ref_graph(name)
    s = g.symmetrize()
    ref_check(c, "cc", canon(O.cc(s.n, s.off, s.E)))
    ref_check(c, "bfs", O.bfs_seq(s.n, s.off, s.E, 0))
    if g.n >= 2:
        perm = psc.random_permutation(s.n, REF_LE_SEED)
        ref_check(c, "le", O.lelist_par(s.n, s.off, s.E, perm))
        ref_check(c, "le", O.lelist_seq(s.n, s.off, s.E, perm))


# ------------------------------------------------- live, where oracle/_ref is
live = pytest.mark.skipif(not pyref.available(),
                          reason="oracle/_ref is built only where the reference checkout is present")


@live
@pytest.mark.parametrize("kind,size,seed", [("rmat", 12, 3), ("rmat", 15, 4), ("knn", 30000, 5),
                                            ("grid", 128, 6)])
@pytest.mark.parametrize("params", [dict(), dict(tau=1), dict(tau=64), dict(beta=1.1),
                                    dict(beta=2.0), dict(beta=8.0),
                                    dict(local_reach=False, local_scc=False)])
def test_live_scc(kind, size, seed, params):
    g = generated(kind, size, seed)
    a = pyref.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=seed + 10, **params)
    b = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=seed + 10, **params)
    assert np.array_equal(a, b)


@live
@pytest.mark.parametrize("kind,size,seed", [("rmat", 12, 3), ("knn", 30000, 5), ("grid", 128, 6)])
def test_live_cc_lelist_bfs(kind, size, seed):
    s = generated(kind, size, seed).symmetrize()
    assert np.array_equal(canon(pyref.cc(s.n, s.off, s.E)), canon(O.cc(s.n, s.off, s.E)))
    for pseed in (1, 9):
        perm = psc.random_permutation(s.n, pseed)
        assert np.array_equal(pyref.lelist(s.n, s.off, s.E, perm),
                              O.lelist_par(s.n, s.off, s.E, perm))
    assert np.array_equal(pyref.bfs(s.n, s.off, s.E, 5), O.bfs_seq(s.n, s.off, s.E, 5))


@live
def test_live_reference_oracle_is_the_one_pinned():
    """The committed vectors are what the reference build computes now."""
    c = ref_vectors()["rmat13_s2"]
    g = ref_graph("rmat13_s2")
    ref_check(c, "scc_s7", pyref.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=7))


@live
@pytest.mark.parametrize("kind,size,seed", [("knn", 20000, 3), ("rmat", 14, 2)])
def test_live_reference_ldd_uses_the_same_candidates(kind, size, seed):
    """The reference's LDD (src/ldd.hpp:325-417) over the stand-in's hash32
    draws its centres from the candidates hash32(1024 + i) % n that the
    device LDD offers (tests/test_gpu_cc.py checks the device side), and its
    first candidate is always a centre."""
    s = generated(kind, size, seed).symmetrize()
    n = s.n
    lab, rounds = pyref.ldd(n, s.off, s.E, 0.2)
    cand = np.unique(np.array([O.lib().orc_hash32_at(1024 + i) % n for i in range(1024)],
                              np.uint32))
    centres = np.unique(lab[lab != np.arange(n)])
    assert np.isin(centres, cand).all()
    c0 = O.lib().orc_hash32_at(1024) % n
    assert lab[c0] == c0
    assert rounds >= 1

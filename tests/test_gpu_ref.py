"""GPU parity against the reference's own code.

Every output of the CUDA library through the C ABI is compared bit for bit
with what the reference's headers compute on the same input
(tests/golden/ref_vectors.npz, written by tests/golden/make_ref_golden.py from
the reference build of oracle/ref.mk): raw SCC labels (src/scc.hpp:277-476)
with VGC on and off, REACH sets (src/reach.hpp:208-243), the device transpose
(make_directed, src/graph.hpp:222-245), Connectivity partitions
(src/Connectivity.h:37-119), BFS distances (src/bfs.hpp:200-238) and LE-lists
(src/LeList.hpp:219-328)."""
import numpy as np
import pytest

import psc
from _cases import REF_LE_SEED, REF_SCC_SEEDS, canon, ref_check, ref_graph, ref_names, ref_vectors

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _dev(cuda_device):
    return cuda_device


@pytest.mark.parametrize("name", ref_names())
def test_scc_equals_reference(name):
    c, g = ref_vectors()[name], ref_graph(name)
    with psc.DeviceGraph(g) as dg:
        for s in REF_SCC_SEEDS:
            ref_check(c, f"scc_s{s}", dg.scc(psc.default_params(seed=s)))
        ref_check(c, "scc_plain_s1", dg.scc(psc.default_params(seed=1, local_reach=0,
                                                               local_scc=0)))
        ref_check(c, "reach_f", dg.reach(0))
        ref_check(c, "reach_b", dg.reach(0, backward=True))
        ref_check(c, "reach_f", dg.reach(0, local=False))


@pytest.mark.parametrize("name", ref_names())
def test_device_transpose_equals_reference(name):
    c, g = ref_vectors()[name], ref_graph(name)
    with psc.DeviceGraph.directed(g.off, g.E) as dg:
        io, iE = dg.transpose()
        ref_check(c, "in_off", io)
        ref_check(c, "in_E", iE)
        ref_check(c, "scc_s1", dg.scc(psc.default_params(seed=1)))


@pytest.mark.parametrize("name", ref_names())
def test_cc_bfs_lelist_equal_reference(name):
    c, g = ref_vectors()[name], ref_graph(name)
    s = g.symmetrize()
    with psc.DeviceGraph(s) as dg:
        ref_check(c, "cc", canon(dg.cc()))
        ref_check(c, "bfs", dg.bfs(0))
        if g.n >= 2:
            ref_check(c, "le", dg.lelist(psc.random_permutation(s.n, REF_LE_SEED)))


@pytest.mark.parametrize("name", ref_names())
def test_device_symmetrize_equals_reference(name):
    c, g = ref_vectors()[name], ref_graph(name)
    with psc.DeviceGraph.symmetrized(g.off, g.E) as dg:
        so, sE = dg.download()
        ref_check(c, "sym_off", so)
        ref_check(c, "sym_E", sE)
        ref_check(c, "cc", canon(dg.cc()))

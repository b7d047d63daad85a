"""GPU tests of the request server: results in a mixed, continuously batched
stream equal the solo results (SCC raw labels bit for bit, connectivity
partitions), admission respects the device-memory budget, and concurrent
submitters are served."""
import threading

import numpy as np
import pytest

import psc
import pyoracle as O
from psc.server import CC, SCC

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _dev(cuda_device):
    return cuda_device


def stream(count, seed0=500, lo=4, hi=12):
    """Seeded request stream: (graph, kind, seed); every fifth one a
    connectivity request on the symmetrised graph."""
    out = []
    for k in range(count):
        g = psc.batch_member(k, seed0, lo, hi)
        if k % 5 == 4:
            out.append((g.symmetrize(), CC, 0))
        else:
            out.append((g, SCC, 1000 + k))
    return out


def check_result(g, kind, seed, lab):
    if kind == SCC:
        ref = O.scc(g.n, g.off, g.E, g.in_off, g.in_E, seed=seed)
        assert np.array_equal(lab, ref)
    else:
        assert (lab < g.n).all()
        assert np.array_equal(O.canon(lab), O.canon(O.cc(g.n, g.off, g.E)))


def test_server_mixed_equals_solo():
    reqs = stream(40)
    with psc.Server(workers=3, max_batch=8) as srv:
        # every other SCC request brings its host transpose
        ids = [srv.submit(g, kind, seed, with_transpose=(k % 2 == 0))
               for k, (g, kind, seed) in enumerate(reqs)]
        mixed = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert st.completed == len(reqs) and st.failed == 0
    assert st.batches < len(reqs), "requests were batched"
    for (g, kind, seed), (lab, info) in zip(reqs, mixed):
        assert info.status == 0 and info.batch_size >= 1
        assert 0 <= info.queue_ms <= info.latency_ms
        check_result(g, kind, seed, lab)
    # the same requests alone, one per batch
    with psc.Server(workers=1, max_batch=1) as solo:
        for (g, kind, seed), (lab, _) in list(zip(reqs, mixed))[::3]:
            alone, info = solo.wait(solo.submit(g, kind, seed))
            assert info.batch_size == 1
            if kind == SCC:
                assert np.array_equal(alone, lab)
            else:
                assert np.array_equal(O.canon(alone), O.canon(lab))


def test_server_matches_plain_calls():
    reqs = stream(12, seed0=77, lo=8, hi=13)
    with psc.Server(workers=2) as srv:
        ids = [srv.submit(g, kind, seed) for g, kind, seed in reqs]
        res = [srv.wait(i)[0] for i in ids]
    for (g, kind, seed), lab in zip(reqs, res):
        with psc.DeviceGraph(g) as dg:
            if kind == SCC:
                assert np.array_equal(dg.scc(psc.default_params(seed=seed)), lab)
            else:
                assert np.array_equal(O.canon(dg.cc()), O.canon(lab))


def test_server_budget_admission():
    reqs = stream(24, seed0=9, lo=9, hi=11)
    # room for about two requests at a time
    big = max(16 * (g.n + 1) + 22 * g.m + 168 * g.n for g, _, _ in reqs)
    budget = 2 * big + 1
    with psc.Server(workers=4, max_batch=64, hbm_budget=budget) as srv:
        ids = [srv.submit(g, kind, seed) for g, kind, seed in reqs]
        res = [srv.wait(i) for i in ids]
        st = srv.stats()
        with pytest.raises(psc.PscError):
            g = psc.HostGraph.rmat(14, 16 << 14, seed=1)
            srv.submit(g, SCC, 1)  # larger than the whole budget
        st2 = srv.stats()
    assert st.peak_bytes <= budget
    assert st2.rejected == 1
    for (g, kind, seed), (lab, info) in zip(reqs, res):
        check_result(g, kind, seed, lab)


def test_server_concurrent_submitters():
    reqs = stream(30, seed0=3, lo=5, hi=11)
    results = {}
    with psc.Server(workers=4, max_batch=16) as srv:
        def client(part):
            for k in part:
                g, kind, seed = reqs[k]
                results[k] = srv.wait(srv.submit(g, kind, seed))[0]

        threads = [threading.Thread(target=client, args=(list(range(t, 30, 3)),)) for t in range(3)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        srv.drain()
        assert srv.stats().queued == 0
    for k, (g, kind, seed) in enumerate(reqs):
        check_result(g, kind, seed, results[k])


def test_server_rejects_bad_requests():
    with psc.Server(workers=1) as srv:
        g = psc.HostGraph.from_edges(3, [0, 1], [1, 2])
        with pytest.raises(psc.PscError):
            srv.submit(g, 7, 1)  # unknown kind
        with pytest.raises(psc.PscError):
            srv.wait(12345)      # unknown id
        lab, _ = srv.wait(srv.submit(g, SCC, 1))
        assert len(np.unique(lab)) == 3


def test_server_edge_cap_splits_batches():
    """max_batch_edges: a batch holds at most that many edges (a larger
    request goes alone), and results stay those of solo solves."""
    reqs = stream(24, seed0=700)
    cap = max(g.m for g, _, _ in reqs) // 2
    with psc.Server(workers=2, max_batch_edges=cap) as srv:
        ids = [srv.submit(g, kind, seed, with_transpose=(k % 2 == 0))
               for k, (g, kind, seed) in enumerate(reqs)]
        infos = []
        for rid, (g, kind, seed) in zip(ids, reqs):
            lab, info = srv.wait(rid)
            assert info.status == 0
            check_result(g, kind, seed, lab)
            infos.append((info.batch_size, g.m))
    # a request above the cap was solved alone
    assert all(bs == 1 for bs, m in infos if m > cap)
    assert psc.server_config().max_batch_edges == 1 << 28

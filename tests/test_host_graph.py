"""Host graph construction (libpsc_host.so): generator pins, CSR invariants,
transpose / symmetrise semantics and the GBBS .bin format.  CPU only."""
import numpy as np
import pytest

import psc
import pyoracle as O
from _cases import golden


def check_csr(g, allow_self=False):
    assert g.off[0] == 0 and g.off[-1] == g.m and len(g.off) == g.n + 1
    assert (np.diff(g.off.astype(np.int64)) >= 0).all()
    for u in range(min(g.n, 2000)):
        a = g.E[g.off[u]:g.off[u + 1]]
        assert (np.diff(a.astype(np.int64)) > 0).all(), "adjacency sorted and unique"
        if not allow_self:
            assert u not in a


@pytest.mark.parametrize("name,make", [
    ("gen_rmat8", lambda: psc.HostGraph.rmat(8, 1 << 11, seed=11)),
    ("gen_knn300", lambda: psc.HostGraph.knn(300, 5, seed=12)),
    ("gen_grid12", lambda: psc.HostGraph.grid(12, 12, 0.3, seed=13)),
])
def test_generators_are_pinned(name, make):
    c = golden()[name]
    g = make()
    assert g.n == c["n"]
    assert np.array_equal(g.off, c["off"]) and np.array_equal(g.E, c["E"])


def test_rmat_shape():
    g = psc.HostGraph.rmat(14, 1 << 18, seed=1)
    assert g.n == 1 << 14 and 0 < g.m <= 1 << 18
    check_csr(g)
    # skewed: the top 1% of vertices hold well over 1% of the edges
    deg = np.sort(np.diff(g.off))[::-1]
    assert deg[: g.n // 100].sum() > 0.1 * g.m


def test_knn_is_exact():
    g = psc.HostGraph.knn(700, 5, seed=3)
    check_csr(g)
    assert (np.diff(g.off) == 5).all()
    # brute force over the same points (the generator's SplitMix64 stream)
    M = (1 << 64) - 1

    def mix(x):
        x ^= x >> 30
        x = (x * 0xBF58476D1CE4E5B9) & M
        x ^= x >> 27
        x = (x * 0x94D049BB133111EB) & M
        return x ^ (x >> 31)

    def unit(seed, i):
        return (mix((mix(seed) + (i + 1) * 0x9E3779B97F4A7C15) & M) >> 11) * (1.0 / 9007199254740992.0)

    X = np.array([unit(3, 2 * i) for i in range(700)])
    Y = np.array([unit(3, 2 * i + 1) for i in range(700)])
    d2 = (X[:, None] - X[None, :]) ** 2 + (Y[:, None] - Y[None, :]) ** 2
    np.fill_diagonal(d2, np.inf)
    for i in range(700):
        order = np.lexsort((np.arange(700), d2[i]))[:5]
        assert np.array_equal(np.sort(order), g.E[g.off[i]:g.off[i + 1]])


def test_grid_edge_counts():
    rows, cols = 40, 50
    g = psc.HostGraph.grid(rows, cols, 0.3, seed=7)
    check_csr(g)
    lattice = rows * (cols - 1) + (rows - 1) * cols
    s = g.symmetrize()
    assert s.m == 2 * lattice  # every lattice edge present in >= 1 direction
    both = g.m - lattice
    assert 0.2 * lattice < both < 0.4 * lattice
    src, dst = g.edge_list()
    dr = np.abs(src.astype(np.int64) // cols - dst.astype(np.int64) // cols)
    dc = np.abs(src.astype(np.int64) % cols - dst.astype(np.int64) % cols)
    assert ((dr + dc) == 1).all()


def test_from_edges_dedup_and_selfloops():
    g = psc.HostGraph.from_edges(5, [0, 0, 1, 1, 2, 4], [1, 1, 1, 2, 0, 4], drop_self=True)
    assert g.m == 3
    assert g.E.tolist() == [1, 2, 0]
    g2 = psc.HostGraph.from_edges(5, [0, 0, 1, 4], [1, 1, 1, 4], drop_self=False)
    assert g2.m == 3


def test_transpose_matches_oracle():
    g = psc.HostGraph.rmat(12, 1 << 16, seed=9)
    io, iE = O.transpose(g.n, g.off, g.E)
    assert np.array_equal(io, g.in_off) and np.array_equal(iE, g.in_E)


def test_symmetrize_semantics():
    g = psc.HostGraph.from_edges(6, [0, 1, 2, 3, 3, 5], [1, 0, 3, 2, 3, 1], drop_self=False)
    s = g.symmetrize()
    pairs = set()
    src, dst = g.edge_list()
    for a, b in zip(src.tolist(), dst.tolist()):
        if a != b:
            pairs.add((a, b))
            pairs.add((b, a))
    ss, sd = s.edge_list()
    assert sorted(zip(ss.tolist(), sd.tolist())) == sorted(pairs)
    assert s.symmetric and s.in_off is s.off


def test_bin_round_trip(tmp_path):
    g = psc.HostGraph.rmat(10, 1 << 13, seed=2)
    p = tmp_path / "g.bin"
    g.write_bin(p)
    raw = np.fromfile(p, dtype=np.uint64, count=3)
    assert raw[0] == g.n and raw[1] == g.m and raw[2] == (g.n + 1) * 8 + g.m * 4 + 24
    h = psc.HostGraph.read_bin(p)
    assert np.array_equal(h.off, g.off) and np.array_equal(h.E, g.E)
    assert np.array_equal(h.in_off, g.in_off) and np.array_equal(h.in_E, g.in_E)
    # two CSRs back to back = the -large format (src/graph.hpp:279-315)
    q = tmp_path / "g_large.bin"
    t = psc.HostGraph(g.n, g.m, g.in_off, g.in_E)
    t2 = tmp_path / "t.bin"
    t.write_bin(t2)
    q.write_bytes(p.read_bytes() + t2.read_bytes())
    L = psc.HostGraph.read_bin(q, large=True)
    assert np.array_equal(L.in_off, g.in_off) and np.array_equal(L.in_E, g.in_E)
    bad = tmp_path / "bad.bin"
    bad.write_bytes(p.read_bytes() + b"x")
    with pytest.raises(RuntimeError):
        psc.HostGraph.read_bin(bad)
    with pytest.raises(RuntimeError):
        psc.HostGraph.read_bin(tmp_path / "missing.bin")


def test_adj_reader(tmp_path):
    g = psc.HostGraph.rmat(8, 1 << 10, seed=5)
    p = tmp_path / "g.adj"
    lines = ["AdjacencyGraph", str(g.n), str(g.m)] + [str(x) for x in g.off[:-1]] + \
        [str(x) for x in g.E]
    p.write_text("\n".join(lines) + "\n")
    lib = psc.host()
    h = lib.psc_hgraph_read_adj(str(p).encode())
    assert h
    r = psc.HostGraph._adopt(h, "adj")
    assert np.array_equal(r.off, g.off) and np.array_equal(r.E, g.E)
    (tmp_path / "bad.adj").write_text("AdjacencyGraph\n5\n")
    assert not lib.psc_hgraph_read_adj(str(tmp_path / "bad.adj").encode())


def test_batch_member_spec():
    specs = [psc.batch_member_spec(k, 1000, 8, 18) for k in range(400)]
    assert [s[0] for s in specs[:4]] == ["rmat", "knn", "rmat", "knn"]
    for kind, size in specs:
        if kind == "rmat":
            assert 8 <= size <= 18
        else:
            assert 256 <= size < 1 << 18
    # log-uniform: about half the kNN members lie below 2^13
    knn = np.array([s for k, s in specs if k == "knn"])
    assert 0.35 < np.mean(knn < 1 << 13) < 0.65
    assert specs == [psc.batch_member_spec(k, 1000, 8, 18) for k in range(400)]
    with pytest.raises(ValueError):
        psc.batch_member_spec(0, 1, 5, 40)


def test_batch_workload_is_packed_members():
    count = 9
    u, vb = psc.batch_workload(count, 11, 4, 10)
    members = [psc.batch_member(k, 11, 4, 10) for k in range(count)]
    assert len(vb) == count + 1 and vb[0] == 0 and vb[-1] == u.n
    for k, m in enumerate(members):
        kind, size = psc.batch_member_spec(k, 11, 4, 10)
        assert m.n == (1 << size if kind == "rmat" else size)
        assert int(vb[k + 1] - vb[k]) == m.n
    p, pvb = psc.HostGraph.pack(members)
    assert np.array_equal(pvb, vb)
    for f in ("off", "E", "in_off", "in_E"):
        assert np.array_equal(getattr(u, f), getattr(p, f)), f
    # no edge leaves its member's id range
    src, dst = u.edge_list()
    gs = np.searchsorted(vb, src, side="right") - 1
    assert ((dst >= vb[gs]) & (dst < vb[gs + 1])).all()
    # transpose of the union = union of the transposes
    t_off, t_E = O.transpose(u.n, u.off, u.E)
    assert np.array_equal(t_off, u.in_off) and np.array_equal(t_E, u.in_E)


def test_pack_symmetric_and_single():
    a = psc.HostGraph.rmat(6, 300, seed=1).symmetrize()
    b = psc.HostGraph.knn(50, 5, seed=2).symmetrize()
    s, vb = psc.HostGraph.pack([a, b])
    assert s.symmetric and s.in_E is s.E
    assert list(vb) == [0, a.n, a.n + b.n]
    one, vb1 = psc.HostGraph.pack([a])
    assert np.array_equal(one.E, a.E) and list(vb1) == [0, a.n]
    d, _ = psc.HostGraph.pack([a, psc.HostGraph.rmat(5, 100, seed=3)])
    assert not d.symmetric and d.in_off is not None

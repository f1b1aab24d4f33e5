"""Seeded structured graphs that stress the traversal engine's edge cases,
each checked against the oracle on the CSR, PMA and packed CSR containers:
BFS levels and min-id parents under every direction policy (including the
learned one), CC and BFS-CC labels, triangle counts, 64-source BFS levels and
PageRank (FP32-Kahan within 1e-6 L1 of FP64, FP64 within 1e-12).

  path      a path of 3000 vertices: 3000 BFS rounds, every one tiny
  star      one hub adjacent to every other vertex (a degree of n - 1 in the
            first round), plus a second small star
  cliques   disjoint cliques of sizes 1-90 (many components, triangle-rich)
  tree      a random recursive tree (deep and bushy)
  lollipop  a 200-clique with a 2000-vertex tail
  sparse    a random graph with most vertices isolated, n not a multiple of 32
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PR_TOL = 1e-6


def _graphs(O):
    rng = np.random.default_rng(131)
    out = {}
    n = 3000
    out["path"] = (n, np.arange(n - 1), np.arange(1, n))
    n = 5003
    hub = np.zeros(n - 1, np.int64)
    leaves = np.arange(1, n)
    s2 = np.full(40, 4000)
    d2 = np.arange(4001, 4041)
    out["star"] = (n, np.concatenate([hub, s2]), np.concatenate([leaves, d2]))
    src, dst, base = [], [], 0
    for size in rng.integers(1, 91, 40):
        a, b = np.triu_indices(int(size), 1)
        src.append(a + base)
        dst.append(b + base)
        base += int(size)
    out["cliques"] = (base + 7, np.concatenate(src), np.concatenate(dst))
    n = 20000
    par = np.array([rng.integers(0, v) for v in range(1, n)])
    out["tree"] = (n, par, np.arange(1, n))
    a, b = np.triu_indices(200, 1)
    tail = np.arange(200, 2200)
    out["lollipop"] = (2200, np.concatenate([a, tail - 1]), np.concatenate([b, tail]))
    n = 100003
    p = rng.integers(0, 30000, size=(20000, 2))
    out["sparse"] = (n, p[:, 0], p[:, 1] * 3)
    return out


@pytest.mark.parametrize("name", ["path", "star", "cliques", "tree", "lollipop", "sparse"])
def test_structured_graphs(ctx, oracle_mod, name):
    import torch

    import byo_gb300 as byo
    O = oracle_mod
    n, s, d = _graphs(O)[name]
    off, nb = O.build_csr(n, np.asarray(s, np.uint32), np.asarray(d, np.uint32))
    deg = np.diff(off.astype(np.int64))
    rng = np.random.default_rng(132)
    srcs = [0, int(np.argmax(deg)), int(rng.integers(0, n)), n - 1]
    olab = O.cc(off, nb)
    otc = O.triangle_count(off, nb)
    op, oit, _ = O.pagerank(off, nb, 1e-6, 60)
    multi = rng.integers(0, n, 64).astype(np.uint32)
    for container in ("csr", "pma", "pcsr"):
        G = byo.Graph.from_csr(ctx, off, nb, container=container)
        for src in srcs:
            opar, olev = O.bfs(off, nb, src)
            for pol in (0, 1, 2, 3, 4, 5):
                par, lev = byo.BFS(G, src, policy=pol, levels=True)
                assert np.array_equal(lev, olev), (container, src, pol, "levels")
                assert np.array_equal(par, opar), (container, src, pol, "parents")
        assert np.array_equal(byo.SimpleUnionAsync(G), olab), container
        assert np.array_equal(byo.bfs_cc(G), olab), container
        assert byo.Triangle_degree_ordering(G) == otc, container
        lv = byo.BFS_multi(G, multi)
        for j in range(0, 64, 9):
            assert np.array_equal(lv[j], O.bfs(off, nb, int(multi[j]))[1]), (container, j)
        p, it, _ = byo.PageRank(G, 1e-6, 60, info=True)
        assert abs(it - oit) <= 1, container
        if it == oit:
            assert float(np.abs(p - op).sum()) <= PR_TOL, container
        p64, it64, _ = byo.PageRank(G, 1e-6, 60, precision=1, info=True)
        assert it64 == oit and float(np.abs(p64 - op).sum()) <= 1e-12, container
        G.close()


def test_cc_labels_stable_over_repeats(ctx, oracle_mod):
    """Connectivity on a graph of thousands of small components, repeated:
    the labels must be the component minima on every run (a compress pass
    whose finds halved paths once left one vertex pointing at a non-root
    ancestor in about one run of 40)."""
    import byo_gb300 as byo
    O = oracle_mod
    n, s, d = _graphs(O)["sparse"]
    off, nb = O.build_csr(n, np.asarray(s, np.uint32), np.asarray(d, np.uint32))
    olab = O.cc(off, nb)
    for container in ("csr", "pcsr"):
        G = byo.Graph.from_csr(ctx, off, nb, container=container)
        for _ in range(150):
            assert np.array_equal(byo.SimpleUnionAsync(G), olab), container
        for _ in range(20):
            assert np.array_equal(byo.bfs_cc(G), olab), container
        G.close()


@pytest.mark.parametrize("name", ["sparse", "star", "rmat"])
def test_traversals_repeat_identically(ctx, oracle_mod, name):
    """Races show up as rare differences between runs: BFS under every
    policy, 64-source BFS and PageRank repeated on the same graph must give
    the oracle's levels and min-id parents every time, and PageRank the same
    bits every time (its sums have a fixed order)."""
    import byo_gb300 as byo
    O = oracle_mod
    if name == "rmat":
        s, d = O.rmat_edges(141, 15, 1 << 19)
        n = 1 << 15
    else:
        n, s, d = _graphs(O)[name]
    off, nb = O.build_csr(n, np.asarray(s, np.uint32), np.asarray(d, np.uint32))
    deg = np.diff(off.astype(np.int64))
    src = int(np.argmax(deg))
    opar, olev = O.bfs(off, nb, src)
    multi = np.random.default_rng(142).integers(0, n, 64).astype(np.uint32)
    exp_multi = [O.bfs(off, nb, int(x))[1] for x in multi[:8]]
    for container in ("csr", "pma"):
        G = byo.Graph.from_csr(ctx, off, nb, container=container)
        for _ in range(12):
            for pol in (0, 1, 2, 3, 4, 5):
                par, lev = byo.BFS(G, src, policy=pol, levels=True)
                assert np.array_equal(lev, olev) and np.array_equal(par, opar), (container, pol)
        for _ in range(6):
            lv = byo.BFS_multi(G, multi)
            for j in range(8):
                assert np.array_equal(lv[j], exp_multi[j]), (container, j)
        p0 = byo.PageRank(G, 1e-6, 20)
        for _ in range(5):
            assert np.array_equal(byo.PageRank(G, 1e-6, 20), p0), container
        G.close()


def _remote(n, rng):
    """Test_Map_Remote arrays of widths 0 (a bit vector), 4 and 16 bytes."""
    bits = rng.integers(0, 2, size=n).astype(bool)
    packed = np.concatenate([np.packbits(bits, bitorder="little"),
                             np.zeros((-((n + 7) // 8)) % 8, np.uint8)]).view(np.uint64)
    wide = np.full((n, 2), 5, np.uint64)  # the padding word is not read
    wide[:, 0] = rng.integers(0, 1 << 40, size=n)
    return {0: packed, 4: rng.integers(0, 1 << 31, size=n).astype(np.uint32), 16: wide}


@pytest.mark.parametrize("name", ["path", "star", "cliques", "tree", "lollipop", "sparse"])
def test_structured_delta_map_bytepd(ctx, oracle_mod, name):
    """PageRankDelta (the oracle's round count, L1 <= 1e-6), Test_Map and
    Test_Map_Remote on every container (the PMA's gaps, the packed CSR's
    sentinel slots and the vector of runs' slack all read as no edge), and
    the byte-PD encoder (byte-identical) and decoder at block sizes 1000, 7
    and 1 on the structured graphs."""
    import byo_gb300 as byo
    O = oracle_mod
    n, s, d = _graphs(O)[name]
    off, nb = O.build_csr(n, np.asarray(s, np.uint32), np.asarray(d, np.uint32))
    rng = np.random.default_rng(134)
    od, orr, _ = O.pagerank_delta(off, nb, 1e-7, 1e-3, 100)
    remote = _remote(n, rng)
    exp_remote = {w: O.map_remote(off, nb, a, w) for w, a in remote.items()}
    exp_map = O.map_sum(off, nb)
    for container in ("csr", "pma", "pcsr", "vos"):
        G = byo.Graph.from_csr(ctx, off, nb, container=container)
        p, r, _ = byo.PageRankDelta(G, 1e-7, 1e-3, 100, info=True)
        assert r == orr and float(np.abs(p - od).sum()) <= 1e-6, container
        assert byo.Test_Map(G) == exp_map, container
        for w, a in remote.items():
            assert byo.Test_Map_Remote(G, a, w) == exp_remote[w], (container, w)
        G.close()
    G = byo.Graph.from_csr(ctx, off, nb)
    for P in (1000, 7, 1):
        obo, odg, odata = O.bytepd_encode(off, nb, P)
        bo, dg, data = G.to_bytepd(P)
        assert np.array_equal(bo, obo) and np.array_equal(dg, odg) and bytes(data) == bytes(odata), P
        H = byo.Graph.from_bytepd(ctx, obo, odg, odata, block=P, container="pcsr")
        o2, n2 = H.export_csr()
        assert np.array_equal(o2, off) and np.array_equal(n2, nb), P
        H.close()
    G.close()


def _bulk_ops(O, gs):
    """(graph, [(insert?, keys)]) pairs of whole-structure updates; each
    sequence ends on a symmetric graph (BFS and CC follow out-edges)."""
    out = []
    n, _, _ = gs["star"]
    hub = O.keys_from_pairs(np.zeros(n - 1, np.int64), np.arange(1, n))
    out.append(("star", [(False, hub), (True, hub[: n // 2]), (True, hub)]))
    cut = np.arange(0, 2999, 10)
    cuts = O.keys_from_pairs(cut, cut + 1)
    out.append(("path", [(False, cuts), (True, cuts[::2]), (True, cuts)]))
    a, b = np.triu_indices(90, 1)
    big = O.keys_from_pairs(a + 500, b + 500)  # overlaps cliques from id 500 on
    out.append(("cliques", [(True, big), (False, big), (True, O.keys_from_pairs(a[::3] + 500, b[::3] + 500))]))
    a, b = np.triu_indices(150, 1)
    fresh = O.keys_from_pairs(a + 95000, b + 95000)  # ids past every edge so far
    out.append(("sparse", [(True, fresh), (False, fresh[: len(fresh) // 2]), (False, fresh)]))
    tail = np.arange(200, 2200)
    out.append(("lollipop", [(False, O.keys_from_pairs(tail - 1, tail)),
                             (True, O.keys_from_pairs(np.zeros(2000, np.int64), tail))]))
    return out


@pytest.mark.parametrize("container", ["pma", "pcsr", "vos"])
def test_structured_bulk_updates(ctx, oracle_mod, container):
    """Whole-structure updates: the star's hub loses every edge (one vertex's
    run across many leaves), regains half, then all; every tenth edge of the
    path is cut and rejoined; a 90-clique is laid over the cliques and taken
    off; a 150-clique appears among ids that had no edges and goes in two
    steps; the lollipop's tail becomes a second star.  The changed count,
    contents and degrees after every batch, BFS and CC after each graph, all
    against the oracle."""
    import byo_gb300 as byo
    O = oracle_mod
    gs = _graphs(O)
    for name, ops in _bulk_ops(O, gs):
        n, s, d = gs[name]
        off, nb = O.build_csr(n, np.asarray(s, np.uint32), np.asarray(d, np.uint32))
        G = byo.Graph.from_csr(ctx, off, nb, container=container)
        st = O.Store(off, nb)
        rng = np.random.default_rng(135)
        for i, (ins, keys) in enumerate(ops):
            k = keys.copy()
            rng.shuffle(k)
            if ins:
                assert G.insert_batch(k) == st.insert_batch(k), (name, i)
            else:
                assert G.remove_batch(k) == st.remove_batch(k), (name, i)
            ro, rn = st.export_csr()
            go, gn = G.export_csr()
            assert np.array_equal(go, ro) and np.array_equal(gn, rn), (name, i)
            assert np.array_equal(G.degrees(), np.diff(ro).astype(np.uint32)), (name, i)
        for src in (0, int(np.argmax(np.diff(ro)))):
            opar, olev = O.bfs(ro, rn, src)
            par, lev = byo.BFS(G, src, levels=True)
            assert np.array_equal(lev, olev) and np.array_equal(par, opar), (name, src)
        assert np.array_equal(byo.SimpleUnionAsync(G), O.cc(ro, rn)), name
        G.close()

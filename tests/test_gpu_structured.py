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

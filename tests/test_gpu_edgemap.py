"""The edgeMap / vertexSubset API with the reference's own functors, driven by
the reference's own loops, against the oracle.

  BFS-CC        bfs_cc::CC (benchmarks/Connectivity/BFSCC/Connectivity.h:52-88):
                a host loop over the vertices, a BFS_ComponentLabel_F edgeMap
                traversal from each one not yet labelled (flags
                sparse_blocked | dense_parallel), labels bit-exact.
  PageRank_edgeMap (benchmarks/PageRank/PageRank.h:80-123): edgeMap(PR_F,
                threshold 0, no_output) + vertexMap(PR_Vertex_F) + reset and
                swap; FP64 results bit-exact against the FP64 oracle.
  PageRankDelta (PageRank.h:232-398): PR_Delta_F through edgeMap (dense above
                n/5 members, else threshold M/2) and vertexFilter with the
                first-round and later vertex functions; L1 <= 1e-6 against the
                oracle with the same round count.
Also: vertexSubset from a device bitmap and BitArray(n, true), vertexFilter's
members, every edgeMap direction (sparse, blocked, dense, dense-forward) on a
graph with hubs (dense runs longer than a lane's share), through the C ABI.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

def _on(ctx):
    """torch work on the library's stream, so it is ordered with the library's."""
    import torch
    return torch.cuda.stream(torch.cuda.ExternalStream(ctx.stream))


def _graph(ctx, O, container="csr"):
    """Three RMAT components of different sizes plus isolated vertices."""
    import byo_gb300 as byo
    parts, base = [], 0
    for seed, lg, draws in ((5, 11, 1 << 15), (6, 9, 1 << 12), (7, 6, 300)):
        s, d = O.rmat_edges(seed, lg, draws)
        parts.append((s.astype(np.int64) + base, d.astype(np.int64) + base))
        base += 1 << lg
    n = base + 37  # 37 isolated vertices at the end
    s = np.concatenate([p[0] for p in parts]).astype(np.uint32)
    d = np.concatenate([p[1] for p in parts]).astype(np.uint32)
    off, nb = O.build_csr(n, s, d)
    return byo.Graph.from_csr(ctx, off, nb, container=container), off, nb


def _bfs_cc_via_edgemap(byo, G, torch, flags):
    from byo_gb300 import _abi
    n = G.N()
    deg = G.degrees()
    parents = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    i = 0
    while i < n:
        if deg[i] > 0:  # BFS_ComponentLabel: only sources with an edge start a traversal
            parents[i] = i
            F = byo.vertexSubset(G, i)
            f = byo.BFS_ComponentLabel_F(G, parents, i)
            while not F.isEmpty():
                out = byo.edgeMap(G, F, f, -1, flags)
                F.close()
                F = out
            F.close()
            f.close()
        host = parents.cpu().numpy().view(np.uint32)
        nxt = np.nonzero(host[i + 1:] == _abi.NONE)[0]
        i = i + 1 + int(nxt[0]) if len(nxt) else n
    lab = parents.cpu().numpy().view(np.uint32).copy()
    # unreached (edgeless) vertices keep UINT_E_MAX in the reference; its
    # documented mapping sends them to themselves
    none = lab == _abi.NONE
    lab[none] = np.nonzero(none)[0]
    return lab


@pytest.mark.parametrize("container", ["csr", "pma", "pcsr"])
def test_bfs_cc_as_reference_loop(ctx, oracle_mod, container):
    """On every container: edgeMap reads the container's own view (the PMA's
    and the packed CSR's gaps, the packed CSR's vertex sentinels)."""
    import torch

    import byo_gb300 as byo
    from byo_gb300 import _abi
    O = oracle_mod
    G, off, nb = _graph(ctx, O, container)
    exp = O.cc(off, nb)
    with _on(ctx):
        _bfs_cc_flags(byo, G, torch, exp)
    assert np.array_equal(byo.bfs_cc(G), exp)
    G.close()


def _bfs_cc_flags(byo, G, torch, exp):
    from byo_gb300 import _abi
    for flags in (_abi.FL_SPARSE_BLOCKED | _abi.FL_DENSE_PARALLEL, 0, _abi.FL_DENSE_ONLY, _abi.FL_NO_DENSE,
                  _abi.FL_DENSE_FORWARD):
        lab = _bfs_cc_via_edgemap(byo, G, torch, flags)
        assert np.array_equal(lab, exp), flags


@pytest.mark.parametrize("container", ["csr", "pma", "pcsr"])
def test_pagerank_edgemap_as_reference_loop(ctx, oracle_mod, container):
    import torch

    import byo_gb300 as byo
    from byo_gb300 import _abi
    O = oracle_mod
    s, d = O.rmat_edges(9, 14, 1 << 18)
    off, nb = O.build_csr(1 << 14, s, d)
    G = byo.Graph.from_csr(ctx, off, nb, container=container)
    with _on(ctx):
        _pr_edgemap_loop(byo, G, torch, O, off, nb)
    # the library's own PageRank_edgeMap runs the same loop, with the stop rule
    p, it, l1 = byo.PageRank_edgeMap(G, 1e-6, 100, info=True)
    op, oit, ol1 = O.pagerank(off, nb, 1e-6, 100)
    assert it == oit and l1 == ol1
    assert np.array_equal(p, op)
    G.close()


def _pr_edgemap_loop(byo, G, torch, O, off, nb):
    from byo_gb300 import _abi
    n = G.N()
    p_curr = torch.full((n,), 1.0 / n, dtype=torch.float64, device="cuda")
    p_next = torch.zeros(n, dtype=torch.float64, device="cuda")
    Frontier = byo.vertexSubset.all(G)
    assert Frontier.size() == n and Frontier.isDense
    iters = 20
    for it in range(iters):
        f = byo.PR_F(G, p_curr, p_next)
        out = byo.edgeMap(G, Frontier, f, 0, _abi.FL_NO_OUTPUT)
        assert out.size() == 0
        out.close()
        f.close()
        byo.vertexMap(Frontier, _abi.VOP_PR_UPDATE, a=p_next, damping=0.85)
        if it == iters - 1:
            break
        byo.vertexMap(Frontier, _abi.VOP_ZERO, a=p_curr)
        p_curr, p_next = p_next, p_curr
    op, oit, _ = O.pagerank(off, nb, 0.0, iters)
    assert oit == iters
    got = p_next.cpu().numpy()
    assert np.array_equal(got, op), "max abs diff %g" % np.abs(got - op).max()
    Frontier.close()


def test_pagerank_delta_as_reference_loop(ctx, oracle_mod):
    import torch

    import byo_gb300 as byo
    from byo_gb300 import _abi
    O = oracle_mod
    s, d = O.rmat_edges(12, 13, 1 << 17)
    off, nb = O.build_csr(1 << 13, s, d)
    G = byo.Graph.from_csr(ctx, off, nb)
    with _on(ctx):
        _pr_delta_loop(byo, G, torch, O, off, nb)
    G.close()


def _pr_delta_loop(byo, G, torch, O, off, nb):
    from byo_gb300 import _abi
    n, m = G.N(), G.M()
    deg = torch.from_numpy(G.degrees().astype(np.float64)).cuda()
    eps, local_eps, max_iters = 1e-7, 0.01, 30
    p = torch.zeros(n, dtype=torch.float64, device="cuda")
    delta = torch.empty((n, 2), dtype=torch.float64, device="cuda")
    delta[:, 0] = 1.0 / n
    delta[:, 1] = (1.0 / n) / deg
    ngh = torch.zeros(n, dtype=torch.float64, device="cuda")
    Frontier = byo.vertexSubset.all(G)
    All = byo.vertexSubset.all(G)
    rounds = 0
    while rounds < max_iters:
        rounds += 1
        f = byo.PR_Delta_F(G, delta, ngh)
        # sparse_or_dense (PageRank.h:232-276): the dense reduce equals a dense
        # edgeMap of PR_Delta_F over ngh = 0
        thr = 0 if Frontier.size() > n // 5 else m // 2
        out = byo.edgeMap(G, Frontier, f, thr, _abi.FL_NO_OUTPUT)
        out.close()
        f.close()
        kind = _abi.VOP_PR_DELTA_FIRST if rounds == 1 else _abi.VOP_PR_DELTA
        active = byo.vertexFilter(All, kind, a=p, b=delta, c=ngh, damping=0.85, eps2=local_eps)
        L1 = float(delta[:, 0].abs().sum())
        if L1 < eps:
            active.close()
            break
        ngh.zero_()
        Frontier.close()
        Frontier = active
    op, orounds, _ = O.pagerank_delta(off, nb, eps, local_eps, max_iters)
    assert rounds == orounds
    l1 = float(np.abs(p.cpu().numpy() - op).sum())
    assert l1 <= 1e-6, l1
    Frontier.close()
    All.close()


def test_vertex_subset_from_bitmap_and_filter(ctx, oracle_mod):
    import torch

    import byo_gb300 as byo
    from byo_gb300 import _abi
    O = oracle_mod
    s, d = O.rmat_edges(3, 12, 1 << 15)
    off, nb = O.build_csr((1 << 12) + 7, s, d)  # n not a multiple of 32
    G = byo.Graph.from_csr(ctx, off, nb)
    with _on(ctx):
        _bitmap_filter(byo, G, torch)
    G.close()


def _bitmap_filter(byo, G, torch):
    from byo_gb300 import _abi
    n = G.N()
    rng = np.random.default_rng(1)
    members = np.sort(rng.choice(n, 700, replace=False)).astype(np.uint32)
    words = np.zeros((n + 31) // 32, np.uint32)
    np.bitwise_or.at(words, members >> 5, (np.uint32(1) << (members & 31)).astype(np.uint32))
    words[-1] |= np.uint32(0xFFFFFFFF) << np.uint32(n & 31)  # bits past n are ignored
    vs = byo.vertexSubset.from_bitmap(G, torch.from_numpy(words.view(np.int32)).cuda())
    assert vs.size() == len(members) and vs.isDense
    assert np.array_equal(vs.to_list(), members)
    # vertexFilter with PR_Vertex_F (delta): keeps |nghSum * damping| > eps2 * p
    p = torch.from_numpy(rng.random(n)).cuda()
    ngh = torch.from_numpy(rng.normal(0, 1, n)).cuda()
    delta = torch.zeros((n, 2), dtype=torch.float64, device="cuda")
    p0, g0 = p.cpu().numpy().copy(), ngh.cpu().numpy()
    kept = byo.vertexFilter(vs, _abi.VOP_PR_DELTA, a=p, b=delta, c=ngh, damping=0.85, eps2=0.5)
    nd = g0[members] * 0.85
    keep = np.abs(nd) > 0.5 * p0[members]
    assert np.array_equal(kept.to_list(), members[keep])
    pn = p.cpu().numpy()
    assert np.array_equal(pn[members[keep]], p0[members[keep]] + nd[keep])
    assert np.array_equal(pn[members[~keep]], p0[members[~keep]])
    kept.close()
    vs.close()

"""CUDA path (through the C ABI) against the oracle: bit-exact BFS levels and
min-id parents, CC labels, triangle counts, generated graphs; PageRank within
1e-6 L1 of the FP64 oracle."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POLICIES = [0, 2, 3, 4, 5]  # m/20, push, pull, blocked, m/20+blocked
PR_TOL = 1e-6               # L1 vs the FP64 oracle


def _csr(g):
    return np.array(g["offsets"], np.uint64), np.array(g["nbrs"], np.uint32)


def _check_all(byo, O, G, off, nb, srcs, policies=POLICIES, pr_iters=(100,)):
    n = len(off) - 1
    for s in srcs:
        opar, olev = O.bfs(off, nb, s)
        for pol in policies:
            par, lev = byo.BFS(G, s, policy=pol, levels=True)
            assert np.array_equal(lev, olev), ("level", s, pol)
            assert np.array_equal(par, opar), ("parent", s, pol)
    olab = O.cc(off, nb)
    assert np.array_equal(byo.SimpleUnionAsync(G), olab)
    assert np.array_equal(byo.bfs_cc(G), olab)
    assert byo.Triangle_degree_ordering(G) == O.triangle_count(off, nb)
    for iters in pr_iters:
        op, oit, _ = O.pagerank(off, nb, 1e-6, iters)
        p, it, _ = byo.PageRank(G, 1e-6, iters, info=True)
        assert abs(it - oit) <= 1
        if it == oit:
            assert float(np.abs(p - op).sum()) <= PR_TOL
        p64, it64, _ = byo.PageRank(G, 1e-6, iters, precision=1, info=True)
        assert it64 == oit
        assert float(np.abs(p64 - op).sum()) <= 1e-12


def test_golden_graphs(ctx, golden, oracle_mod):
    import byo_gb300 as byo
    for g in golden["graphs"]:
        off, nb = _csr(g)
        G = byo.Graph.from_csr(ctx, off, nb)
        assert G.N() == g["n"] and G.M() == len(g["nbrs"])
        for src, exp in g["bfs"].items():
            for pol in POLICIES:
                par, lev = byo.BFS(G, int(src), policy=pol, levels=True)
                assert lev.tolist() == exp["level"], (g["name"], src, pol)
                assert par.tolist() == exp["parent"], (g["name"], src, pol)
            if "reference_bfs" in g:
                par = byo.BFS(G, int(src))
                for v, choices in enumerate(g["reference_bfs"][src]):
                    assert int(par[v]) in choices
        assert byo.SimpleUnionAsync(G).tolist() == g["cc"]
        assert byo.bfs_cc(G).tolist() == g["cc"]
        assert byo.Triangle_degree_ordering(G) == g["triangles"]
        for pr in g["pagerank"].values():
            p, it, _ = byo.PageRank(G, pr["eps"], pr["max_iters"], info=True)
            assert it == pr["iters"]
            assert float(np.abs(p - np.array(pr["p"])).sum()) <= PR_TOL
        o2, n2 = G.export_csr()
        assert np.array_equal(o2, off) and np.array_equal(n2, nb)
        G.close()


@pytest.mark.parametrize("lg,draws,seed", [(10, 1 << 13, 1), (14, 1 << 17, 2), (16, 1 << 20, 3)])
def test_rmat_generated(ctx, oracle_mod, lg, draws, seed):
    import byo_gb300 as byo
    O = oracle_mod
    G = byo.Graph.generate(ctx, "rmat", seed=seed, lg_n=lg, draws=draws)
    s, d = O.rmat_edges(seed, lg, draws)
    off, nb = O.build_csr(1 << lg, s, d)
    go, gn = G.export_csr()
    assert np.array_equal(go, off) and np.array_equal(gn, nb)
    assert np.array_equal(G.degrees(), np.diff(off).astype(np.uint32))
    hub = int(np.argmax(np.diff(off.astype(np.int64))))
    _check_all(byo, O, G, off, nb, [10 % (1 << lg), hub], pr_iters=(20, 100))


def test_er_grid_chung_lu(ctx, oracle_mod):
    import byo_gb300 as byo
    O = oracle_mod
    cases = []
    G = byo.Graph.generate(ctx, "er", seed=5, n=5000, draws=40000)
    s, d = O.uniform_pairs(5, 5000, 40000)
    cases.append((G, *O.build_csr(5000, s, d)))
    G = byo.Graph.generate(ctx, "grid", n=37, draws=53)
    s, d = O.grid_pairs(37, 53)
    cases.append((G, *O.build_csr(37 * 53, s, d)))
    G = byo.Graph.generate(ctx, "chung_lu", seed=7, n=20000, draws=80000, exponent=2.1)
    s, d = O.chung_lu_pairs(7, 20000, 80000, exponent=2.1)
    cases.append((G, *O.build_csr(20000, s, d)))
    for G, off, nb in cases:
        go, gn = G.export_csr()
        assert np.array_equal(go, off) and np.array_equal(gn, nb)
        _check_all(byo, O, G, off, nb, [0, len(off) // 2 - 1])
        G.close()


def test_device_pair_streams(ctx, oracle_mod):
    import torch
    from byo_gb300 import _abi
    L = _abi.lib()
    cnt, first = 4096, 777
    s = torch.empty(cnt, dtype=torch.int32, device="cuda")
    d = torch.empty(cnt, dtype=torch.int32, device="cuda")
    _abi.check(L.byo_gen_rmat_pairs_device(ctx.h, 9, 18, 0.57, 0.19, 0.19, first, cnt, s.data_ptr(),
                                           d.data_ptr()), ctx.h)
    ctx.synchronize()
    os_, od = oracle_mod.rmat_edges(9, 18, cnt, first=first)
    assert np.array_equal(s.cpu().numpy().view(np.uint32), os_)
    assert np.array_equal(d.cpu().numpy().view(np.uint32), od)
    _abi.check(L.byo_gen_uniform_pairs_device(ctx.h, 4, 123457, first, cnt, s.data_ptr(), d.data_ptr()),
               ctx.h)
    ctx.synchronize()
    us, ud = oracle_mod.uniform_pairs(4, 123457, cnt, first=first)
    assert np.array_equal(s.cpu().numpy().view(np.uint32), us)
    assert np.array_equal(d.cpu().numpy().view(np.uint32), ud)


def test_edge_map_api_matches_bfs(ctx, oracle_mod):
    """BFS written as the reference's loop over edgeMap (BFS.h:47-64)."""
    import byo_gb300 as byo
    G = byo.Graph.generate(ctx, "rmat", seed=11, lg_n=13, draws=1 << 16)
    off, nb = G.export_csr()
    for flags in (byo._abi.FL_DENSE_PARALLEL | byo._abi.FL_SPARSE_BLOCKED, byo._abi.FL_NO_DENSE,
                  byo._abi.FL_DENSE_ONLY, byo._abi.FL_DENSE_FORWARD,
                  byo._abi.FL_DENSE_ONLY | byo._abi.FL_DENSE_FORWARD):
        F = byo.BFS_F(G, 10)
        frontier = byo.vertexSubset(G, 10)
        sizes = []
        while not frontier.isEmpty():
            sizes.append(frontier.size())
            frontier = byo.edgeMap(G, frontier, F, -1, flags)
        opar, olev = oracle_mod.bfs(off, nb, 10)
        assert np.array_equal(F.parents(), opar)
        assert sizes == [int((olev == l).sum()) for l in range(len(sizes))]
    vs = byo.vertexSubset(G, [5, 3, 9])
    assert vs.to_list().tolist() == [3, 5, 9]


def test_error_paths(ctx):
    import byo_gb300 as byo
    off = np.array([0, 1, 2], np.uint64)
    with pytest.raises(byo.ByoError) as e:
        byo.Graph.from_csr(ctx, off, np.array([1, 5], np.uint32))  # id >= n
    assert e.value.code == byo._abi.BYO_EINVAL
    with pytest.raises(byo.ByoError) as e:  # adjacency of vertex 0 not increasing
        byo.Graph.from_csr(ctx, np.array([0, 2, 2], np.uint64), np.array([1, 1], np.uint32))
    assert e.value.code == byo._abi.BYO_EINVAL
    G = byo.Graph.from_csr(ctx, off, np.array([1, 0], np.uint32))
    with pytest.raises(byo.ByoError) as e:
        byo.BFS(G, 7)
    assert e.value.code == byo._abi.BYO_EINVAL
    with pytest.raises(byo.ByoError) as e:
        G.insert_batch(np.array([1], np.uint64))
    assert e.value.code == byo._abi.BYO_ENOTSUP
    # the context stays usable after errors
    assert byo.BFS(G, 0).tolist() == [0, 0]


def test_empty_and_isolated(ctx, oracle_mod):
    import byo_gb300 as byo
    off = np.zeros(5, np.uint64)
    G = byo.Graph.from_csr(ctx, off, np.zeros(0, np.uint32))
    for pol in POLICIES:
        assert byo.BFS(G, 2, policy=pol).tolist() == [byo.UINT_E_MAX] * 2 + [2] + [byo.UINT_E_MAX]
    assert byo.SimpleUnionAsync(G).tolist() == [0, 1, 2, 3]
    assert byo.Triangle_degree_ordering(G) == 0
    p = byo.PageRank(G, 1e-6, 10)
    assert np.allclose(p, 0.15 / 4)


def test_bfs_multi_matches_single(ctx, oracle_mod):
    """64 sources in bit lanes give every source's single-BFS levels."""
    import byo_gb300 as byo
    O = oracle_mod
    for spec in (dict(kind="rmat", seed=12, lg_n=14, draws=1 << 17), dict(kind="grid", n=40, draws=70),
                 dict(kind="er", seed=3, n=3000, draws=6000)):
        kind = spec.pop("kind")
        G = byo.Graph.generate(ctx, kind, **spec)
        off, nb = G.export_csr()
        n = len(off) - 1
        rng = np.random.default_rng(n)
        for k in (1, 7, 64):
            srcs = rng.integers(0, n, k).astype(np.uint32)
            srcs[-1] = srcs[0]  # a repeated source
            lev = byo.BFS_multi(G, srcs)
            for s_i, s in enumerate(srcs):
                _, olev = O.bfs(off, nb, int(s))
                assert np.array_equal(lev[s_i], olev), (kind, k, s_i)
        G.close()
    G = byo.Graph.generate(ctx, "rmat", seed=12, lg_n=10, draws=1 << 12, container="pma")
    off, nb = G.export_csr()
    lev = byo.BFS_multi(G, [0, 1, 2])
    for s_i in range(3):
        assert np.array_equal(lev[s_i], O.bfs(off, nb, s_i)[1])
    with pytest.raises(byo.ByoError):
        byo.BFS_multi(G, np.arange(65))


def _sym_csr(n, pairs):
    """Symmetric sorted CSR (uint64 offsets, uint32 ids) from undirected pairs."""
    p = np.asarray(pairs, np.int64)
    src = np.concatenate([p[:, 0], p[:, 1]])
    dst = np.concatenate([p[:, 1], p[:, 0]])
    keys = np.unique(src.astype(np.uint64) << np.uint64(32) | dst.astype(np.uint64))
    s = (keys >> np.uint64(32)).astype(np.int64)
    off = np.zeros(n + 1, np.uint64)
    np.add.at(off, s + 1, 1)
    return np.cumsum(off).astype(np.uint64), (keys & np.uint64(0xFFFFFFFF)).astype(np.uint32)


@pytest.mark.gpu
def test_bfs_multi_deep_levels(ctx):
    """Levels from 2^16 on (a path of 70000 vertices) are stored by the
    traversal itself, the lower ones come from the bit planes; an isolated
    vertex stays unreached."""
    import byo_gb300 as byo
    n = 70000
    off, nb = _sym_csr(n + 1, [(i, i + 1) for i in range(n - 1)])
    G = byo.Graph.from_csr(ctx, off, nb)
    srcs = [0, n - 1, 1234]
    lev = byo.BFS_multi(G, srcs)
    for i, s in enumerate(srcs):
        want = np.abs(np.arange(n + 1, dtype=np.int64) - s).astype(np.uint32)
        want[n] = 0xFFFFFFFF
        assert np.array_equal(lev[i], want), i
    G.close()


@pytest.mark.gpu
def test_bfs_multi_launch_shapes(ctx, oracle_mod):
    """Every direction and degree-bucket path of the 64-source kernel (forced
    push, forced pull, warp-per-vertex pull, hub chunks) gives the levels of
    single-source BFS."""
    import byo_gb300 as byo
    O = oracle_mod
    star = [(0, i) for i in range(1, 5001)] + [(5000 + i, 5001 + i) for i in range(99)]
    off_s, nb_s = _sym_csr(5100, star)
    graphs = [byo.Graph.generate(ctx, "rmat", seed=5, lg_n=13, draws=1 << 17),
              byo.Graph.from_csr(ctx, off_s, nb_s),
              byo.Graph.generate(ctx, "rmat", seed=6, lg_n=12, draws=1 << 15, container="pma"),
              byo.Graph.generate(ctx, "grid", n=30, draws=30)]
    shapes = [dict(ms_push_div=1), dict(ms_push_div=0xFFFFFFFF),
              dict(ms_heavy_deg=1, ms_hub_deg=32, ms_push_div=1),
              dict(ms_heavy_deg=1, ms_hub_deg=32, ms_push_div=0xFFFFFFFF),
              dict(ms_heavy_deg=65536, ms_hub_deg=1 << 20, ms_push_div=5)]
    for gi, G in enumerate(graphs):
        off, nb = G.export_csr()
        n = len(off) - 1
        rng = np.random.default_rng(100 + gi)
        srcs = rng.integers(0, n, 64).astype(np.uint32)
        srcs[0] = 0
        srcs[1] = n - 1
        want = [O.bfs(off, nb, int(s))[1] for s in srcs]
        for sh in shapes:
            G.set_tuning(**sh)
            lev = byo.BFS_multi(G, srcs)
            for i in range(64):
                assert np.array_equal(lev[i], want[i]), (gi, sh, i)
        G.set_tuning(ms_heavy_deg=0, ms_hub_deg=0, ms_push_div=0)
        G.close()


@pytest.mark.gpu
def test_tuning_api_and_autotune(ctx, oracle_mod):
    """Launch shapes are per graph, validated, and never change a result."""
    import byo_gb300 as byo
    O = oracle_mod
    G = byo.Graph.generate(ctx, "rmat", seed=9, lg_n=13, draws=1 << 16)
    off, nb = G.export_csr()
    t = G.tuning()
    assert all(v > 0 for v in t.values())
    G.set_tuning(push_group=8, pull_cap=4)
    assert G.tuning()["push_group"] == 8 and G.tuning()["pull_cap"] == 4
    for bad in (dict(push_group=7), dict(hub_min=5), dict(blocked_tile=10), dict(ms_hub_deg=8)):
        with pytest.raises(byo.ByoError):
            G.set_tuning(**bad)
    opar, olev = O.bfs(off, nb, 10)
    for pol in (byo._abi.POLICY_M20, byo._abi.POLICY_M20_BLOCKED, byo._abi.POLICY_PUSH, byo._abi.POLICY_PULL):
        par, lev = byo.BFS(G, 10, policy=pol, levels=True)
        assert np.array_equal(par, opar) and np.array_equal(lev, olev)
    t = G.autotune(bfs=True, multi=True, trials=2)
    assert t["push_group"] in (4, 8, 16, 32) and t["ms_push_div"] in (5, 10, 20, 40, 80)
    assert G.tuning() == t
    par = byo.BFS(G, 10)
    assert np.array_equal(par, opar)
    lev = byo.BFS_multi(G, [10, 11])
    assert np.array_equal(lev[0], olev)
    G.close()


@pytest.mark.gpu
def test_pagerank_delta_and_edgemap(ctx, oracle_mod):
    """PageRankDelta within 1e-6 L1 of the oracle with the same number of
    rounds; PageRank_edgeMap equals PageRank's FP64 recurrence."""
    import byo_gb300 as byo
    O = oracle_mod
    graphs = [byo.Graph.generate(ctx, "rmat", seed=21, lg_n=15, draws=1 << 19),
              byo.Graph.generate(ctx, "er", seed=22, n=20000, draws=80000),
              byo.Graph.generate(ctx, "grid", n=60, draws=70),
              byo.Graph.generate(ctx, "rmat", seed=23, lg_n=13, draws=1 << 16, container="pma")]
    for G in graphs:
        off, nb = G.export_csr()
        for eps, leps, iters in ((1e-4, 0.01, 20), (1e-7, 1e-3, 100)):
            p, r, _ = byo.PageRankDelta(G, eps, leps, iters, info=True)
            op, orr, _ = O.pagerank_delta(off, nb, eps, leps, iters)
            assert r == orr, (G.N(), eps)
            assert float(np.abs(p - op).sum()) <= 1e-6, (G.N(), eps)
        q, it, _ = byo.PageRank_edgeMap(G, 1e-6, 30, info=True)
        oq, oit, _ = O.pagerank(off, nb, 1e-6, 30)
        assert it == oit and float(np.abs(q - oq).sum()) <= 1e-6
        G.close()


@pytest.mark.gpu
def test_graph_files_round_trip(ctx, oracle_mod, tmp_path):
    """write_adj then read_adj, both layouts, into every container."""
    import byo_gb300 as byo
    G = byo.Graph.generate(ctx, "rmat", seed=17, lg_n=12, draws=1 << 15, container="pma")
    G.insert_batch(np.array([(1 << 32) | 2, (2 << 32) | 1], np.uint64))
    off, nb = G.export_csr()
    for binary in (False, True):
        p = str(tmp_path / ("g.bin" if binary else "g.adj"))
        G.write_adj(p, binary)
        for cont in ("csr", "pma", "pcsr"):
            H = byo.Graph.read_adj(ctx, p, binary, container=cont)
            o2, n2 = H.export_csr()
            assert np.array_equal(o2, off) and np.array_equal(n2, nb)
            assert np.array_equal(byo.BFS(H, 1), oracle_mod.bfs(off, nb, 1)[0])
            H.close()
    G.close()


@pytest.mark.gpu
def test_triangle_count_paths(ctx, oracle_mod):
    """Warp-staged, CTA-staged and in-place out-lists give the oracle's count:
    a 700-clique (DAG out-lists up to 699) over an RMAT background."""
    import byo_gb300 as byo
    O = oracle_mod
    s, d = O.rmat_edges(29, 12, 1 << 15)
    k = np.arange(700, dtype=np.int64) * 5 + 3
    cs, cd = np.meshgrid(k, k, indexing="ij")
    mask = cs < cd
    src = np.concatenate([s.astype(np.int64), cs[mask]])
    dst = np.concatenate([d.astype(np.int64), cd[mask]])
    off, nb = O.build_csr(1 << 12, src.astype(np.uint32), dst.astype(np.uint32))
    want = O.triangle_count(off, nb)
    for cont in ("csr", "pma", "pcsr"):
        G = byo.Graph.from_csr(ctx, off, nb, container=cont)
        for stage in (0, 512):
            G.set_tuning(tc_stage=stage)
            assert byo.Triangle_degree_ordering(G) == want, (cont, stage)
        G.close()


def _remote_arrays(n, rng):
    """A remote array per width, as Map_Remote_runner builds them
    (run_unweighted.h:50-126: zeros with one random entry set) plus a random one."""
    out = {}
    for w in (0, 1, 2, 4, 8, 16, 32):
        one = int(rng.integers(0, n))
        if w == 0:
            bits = np.zeros(n, bool)
            bits[one] = True
            rnd = rng.integers(0, 2, size=n).astype(bool)
            pack = lambda b: np.concatenate([np.packbits(b, bitorder="little"),  # noqa: E731
                                             np.zeros((-((n + 7) // 8)) % 8, np.uint8)]).view(np.uint64)
            out[w] = [pack(bits), pack(rnd)]
        elif w <= 8:
            dt = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[w]
            a = np.zeros(n, dt)
            a[one] = 1
            out[w] = [a, rng.integers(0, 250, size=n).astype(dt)]
        else:
            a = np.zeros((n, w // 8), np.uint64)
            a[one, 0] = 1
            b = np.full((n, w // 8), 3, np.uint64)  # padding words are not read
            b[:, 0] = rng.integers(0, 1 << 40, size=n)
            out[w] = [a, b]
    return out


@pytest.mark.gpu
def test_map_benchmarks(ctx, oracle_mod):
    """Test_Map and Test_Map_Remote (every width) equal the oracle on a CSR and
    on a PMA (scanned with its gaps, before and after a batch), from host and
    device remote arrays."""
    import torch
    import byo_gb300 as byo
    O = oracle_mod
    rng = np.random.default_rng(12)
    G1 = byo.Graph.generate(ctx, "rmat", seed=41, lg_n=15, draws=1 << 19)
    G2 = byo.Graph.generate(ctx, "rmat", seed=42, lg_n=14, draws=1 << 18, container="pma")
    for G in (G1, G2):
        for step in range(2):
            if step == 1 and G is G2:
                pairs = rng.integers(0, G.N(), size=(5000, 2))
                G.insert_batch(O.keys_from_pairs(pairs[:, 0], pairs[:, 1]))
            off, nb = G.export_csr()
            assert byo.Test_Map(G) == O.map_sum(off, nb)
            for w, arrs in _remote_arrays(G.N(), rng).items():
                for a in arrs:
                    exp = O.map_remote(off, nb, a, w)
                    assert byo.Test_Map_Remote(G, a, w) == exp, (w,)
                    t = torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).cuda()
                    assert byo.Test_Map_Remote(G, t, w) == exp, (w, "device")
        with pytest.raises(byo.ByoError):
            byo.Test_Map_Remote(G, np.zeros(G.N(), np.uint32), 3)
        G.close()

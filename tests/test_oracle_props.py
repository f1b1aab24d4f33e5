"""Oracle properties: generator slices, CSR build invariants, and the
algorithms against networkx on seeded random graphs."""
import networkx as nx
import numpy as np
import pytest

NONE = 0xFFFFFFFF


def _nx(off, nb):
    g = nx.Graph()
    n = len(off) - 1
    g.add_nodes_from(range(n))
    for v in range(n):
        for j in range(int(off[v]), int(off[v + 1])):
            g.add_edge(v, int(nb[j]))
    return g


def test_generator_slices(oracle_mod):
    s, d = oracle_mod.rmat_edges(7, 14, 5000)
    s2, d2 = oracle_mod.rmat_edges(7, 14, 1000, first=2000)
    assert np.array_equal(s[2000:3000], s2) and np.array_equal(d[2000:3000], d2)
    u, v = oracle_mod.uniform_pairs(3, 1000, 4000)
    u2, v2 = oracle_mod.uniform_pairs(3, 1000, 100, first=3900)
    assert np.array_equal(u[3900:], u2) and np.array_equal(v[3900:], v2)
    assert u.max() < 1000 and v.max() < 1000
    assert s.max() < (1 << 14)


def test_rmat_skew(oracle_mod):
    # quadrant a=0.57 biases both endpoints toward low ids
    s, d = oracle_mod.rmat_edges(1, 16, 200000)
    top = (s < (1 << 15)).mean()
    assert 0.74 < top < 0.78  # P(first src bit 0) = a + b = 0.76


def test_build_csr_invariants(oracle_mod):
    s, d = oracle_mod.rmat_edges(2, 10, 6000)
    off, nb = oracle_mod.build_csr(1024, s, d)
    n = 1024
    keys = set()
    for v in range(n):
        run = nb[off[v]:off[v + 1]]
        assert np.all(np.diff(run.astype(np.int64)) > 0)
        assert v not in run
        keys |= {(v, int(x)) for x in run}
    assert all((b, a) in keys for a, b in keys)


@pytest.mark.parametrize("seed,lg,draws", [(1, 9, 3000), (5, 11, 20000), (9, 8, 100)])
def test_against_networkx(oracle_mod, seed, lg, draws):
    s, d = oracle_mod.rmat_edges(seed, lg, draws)
    n = 1 << lg
    off, nb = oracle_mod.build_csr(n, s, d)
    g = _nx(off, nb)
    src = int(np.argmax(np.diff(off.astype(np.int64))))
    par, lev = oracle_mod.bfs(off, nb, src)
    dist = nx.single_source_shortest_path_length(g, src)
    for v in range(n):
        if v in dist:
            assert lev[v] == dist[v]
            if v != src:
                assert par[v] == min(u for u in g[v] if dist.get(u) == dist[v] - 1)
        else:
            assert lev[v] == NONE and par[v] == NONE
    lab = oracle_mod.cc(off, nb)
    for comp in nx.connected_components(g):
        m = min(comp)
        assert all(lab[v] == m for v in comp)
    assert oracle_mod.triangle_count(off, nb) == sum(nx.triangles(g).values()) // 3


def test_grid_and_chung_lu(oracle_mod):
    s, d = oracle_mod.grid_pairs(5, 7)
    off, nb = oracle_mod.build_csr(35, s, d)
    assert len(nb) == 2 * (2 * 35 - 5 - 7)
    par, lev = oracle_mod.bfs(off, nb, 0)
    assert lev[34] == 4 + 6
    cdf = oracle_mod.chung_lu_cdf(1000, 2.1)
    assert cdf[-1] == 1 << 63 and np.all(np.diff(cdf.astype(np.float64)) >= 0)
    cs, cd = oracle_mod.chung_lu_pairs(4, 1000, 50000, cdf=cdf)
    deg = np.bincount(np.concatenate([cs, cd]), minlength=1000)
    assert deg[0] > deg[10] > deg[500]


def test_pagerank_semantics(oracle_mod):
    # isolated vertex keeps (1-d)/n; no dangling redistribution (PageRank.h:125-193)
    off = np.array([0, 1, 2, 2], np.uint64)
    nb = np.array([1, 0], np.uint32)
    p, it, l1 = oracle_mod.pagerank(off, nb, 1e-12, 100)
    assert abs(p[2] - 0.15 / 3) < 1e-15
    assert abs(p[0] - p[1]) < 1e-15
    assert abs(p.sum() - (2 * (1 / 3) + 0.15 / 3)) < 1e-12


def test_store_model_random(oracle_mod):
    rng = np.random.default_rng(3)
    s, d = oracle_mod.rmat_edges(4, 9, 2000)
    off, nb = oracle_mod.build_csr(512, s, d)
    st = oracle_mod.Store(off, nb)
    cur = {(v, int(x)) for v in range(512) for x in nb[off[v]:off[v + 1]]}
    for it in range(6):
        pairs = rng.integers(0, 512, size=(300, 2))
        keys = (pairs[:, 0].astype(np.uint64) << np.uint64(32)) | pairs[:, 1].astype(np.uint64)
        ps = {(int(a), int(b)) for a, b in pairs}
        if it % 2 == 0:
            assert st.insert_batch(keys) == len(ps - cur)
            cur |= ps
        else:
            assert st.remove_batch(keys) == len(ps & cur)
            cur -= ps
        o2, n2 = st.export_csr()
        got = {(v, int(x)) for v in range(512) for x in n2[o2[v]:o2[v + 1]]}
        assert got == cur


def _pagerank_delta_numpy(off, nb, eps, local_eps, max_iters):
    """A second restatement of delta::PageRankDelta (PageRank.h:340-398) in
    numpy, to pin the C oracle."""
    n = len(off) - 1
    deg = np.diff(off.astype(np.int64)).astype(np.float64)
    src = np.repeat(np.arange(n), np.diff(off.astype(np.int64)))
    p = np.zeros(n)
    with np.errstate(divide="ignore", invalid="ignore"):
        dod = np.full(n, 1.0 / n) / deg
    front = np.ones(n, bool)
    rounds = 0
    while rounds < max_iters:
        rounds += 1
        ngh = np.zeros(n)
        contrib = np.where(front[nb], dod[nb], 0.0)
        for v in range(n):  # left to right over sorted neighbours, like the oracle
            s = 0.0
            for x in contrib[off[v]:off[v + 1]]:
                s += x
            ngh[v] = s
        if rounds == 1:
            pre = 0.85 * ngh + (1 - 0.85) * (1 / n)
            p = p + pre
            nd = pre - 1.0 / n
            nxt = nd > local_eps * p
        else:
            nd = ngh * 0.85
            nxt = np.abs(nd) > local_eps * p
            p = np.where(nxt, p + nd, p)
        with np.errstate(divide="ignore", invalid="ignore"):
            dod = nd / deg
        l1 = 0.0
        for x in np.abs(nd):
            l1 += x
        if l1 < eps:
            break
        front = nxt
    del src
    return p, rounds


@pytest.mark.parametrize("eps,leps", [(1e-4, 0.01), (1e-7, 1e-3)])
def test_pagerank_delta_restatements_agree(oracle_mod, eps, leps):
    O = oracle_mod
    s, d = O.rmat_edges(3, 9, 1 << 12)
    off, nb = O.build_csr(1 << 9, s, d)
    p, r, l1 = O.pagerank_delta(off, nb, eps, leps, 50)
    q, rq = _pagerank_delta_numpy(off, nb, eps, leps, 50)
    assert r == rq
    assert np.array_equal(p, q)
    # it approaches PageRank's fixed point only loosely (round-one decreases
    # never propagate), but every vertex with edges moved away from 0
    assert np.all(p > 0)


def test_map_restatement(oracle_mod):
    """Test_Map / Test_Map_Remote in the oracle equal a numpy gather-and-sum
    for every remote element width, bitmap included."""
    O = oracle_mod
    s, d = O.rmat_edges(3, 10, 1 << 13)
    off, nb = O.build_csr(1 << 10, s, d)
    n = len(off) - 1
    assert O.map_sum(off, nb) == int(nb.astype(np.uint64).sum())
    rng = np.random.default_rng(1)
    for w in (0, 1, 2, 4, 8, 16, 32):
        if w == 0:
            bits = rng.integers(0, 2, size=n).astype(bool)
            words = np.packbits(bits, bitorder="little")
            words = np.concatenate([words, np.zeros((-len(words)) % 8, np.uint8)]).view(np.uint64)
            assert O.map_remote(off, nb, words, 0) == int(bits[nb].sum())
        elif w <= 8:
            r = rng.integers(0, 200, size=n).astype({1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[w])
            assert O.map_remote(off, nb, r, w) == int(r[nb].astype(np.uint64).sum())
        else:
            r = np.full((n, w // 8), 7, np.uint64)
            r[:, 0] = rng.integers(0, 1000, size=n)
            assert O.map_remote(off, nb, r, w) == int(r[nb, 0].sum())


def test_bytepd_golden_and_round_trip(oracle_mod):
    """The byte-PD amortized layout, byte for byte on a hand-encoded vertex
    (byte_pd_amortized.cc:7-55: first neighbour as a signed difference from
    the source with 6 bits in its first byte, then 7-bit differences), and
    encode -> decode round trips for several block sizes."""
    O = oracle_mod
    # vertex 5 with neighbours 3, 7, 200 (others empty), one block
    off = np.array([0, 0, 0, 0, 0, 0, 3, 3], np.uint64)
    nb = np.array([3, 7, 200], np.uint32)
    bo, deg, data = O.bytepd_encode(off, nb, 1000)
    exp = bytes([3, 0, 0, 0,  0, 0, 0, 0,  0x42, 0x04, 0xC1, 0x01])
    assert bytes(data) == exp and bo.tolist() == [0] * 6 + [12, 12] and deg.tolist() == [0] * 5 + [3, 0]
    # two blocks of 2: block offsets, block start indices, the first edge of
    # block 1 again relative to the source (200 - 5 = 195 = 0b11 000011)
    off2 = np.array([0, 0, 0, 0, 0, 0, 3], np.uint64)
    bo, deg, data = O.bytepd_encode(off2, nb, 2)
    exp = bytes([3, 0, 0, 0,  14, 0, 0, 0,  0, 0, 0, 0,  0x42, 0x04,  2, 0, 0, 0,  0x83, 0x03])
    assert bytes(data) == exp
    for P in (1000, 256, 7, 1):
        s, d = O.rmat_edges(11, 12, 1 << 16)
        o, n_ = O.build_csr(1 << 12, s, d)
        bo, deg, data = O.bytepd_encode(o, n_, P)
        o2, n2 = O.bytepd_decode(bo, deg, data, P)
        assert np.array_equal(o2, o) and np.array_equal(n2, n_)


def test_mlp_ref_gradient_matches_finite_differences():
    """The FP64 restatement of the policy network's loss gradient (the checker
    of the device training kernels) against central differences of its own
    loss, on up to 10 random parameters of every weight and bias block."""
    from oracle import mlp_ref
    rng = np.random.default_rng(71)
    p = rng.normal(0, 0.3, mlp_ref.NPARAMS)
    X = rng.normal(0, 1, (24, mlp_ref.NIN))
    Y = rng.normal(0, 1, (24, mlp_ref.NOUT))
    mask = rng.integers(1, 1 << mlp_ref.NOUT, 24).astype(np.uint8)
    loss, g = mlp_ref.loss_grad(p, X, Y, mask)
    assert g.shape == (mlp_ref.NPARAMS,) and loss > 0
    h = 1e-6
    picks, o = [], 0
    for _, shape in mlp_ref.SIZES:
        k = int(np.prod(shape))
        picks += list(o + rng.choice(k, min(k, 10), replace=False))
        o += k
    for i in picks:
        q = p.copy()
        q[i] += h
        lp, _ = mlp_ref.loss_grad(q, X, Y, mask)
        q[i] -= 2 * h
        lm, _ = mlp_ref.loss_grad(q, X, Y, mask)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (int(i), fd, g[i])

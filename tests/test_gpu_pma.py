"""Packed-memory-array container on the GPU against the oracle's container
model: contents after every batch (sorted adjacency, bit-exact), the number of
keys changed, and BFS / CC / PageRank / TC run directly on the PMA."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check_view(byo, O, G, ref_off, ref_nb, bfs_src=(0,)):
    off, nb = G.export_csr()
    assert np.array_equal(off, ref_off) and np.array_equal(nb, ref_nb)
    assert G.M() == len(ref_nb)
    assert np.array_equal(G.degrees(), np.diff(ref_off).astype(np.uint32))
    for s in bfs_src:
        opar, olev = O.bfs(ref_off, ref_nb, s)
        for pol in (0, 2, 3, 4):
            par, lev = byo.BFS(G, s, policy=pol, levels=True)
            assert np.array_equal(lev, olev) and np.array_equal(par, opar), (s, pol)
    assert np.array_equal(byo.SimpleUnionAsync(G), O.cc(ref_off, ref_nb))


def test_golden_update_sequence(ctx, golden, oracle_mod):
    import byo_gb300 as byo
    u = golden["updates"]
    G = byo.Graph.from_csr(ctx, np.array(u["offsets"], np.uint64), np.array(u["nbrs"], np.uint32),
                           container="pma")
    assert G.container == "pma"
    for b in u["batches"]:
        keys = np.array(b["keys"], np.uint64)
        ch = G.insert_batch(keys) if b["op"] == "insert" else G.remove_batch(keys)
        assert ch == b["changed"]
        off, nb = G.export_csr()
        assert off.tolist() == b["offsets"] and nb.tolist() == b["nbrs"]


@pytest.mark.parametrize("lg,draws,batch", [(10, 6000, 500), (13, 1 << 16, 20000), (15, 1 << 18, 300000)])
def test_random_batches(ctx, oracle_mod, lg, draws, batch):
    import byo_gb300 as byo
    O = oracle_mod
    n = 1 << lg
    G = byo.Graph.generate(ctx, "rmat", seed=lg, lg_n=lg, draws=draws, container="pma")
    s, d = O.rmat_edges(lg, lg, draws)
    off, nb = O.build_csr(n, s, d)
    _check_view(byo, O, G, off, nb, (10,))
    st = O.Store(off, nb)
    batches = []
    for k in range(4):
        us, ud = O.uniform_pairs(100 + k, n, batch)
        keys = O.keys_from_pairs(us, ud)            # symmetrised, unsorted, duplicates
        batches.append(keys)
        assert G.insert_batch(keys) == st.insert_batch(keys)
        ro, rn = st.export_csr()
        _check_view(byo, O, G, ro, rn, (10,))
    for keys in batches[:3]:
        assert G.remove_batch(keys) == st.remove_batch(keys)
        ro, rn = st.export_csr()
        _check_view(byo, O, G, ro, rn, (10,))
    ro, rn = st.export_csr()
    p = byo.PageRank(G, 1e-6, 30)
    op, _, _ = O.pagerank(ro, rn, 1e-6, 30)
    assert float(np.abs(p - op).sum()) <= 1e-6
    assert byo.Triangle_degree_ordering(G) == O.triangle_count(ro, rn)


def test_skewed_batch_grows_and_shrinks(ctx, oracle_mod):
    """One hub receives a batch far larger than a leaf (windows / growth),
    then everything is removed again (shrink)."""
    import byo_gb300 as byo
    O = oracle_mod
    n = 1 << 14
    G = byo.Graph.generate(ctx, "rmat", seed=3, lg_n=14, draws=1 << 15, container="pma")
    s, d = O.rmat_edges(3, 14, 1 << 15)
    off, nb = O.build_csr(n, s, d)
    st = O.Store(off, nb)
    hub = 12345
    others = np.arange(n, dtype=np.uint64)
    keys = np.concatenate([(np.uint64(hub) << np.uint64(32)) | others, (others << np.uint64(32)) | np.uint64(hub)])
    assert G.insert_batch(keys) == st.insert_batch(keys)
    ro, rn = st.export_csr()
    _check_view(byo, O, G, ro, rn, (hub, 0))
    sk = np.sort(np.unique(keys))
    assert G.remove_batch(sk, sorted=True) == st.remove_batch(sk)
    ro, rn = st.export_csr()
    _check_view(byo, O, G, ro, rn, (0,))
    # remove everything, then re-insert everything
    all_keys = O.keys_from_pairs(s, d)
    assert G.remove_batch(all_keys) == st.remove_batch(all_keys)
    assert G.M() == st.num_edges
    ro, rn = st.export_csr()
    _check_view(byo, O, G, ro, rn, (0,))
    assert G.insert_batch(all_keys) == st.insert_batch(all_keys)
    ro, rn = st.export_csr()
    _check_view(byo, O, G, ro, rn, (10,))


def test_small_batches_and_errors(ctx, oracle_mod):
    import byo_gb300 as byo
    O = oracle_mod
    n = 1 << 12
    G = byo.Graph.generate(ctx, "rmat", seed=9, lg_n=12, draws=1 << 14, container="pma")
    s, d = O.rmat_edges(9, 12, 1 << 14)
    off, nb = O.build_csr(n, s, d)
    st = O.Store(off, nb)
    rng = np.random.default_rng(5)
    for size in (1, 2, 10, 100, 1000):
        # symmetrised both ways: the graph stays undirected, as BFS assumes
        pairs = rng.integers(0, n, size=(size, 2))
        keys = O.keys_from_pairs(pairs[:, 0], pairs[:, 1])
        half = O.keys_from_pairs(pairs[: size // 2 + 1, 0], pairs[: size // 2 + 1, 1])
        assert G.insert_batch(keys) == st.insert_batch(keys)
        assert G.remove_batch(half) == st.remove_batch(half)
    ro, rn = st.export_csr()
    _check_view(byo, O, G, ro, rn, (1,))
    assert G.insert_batch(np.zeros(0, np.uint64)) == 0
    with pytest.raises(byo.ByoError) as e:
        G.insert_batch(np.array([(5 << 32) | n], np.uint64))
    assert e.value.code == byo._abi.BYO_EINVAL
    with pytest.raises(byo.ByoError) as e:
        G.insert_batch(np.array([(5 << 32) | 7, (5 << 32) | 3], np.uint64), sorted=True)
    assert e.value.code == byo._abi.BYO_EINVAL
    # valid keys next to an invalid one: nothing of the batch is applied
    for bad in ((n << 32) | 1, (1 << 32) | (n + 3)):
        with pytest.raises(byo.ByoError) as e:
            G.insert_batch(np.array([(3 << 32) | 4, (4 << 32) | 3, bad], np.uint64))
        assert e.value.code == byo._abi.BYO_EINVAL
        u = int(np.flatnonzero(np.diff(ro))[0])  # an edge that exists
        with pytest.raises(byo.ByoError) as e:
            G.remove_batch(np.array([(u << 32) | int(rn[ro[u]]), bad], np.uint64))
        assert e.value.code == byo._abi.BYO_EINVAL
    # the container is unchanged by rejected batches
    o2, n2 = G.export_csr()
    assert np.array_equal(o2, ro) and np.array_equal(n2, rn)


@pytest.mark.parametrize("lg,draws,sizes", [(17, 1 << 20, (1, 7, 100, 1000, 1300)), (19, 1 << 22, (3000,))])
def test_small_batch_fast_path(ctx, oracle_mod, lg, draws, sizes):
    """Batches of at most half as many keys as there are leaves visit only
    their own leaves (segment list), keep degrees current in the merge and
    refresh the view around those leaves; checked after every batch, with
    one batch that overflows a leaf (a hub gains 700 neighbours)."""
    import byo_gb300 as byo
    O = oracle_mod
    n = 1 << lg
    G = byo.Graph.generate(ctx, "rmat", seed=lg, lg_n=lg, draws=draws, container="pma")
    s, d = O.rmat_edges(lg, lg, draws)
    off, nb = O.build_csr(n, s, d)
    st = O.Store(off, nb)
    assert 2 * 2 * max(sizes) <= G.nslots() // 512
    rng = np.random.default_rng(lg)
    for size in sizes:
        pairs = rng.integers(0, n, size=(size, 2))
        keys = O.keys_from_pairs(pairs[:, 0], pairs[:, 1])
        assert G.insert_batch(keys) == st.insert_batch(keys)
        ro, rn = st.export_csr()
        _check_view(byo, O, G, ro, rn, (10,))
        half = O.keys_from_pairs(pairs[: size // 2 + 1, 0], pairs[: size // 2 + 1, 1])  # stays symmetric
        assert G.remove_batch(half) == st.remove_batch(half)
        ro, rn = st.export_csr()
        _check_view(byo, O, G, ro, rn, (10,))
    hub = 77
    others = rng.choice(n, 700, replace=False).astype(np.uint64)
    keys = np.concatenate([(np.uint64(hub) << np.uint64(32)) | others, (others << np.uint64(32)) | np.uint64(hub)])
    assert G.insert_batch(keys) == st.insert_batch(keys)
    ro, rn = st.export_csr()
    _check_view(byo, O, G, ro, rn, (hub,))
    assert G.remove_batch(keys) == st.remove_batch(keys)
    ro, rn = st.export_csr()
    _check_view(byo, O, G, ro, rn, (hub,))


def test_large_batches(ctx, oracle_mod):
    """Batches of more than 2^20 keys: a uniform one, and one where a few
    sources get more than 512 keys each (their buckets go to the LSD
    fallback of the batch sort)."""
    import byo_gb300 as byo
    O = oracle_mod
    lg = 20
    n = 1 << lg
    G = byo.Graph.generate(ctx, "rmat", seed=7, lg_n=lg, draws=1 << 22, container="pma")
    s, d = O.rmat_edges(7, lg, 1 << 22)
    off, nb = O.build_csr(n, s, d)
    st = O.Store(off, nb)
    us, ud = O.uniform_pairs(300, n, 700000)
    keys = O.keys_from_pairs(us, ud)
    assert G.insert_batch(keys) == st.insert_batch(keys)
    ro, rn = st.export_csr()
    _check_view(byo, O, G, ro, rn, (10,))
    rng = np.random.default_rng(3)
    hubs = np.array([5, 99, 12345], np.uint64)
    extra = np.concatenate([(h << np.uint64(32)) | rng.choice(n, 900, replace=False).astype(np.uint64) for h in hubs])
    skew = np.concatenate([O.keys_from_pairs(us[:600000], ud[:600000]), extra,
                           ((extra & np.uint64(0xFFFFFFFF)) << np.uint64(32)) | (extra >> np.uint64(32))])
    assert G.remove_batch(skew) == st.remove_batch(skew)
    assert G.insert_batch(skew) == st.insert_batch(skew)
    ro, rn = st.export_csr()
    _check_view(byo, O, G, ro, rn, (5,))


@pytest.mark.gpu
def test_two_level_sort_batches(ctx, oracle_mod):
    """Batches of more than 2^21 keys take the two-level sort (coarse bins of
    src, then a shared-memory sort per bin): a uniform batch, and a skewed one
    with a bin above the shared-memory capacity and sources with more than 512
    keys (both sorted afterwards on their ranges)."""
    import byo_gb300 as byo
    O = oracle_mod
    lg = 20
    n = 1 << lg
    G = byo.Graph.generate(ctx, "rmat", seed=8, lg_n=lg, draws=1 << 21, container="pma")
    s, d = O.rmat_edges(8, lg, 1 << 21)
    off, nb = O.build_csr(n, s, d)
    st = O.Store(off, nb)
    us, ud = O.uniform_pairs(301, n, 1_200_000)
    keys = O.keys_from_pairs(us, ud)
    assert len(keys) > (1 << 21)
    assert G.insert_batch(keys) == st.insert_batch(keys)
    ro, rn = st.export_csr()
    _check_view(byo, O, G, ro, rn, (10,))
    rng = np.random.default_rng(4)
    # 16000 pairs with src < 4096 (one coarse bin) and two sources with 2000 keys each
    ls = rng.integers(0, 4096, 16000)
    ld = rng.integers(0, n, 16000)
    hub = np.concatenate([np.full(2000, 7), np.full(2000, 3000)])
    hd = np.concatenate([rng.choice(n, 2000, replace=False), rng.choice(n, 2000, replace=False)])
    skew = O.keys_from_pairs(np.concatenate([us[:1_100_000], ls, hub]), np.concatenate([ud[:1_100_000], ld, hd]))
    assert G.remove_batch(skew) == st.remove_batch(skew)
    assert G.insert_batch(skew) == st.insert_batch(skew)
    ro, rn = st.export_csr()
    _check_view(byo, O, G, ro, rn, (5,))
    G.close()


def _stream_batches(O, rng, n, sizes, halves=False):
    """Symmetrised batches of `sizes` random pairs (and of the first half of
    each batch's pairs, so that removing them keeps the graph undirected)."""
    out, half = [], []
    for k in sizes:
        pairs = rng.integers(0, n, size=(k, 2))
        out.append(O.keys_from_pairs(pairs[:, 0], pairs[:, 1]))
        half.append(O.keys_from_pairs(pairs[: k // 2, 0], pairs[: k // 2, 1]))
    return (out, half) if halves else out


@pytest.mark.gpu
def test_update_stream_matches_batch_by_batch(ctx, oracle_mod):
    """byo_graph_update_stream: runs of small batches in one persistent
    kernel give the oracle's per-batch changed counts and contents; a batch
    of more than 4096 keys in between takes the ordinary update."""
    import byo_gb300 as byo
    O = oracle_mod
    n = 1 << 15
    G = byo.Graph.generate(ctx, "rmat", seed=61, lg_n=15, draws=1 << 19, container="pma")
    s, d = O.rmat_edges(61, 15, 1 << 19)
    off, nb = O.build_csr(n, s, d)
    st = O.Store(off, nb)
    rng = np.random.default_rng(7)
    sizes = [1, 3, 40, 700, 1, 2000, 9000, 64, 5, 300]
    ins, halves = _stream_batches(O, rng, n, sizes, halves=True)
    batches = ins + [ins[i] for i in (3, 0, 6, 9)] + [halves[5]]
    ops = [True] * len(ins) + [False] * 5
    exp = [st.insert_batch(b) if op else st.remove_batch(b) for b, op in zip(batches, ops)]
    got = G.update_stream(batches, ops)
    assert got.tolist() == exp
    ro, rn = st.export_csr()
    _check_view(byo, O, G, ro, rn, (0, 3))
    G.close()


@pytest.mark.gpu
def test_update_stream_overflow_shrink_invalid(ctx, oracle_mod):
    """A batch that overflows a leaf stops the persistent kernel, is finished
    on the windowed path, and the stream resumes; removes that shrink the
    array rebuild it; a key >= n stops the stream with the batches before it
    applied."""
    import byo_gb300 as byo
    O = oracle_mod
    n = 1 << 12
    G = byo.Graph.generate(ctx, "rmat", seed=62, lg_n=12, draws=1 << 15, container="pma")
    s, d = O.rmat_edges(62, 12, 1 << 15)
    off, nb = O.build_csr(n, s, d)
    st = O.Store(off, nb)
    rng = np.random.default_rng(8)
    # 600 new neighbours of one vertex overflow its leaf
    hub = O.keys_from_pairs(np.full(600, 77), rng.choice(n, 600, replace=False))
    small = _stream_batches(O, rng, n, [50, 20, 5])
    batches = [small[0], hub, small[1], small[2]]
    ops = [True, True, True, True]
    exp = [st.insert_batch(b) for b in batches]
    assert G.update_stream(batches, ops).tolist() == exp
    ro, rn = st.export_csr()
    _check_view(byo, O, G, ro, rn, (77,))
    # remove nearly everything in small batches: the array shrinks (rebuilds) on the way
    src = np.repeat(np.arange(n, dtype=np.uint64), np.diff(ro).astype(np.int64))
    und = src < rn.astype(np.uint64)  # each undirected edge once; its batch removes both directions
    us, ud = src[und], rn[und].astype(np.uint64)
    chunks = [O.keys_from_pairs(us[i:i + 1500], ud[i:i + 1500]) for i in range(0, len(us) - 1500, 1500)]
    exp = [st.remove_batch(c) for c in chunks]
    assert G.update_stream(chunks, [False] * len(chunks)).tolist() == exp
    ro, rn = st.export_csr()
    _check_view(byo, O, G, ro, rn, (0,))
    # an invalid key in the third batch: the first two are applied
    good = _stream_batches(O, rng, n, [10, 10])
    bad = np.array([(5 << 32) | n], np.uint64)
    with pytest.raises(byo.ByoError) as e:
        G.update_stream(good + [bad, good[0]], [True, True, True, True])
    assert e.value.code == byo._abi.BYO_EINVAL
    for b in good:
        st.insert_batch(b)
    ro, rn = st.export_csr()
    o2, n2 = G.export_csr()
    assert np.array_equal(o2, ro) and np.array_equal(n2, rn)
    G.close()

"""The Packed CSR container (BYO_CONTAINER_PCSR, the reference's PCSR target,
run_pcsr.cc:24-99): every batch gives the oracle's contents and changed
counts; leaves that overflow are redistributed over windows, the array grows
when the root is too dense and shrinks when a remove leaves it too sparse;
the per-vertex index the updates maintain (the container's own gapped view,
read by neighbors()) and the compact snapshot the traversals use both equal
the oracle's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check(byo, O, G, ro, rn, srcs=(0,), nbr_sample=64, seed=0):
    o2, n2 = G.export_csr()
    assert np.array_equal(o2, ro) and np.array_equal(n2, rn)
    n = len(ro) - 1
    assert G.M() == len(rn) and np.array_equal(G.degrees(), np.diff(ro).astype(np.uint32))
    assert G.nslots() % 512 == 0 and G.nslots() >= n + len(rn)
    # the gapped view: [vbeg[v], vbeg[v+1]) read directly from the packed array
    rng = np.random.default_rng(seed)
    vs = rng.choice(n, min(n, nbr_sample), replace=False) if n else []
    for v in list(vs) + [0, n - 1]:
        assert np.array_equal(G.neighbors(int(v)), rn[ro[v]:ro[v + 1]]), v
    for s in srcs:
        opar, olev = O.bfs(ro, rn, s)
        for pol in (0, 2, 4):
            par, lev = byo.BFS(G, s, policy=pol, levels=True)
            assert np.array_equal(lev, olev) and np.array_equal(par, opar), (s, pol)
    assert np.array_equal(byo.SimpleUnionAsync(G), O.cc(ro, rn))
    assert byo.Test_Map(G) == O.map_sum(ro, rn)


def test_pcsr_batches_match_oracle_and_pma(ctx, oracle_mod):
    import byo_gb300 as byo
    O = oracle_mod
    n = 1 << 14
    s, d = O.rmat_edges(81, 14, 1 << 17)
    off, nb = O.build_csr(n, s, d)
    G = byo.Graph.from_csr(ctx, off, nb, container="pcsr")
    assert G.container == "pcsr"
    P = byo.Graph.from_csr(ctx, off, nb, container="pma")
    st = O.Store(off, nb)
    _check(byo, O, G, off, nb)
    rng = np.random.default_rng(12)
    for size in (1, 5, 100, 3000, 60000):
        pairs = rng.integers(0, n, size=(size, 2))
        keys = O.keys_from_pairs(pairs[:, 0], pairs[:, 1])
        half = O.keys_from_pairs(pairs[: size // 2, 0], pairs[: size // 2, 1])
        exp = st.insert_batch(keys)
        assert G.insert_batch(keys) == exp and P.insert_batch(keys) == exp
        u = G.last_update_stats()
        assert u["leaf_slots"] == 512 and u["changed"] == exp and u["touched_leaves"] >= 1
        exp = st.remove_batch(half)
        assert G.remove_batch(half) == exp and P.remove_batch(half) == exp
        ro, rn = st.export_csr()
        _check(byo, O, G, ro, rn, seed=size)
    po, pn = P.export_csr()
    assert np.array_equal(po, ro) and np.array_equal(pn, rn)
    assert np.array_equal(byo.PageRank(G, 1e-6, 20), byo.PageRank(P, 1e-6, 20))
    # an update stream on this container: one update per batch
    b1 = O.keys_from_pairs(*rng.integers(0, n, size=(2, 40)))
    got = G.update_stream([b1, b1, b1], [True, False, True])
    assert got.tolist() == [st.insert_batch(b1), st.remove_batch(b1), st.insert_batch(b1)]
    ro, rn = st.export_csr()
    _check(byo, O, G, ro, rn)
    G.close()
    P.close()


def test_pcsr_windows_grow_and_shrink(ctx, oracle_mod):
    """A hub that gains thousands of neighbours overflows its leaves (windowed
    redistribution); a large batch pushes the root past its bound (a new,
    larger layout); removing nearly everything lays the array out smaller."""
    import byo_gb300 as byo
    O = oracle_mod
    n = 20000
    s, d = O.uniform_pairs(91, n, 30000)
    off, nb = O.build_csr(n, s, d)
    G = byo.Graph.from_csr(ctx, off, nb, container="pcsr")
    st = O.Store(off, nb)
    slots0 = G.nslots()
    rng = np.random.default_rng(92)
    # one vertex gains 6000 neighbours (both directions; a sorted batch)
    hub = np.unique(O.keys_from_pairs(np.full(6000, 17), rng.choice(n, 6000, replace=False)))
    assert G.insert_batch(hub, sorted=True) == st.insert_batch(hub)
    assert G.last_update_stats()["path"] == 2
    ro, rn = st.export_csr()
    _check(byo, O, G, ro, rn, (17, 3))
    # grow: three times the elements the array holds
    pairs = rng.integers(0, n, size=(3 * slots0 // 2, 2))
    keys = O.keys_from_pairs(pairs[:, 0], pairs[:, 1])
    assert G.insert_batch(keys) == st.insert_batch(keys)
    assert G.nslots() > slots0
    ro, rn = st.export_csr()
    _check(byo, O, G, ro, rn, (17, 3))
    big = G.nslots()
    # shrink: remove all but 150 undirected edges
    allk = (np.repeat(np.arange(n, dtype=np.uint64), np.diff(ro).astype(np.int64)) << np.uint64(32)) | rn
    lo = allk[(allk >> np.uint64(32)) < (allk & np.uint64(0xFFFFFFFF))][:150]
    keep = np.unique(np.concatenate([lo, ((lo & np.uint64(0xFFFFFFFF)) << np.uint64(32)) | (lo >> np.uint64(32))]))
    drop = np.setdiff1d(allk, keep)
    assert G.remove_batch(drop) == st.remove_batch(drop)
    assert G.nslots() < big
    ro, rn = st.export_csr()
    assert len(rn) == 300
    _check(byo, O, G, ro, rn, (0, int(keep[0] >> np.uint64(32))))
    # and back
    assert G.insert_batch(drop) == st.insert_batch(drop)
    ro, rn = st.export_csr()
    _check(byo, O, G, ro, rn, (17,))
    G.close()


def test_pcsr_edge_cases(ctx, oracle_mod):
    """No edges at all, isolated vertices around hubs, rejected batches that
    leave the container unchanged, empty batches, self loops."""
    import byo_gb300 as byo
    O = oracle_mod
    n = 5003
    G = byo.Graph.from_csr(ctx, np.zeros(n + 1, np.uint64), np.zeros(0, np.uint32), container="pcsr")
    st = O.Store(np.zeros(n + 1, np.uint64), np.zeros(0, np.uint32))
    ro, rn = st.export_csr()
    _check(byo, O, G, ro, rn)
    assert G.insert_batch(np.zeros(0, np.uint64)) == 0
    # edges only among the last ten vertices, and self loops
    tail = np.arange(n - 10, n, dtype=np.uint64)
    keys = np.unique(np.concatenate([(tail[:, None] << np.uint64(32)) | tail[None, :]]).ravel())
    assert G.insert_batch(keys) == st.insert_batch(keys)
    ro, rn = st.export_csr()
    _check(byo, O, G, ro, rn, (n - 1, 0))
    with pytest.raises(byo.ByoError) as e:
        G.insert_batch(np.array([(3 << 32) | 4, (n << 32) | 1], np.uint64))
    assert e.value.code == byo._abi.BYO_EINVAL
    with pytest.raises(byo.ByoError) as e:
        G.insert_batch(np.array([(5 << 32) | 1, (4 << 32) | 1], np.uint64), sorted=True)
    assert e.value.code == byo._abi.BYO_EINVAL
    with pytest.raises(byo.ByoError) as e:
        G.remove_batch(np.array([(5 << 32) | 1, (5 << 32) | 1], np.uint64), sorted=True)
    assert e.value.code == byo._abi.BYO_EINVAL
    _check(byo, O, G, ro, rn, (n - 1,))
    # removing absent keys and inserting present ones change nothing
    assert G.remove_batch(np.array([(1 << 32) | 2], np.uint64)) == 0
    assert G.insert_batch(keys[:7]) == 0
    assert G.remove_batch(keys) == st.remove_batch(keys) == len(keys)
    ro, rn = st.export_csr()
    _check(byo, O, G, ro, rn)
    G.close()


def test_pcsr_large_batch_generate(ctx, oracle_mod):
    """A generated RMAT graph in the PCSR container and a batch past the
    two-level sort's threshold (2^21 keys): the oracle's contents, the same as
    the PMA's, then removed again."""
    import byo_gb300 as byo
    O = oracle_mod
    lg = 18
    n = 1 << lg
    G = byo.Graph.generate(ctx, "rmat", seed=83, lg_n=lg, draws=1 << 22, container="pcsr")
    P = byo.Graph.generate(ctx, "rmat", seed=83, lg_n=lg, draws=1 << 22, container="pma")
    s, d = O.rmat_edges(83, lg, 1 << 22)
    ro, rn = O.build_csr(n, s, d)
    _check(byo, O, G, ro, rn, (10,))
    st = O.Store(ro, rn)
    rng = np.random.default_rng(84)
    pairs = rng.integers(0, n, size=(1200000, 2))
    keys = O.keys_from_pairs(pairs[:, 0], pairs[:, 1])
    assert len(keys) >= 1 << 21
    exp = st.insert_batch(keys)
    assert G.insert_batch(keys) == exp and P.insert_batch(keys) == exp
    ro, rn = st.export_csr()
    _check(byo, O, G, ro, rn, (10,))
    po, pn = P.export_csr()
    assert np.array_equal(po, ro) and np.array_equal(pn, rn)
    exp = st.remove_batch(keys)
    assert G.remove_batch(keys) == exp
    ro, rn = st.export_csr()
    _check(byo, O, G, ro, rn, (10,))
    G.close()
    P.close()


def test_pcsr_segment_list_overflow(ctx, oracle_mod):
    """Batches of at most one key per leaf take the segment-list merge; one
    that overflows a leaf goes on to the windowed redistribution from it, and
    small unsorted, sorted and invalid batches take the deferred validation."""
    import byo_gb300 as byo
    O = oracle_mod
    n = 100000
    s, d = O.uniform_pairs(95, n, 30000)
    off, nb = O.build_csr(n, s, d)
    G = byo.Graph.from_csr(ctx, off, nb, container="pcsr")
    st = O.Store(off, nb)
    leaves = G.nslots() // 512
    rng = np.random.default_rng(96)
    # 200 new neighbours of vertex 5 (400 keys, fewer than the leaves): its
    # leaf overflows inside a segment-list merge
    pairs = np.stack([np.full(200, 5), rng.choice(n, 200, replace=False)], 1)
    keys = O.keys_from_pairs(pairs[:, 0], pairs[:, 1])
    assert len(keys) <= leaves
    assert G.insert_batch(keys) == st.insert_batch(keys)
    assert G.last_update_stats()["path"] == 2
    ro, rn = st.export_csr()
    _check(byo, O, G, ro, rn, (5, 0))
    # small batches: unsorted with duplicates, sorted, removed again
    for size in (1, 7, 300):
        p = rng.integers(0, n, size=(size, 2))
        k = O.keys_from_pairs(p[:, 0], p[:, 1])
        k = np.concatenate([k, k[: size // 2]])
        assert G.insert_batch(k) == st.insert_batch(k)
        ks = np.unique(k)
        assert G.remove_batch(ks, sorted=True) == st.remove_batch(ks)
        assert G.insert_batch(ks, sorted=True) == st.insert_batch(ks)
    ro, rn = st.export_csr()
    _check(byo, O, G, ro, rn, (5,))
    with pytest.raises(byo.ByoError) as e:
        G.remove_batch(np.array([(2 << 32) | 3, (n << 32) | 3], np.uint64))
    assert e.value.code == byo._abi.BYO_EINVAL
    _check(byo, O, G, ro, rn)
    G.close()

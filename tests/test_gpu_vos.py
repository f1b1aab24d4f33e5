"""The vector-of-runs container (BYO_CONTAINER_VOS, the counterpart of
run_vector_pma.cc / run_vector_vector.cc): every batch gives the oracle's
contents and changed counts, runs that outgrow their regions are laid out
again, and the traversals on it equal the oracle's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check(byo, O, G, ro, rn, srcs=(0,)):
    o2, n2 = G.export_csr()
    assert np.array_equal(o2, ro) and np.array_equal(n2, rn)
    assert G.M() == len(rn) and np.array_equal(G.degrees(), np.diff(ro).astype(np.uint32))
    for s in srcs:
        opar, olev = O.bfs(ro, rn, s)
        for pol in (0, 2, 3, 4):
            par, lev = byo.BFS(G, s, policy=pol, levels=True)
            assert np.array_equal(lev, olev) and np.array_equal(par, opar), (s, pol)
    assert np.array_equal(byo.SimpleUnionAsync(G), O.cc(ro, rn))
    assert byo.Test_Map(G) == O.map_sum(ro, rn)


def test_vos_batches(ctx, oracle_mod):
    import byo_gb300 as byo
    O = oracle_mod
    n = 1 << 14
    s, d = O.rmat_edges(71, 14, 1 << 17)
    off, nb = O.build_csr(n, s, d)
    G = byo.Graph.from_csr(ctx, off, nb, container="vos")
    assert G.container == "vos"
    P = byo.Graph.from_csr(ctx, off, nb, container="pma")
    st = O.Store(off, nb)
    _check(byo, O, G, off, nb)
    rng = np.random.default_rng(11)
    for size in (1, 5, 100, 3000, 60000):
        pairs = rng.integers(0, n, size=(size, 2))
        keys = O.keys_from_pairs(pairs[:, 0], pairs[:, 1])
        half = O.keys_from_pairs(pairs[: size // 2, 0], pairs[: size // 2, 1])
        exp = st.insert_batch(keys)
        assert G.insert_batch(keys) == exp and P.insert_batch(keys) == exp
        exp = st.remove_batch(half)
        assert G.remove_batch(half) == exp and P.remove_batch(half) == exp
        ro, rn = st.export_csr()
        _check(byo, O, G, ro, rn)
    # one vertex gains thousands of neighbours (its run outgrows its region),
    # given as a sorted batch
    hub = O.keys_from_pairs(np.full(5000, 9), rng.choice(n, 5000, replace=False))
    hub = np.unique(hub)
    assert G.insert_batch(hub, sorted=True) == st.insert_batch(hub)
    ro, rn = st.export_csr()
    _check(byo, O, G, ro, rn, (9,))
    # the same contents as the PMA, and the same PageRank
    P.insert_batch(hub, sorted=True)
    po, pn = P.export_csr()
    assert np.array_equal(po, ro) and np.array_equal(pn, rn)
    assert np.array_equal(byo.PageRank(G, 1e-6, 20), byo.PageRank(P, 1e-6, 20))
    with pytest.raises(byo.ByoError) as e:
        G.insert_batch(np.array([(3 << 32) | 4, (n << 32) | 1], np.uint64))
    assert e.value.code == byo._abi.BYO_EINVAL
    o2, n2 = G.export_csr()
    assert np.array_equal(o2, ro) and np.array_equal(n2, rn)
    # an update stream on this container: one update per batch
    b1 = O.keys_from_pairs(*rng.integers(0, n, size=(2, 40)))
    got = G.update_stream([b1, b1], [True, False])
    assert got.tolist() == [st.insert_batch(b1), st.remove_batch(b1)]
    ro, rn = st.export_csr()
    _check(byo, O, G, ro, rn)
    G.close()
    P.close()


def test_vos_generate_and_empty(ctx, oracle_mod):
    import byo_gb300 as byo
    O = oracle_mod
    G = byo.Graph.generate(ctx, "rmat", seed=72, lg_n=12, draws=1 << 15, container="vos")
    s, d = O.rmat_edges(72, 12, 1 << 15)
    ro, rn = O.build_csr(1 << 12, s, d)
    _check(byo, O, G, ro, rn, (10,))
    st = O.Store(ro, rn)
    allk = (np.repeat(np.arange(1 << 12, dtype=np.uint64), np.diff(ro).astype(np.int64)) << np.uint64(32)) | rn
    assert G.remove_batch(allk) == st.remove_batch(allk) == len(rn)
    assert G.M() == 0
    eo, en = st.export_csr()
    _check(byo, O, G, eo, en)
    assert G.insert_batch(allk) == len(rn)
    _check(byo, O, G, ro, rn, (10,))
    G.close()


def test_vos_large_batch_matches_pma(ctx, oracle_mod):
    """A batch past the two-level sort's threshold (2^21 keys), runs that span
    many key chunks, and an empty batch: the VOS container keeps the oracle's
    contents, the same as the PMA's."""
    import byo_gb300 as byo
    O = oracle_mod
    lg = 18
    n = 1 << lg
    G = byo.Graph.generate(ctx, "rmat", seed=73, lg_n=lg, draws=1 << 22, container="vos")
    P = byo.Graph.generate(ctx, "rmat", seed=73, lg_n=lg, draws=1 << 22, container="pma")
    s, d = O.rmat_edges(73, lg, 1 << 22)
    ro, rn = O.build_csr(n, s, d)
    st = O.Store(ro, rn)
    rng = np.random.default_rng(74)
    pairs = rng.integers(0, n, size=(1200000, 2))
    keys = O.keys_from_pairs(pairs[:, 0], pairs[:, 1])
    assert len(keys) >= 1 << 21
    exp = st.insert_batch(keys)
    assert G.insert_batch(keys) == exp and P.insert_batch(keys) == exp
    ro, rn = st.export_csr()
    _check(byo, O, G, ro, rn, (10,))
    po, pn = P.export_csr()
    assert np.array_equal(po, ro) and np.array_equal(pn, rn)
    assert G.insert_batch(np.zeros(0, np.uint64)) == 0
    exp = st.remove_batch(keys)
    assert G.remove_batch(keys) == exp
    ro, rn = st.export_csr()
    _check(byo, O, G, ro, rn, (10,))
    G.close()
    P.close()

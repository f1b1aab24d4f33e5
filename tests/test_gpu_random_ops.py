"""Seeded random sequences of batch updates on every updatable container
(PMA, packed CSR, vector of runs) against the oracle's sorted-set store: the
changed count after every operation, the contents and degrees every few
operations, BFS and CC at the end.  Sizes are log-uniform from 1 to 2*10^4
pairs, so every update path runs (segment list and full-leaf merges, the
register, bucketed and unsorted sorts, leaf overflow, growth and shrinking);
batches come unsorted with duplicates or sorted and deduplicated, and removes
draw half their pairs from the edges present."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check(byo, O, G, st):
    ro, rn = st.export_csr()
    go, gn = G.export_csr()
    assert np.array_equal(go, ro) and np.array_equal(gn, rn)
    assert np.array_equal(G.degrees(), np.diff(ro).astype(np.uint32))
    return ro, rn


@pytest.mark.parametrize("container", ["pma", "pcsr", "vos"])
def test_random_update_sequence(ctx, oracle_mod, container):
    import byo_gb300 as byo
    O = oracle_mod
    lg = 14
    n = 1 << lg
    s, d = O.rmat_edges(101, lg, 1 << 16)
    off, nb = O.build_csr(n, s, d)
    G = byo.Graph.from_csr(ctx, off, nb, container=container)
    st = O.Store(off, nb)
    rng = np.random.default_rng(102)
    for op in range(40):
        size = int(np.round(10.0 ** rng.uniform(0, np.log10(2e4))))
        insert = bool(rng.integers(0, 2))
        if insert:
            p = rng.integers(0, n, size=(size, 2))
        else:
            # half the pairs from the edges present, half random
            ro, rn = st.export_csr()
            src = np.repeat(np.arange(n), np.diff(ro).astype(np.int64))
            pick = rng.integers(0, max(len(rn), 1), size=size // 2 + 1) if len(rn) else np.zeros(0, np.int64)
            p = np.concatenate([np.stack([src[pick], rn[pick]], 1) if len(rn) else np.zeros((0, 2), np.int64),
                                rng.integers(0, n, size=(size - size // 2, 2))])
        keys = O.keys_from_pairs(p[:, 0], p[:, 1])
        sorted_ = bool(rng.integers(0, 3) == 0)
        if sorted_:
            keys = np.unique(keys)
        else:
            keys = np.concatenate([keys, keys[: len(keys) // 5]])  # duplicates
            rng.shuffle(keys)
        if insert:
            assert G.insert_batch(keys, sorted=sorted_) == st.insert_batch(keys), (op, size)
        else:
            assert G.remove_batch(keys, sorted=sorted_) == st.remove_batch(keys), (op, size)
        assert G.M() == st.num_edges
        if op % 5 == 4:
            _check(byo, O, G, st)
    ro, rn = _check(byo, O, G, st)
    for src in (0, 7):
        opar, olev = O.bfs(ro, rn, src)
        par, lev = byo.BFS(G, src, levels=True)
        assert np.array_equal(lev, olev) and np.array_equal(par, opar)
    assert np.array_equal(byo.SimpleUnionAsync(G), O.cc(ro, rn))
    G.close()


@pytest.mark.parametrize("container", ["pma", "pcsr", "vos"])
def test_remove_with_absent_key_of_equal_rank(ctx, oracle_mod, container):
    """A remove batch whose absent key sorts just below a present one of the
    same vertex (both rank 1 in the vertex's run): the present one goes, the
    next vertex's neighbours are untouched."""
    import byo_gb300 as byo
    O = oracle_mod
    n = 64
    pairs = np.array([(3, 10), (3, 20), (3, 30), (4, 11), (4, 12), (5, 40), (9, 1)])
    off, nb = O.build_csr(n, pairs[:, 0].astype(np.uint32), pairs[:, 1].astype(np.uint32))
    G = byo.Graph.from_csr(ctx, off, nb, container=container)
    st = O.Store(off, nb)
    for batch, sorted_ in (([(3, 15), (3, 20), (3, 20)], False), ([(4, 10), (4, 11), (5, 39)], True),
                           ([(3, 29), (3, 30), (4, 12), (5, 41)], False)):
        k = np.array([(a << 32) | b for a, b in batch], np.uint64)
        k = np.unique(k) if sorted_ else k
        assert G.remove_batch(k, sorted=sorted_) == st.remove_batch(k)
        _check(byo, O, G, st)
    G.close()


@pytest.mark.parametrize("container", ["pma", "pcsr", "vos"])
def test_random_update_stream(ctx, oracle_mod, container):
    """60 seeded batches through byo_graph_update_stream (on the PMA drained by
    the persistent kernel, larger batches by the host between its launches):
    sizes log-uniform 1-3000 pairs, unsorted with duplicates, removes half of
    present edges; every batch's count and the final contents against the
    oracle."""
    import byo_gb300 as byo
    O = oracle_mod
    lg = 15
    n = 1 << lg
    s, d = O.rmat_edges(111, lg, 1 << 17)
    off, nb = O.build_csr(n, s, d)
    G = byo.Graph.from_csr(ctx, off, nb, container=container)
    st = O.Store(off, nb)
    rng = np.random.default_rng(112)
    batches, ops = [], []
    shadow = O.Store(off, nb)  # to draw removes from edges present at that point
    for b in range(60):
        size = int(np.round(10.0 ** rng.uniform(0, np.log10(3000))))
        insert = bool(rng.integers(0, 2))
        if insert:
            p = rng.integers(0, n, size=(size, 2))
        else:
            ro, rn = shadow.export_csr()
            src = np.repeat(np.arange(n), np.diff(ro).astype(np.int64))
            pick = rng.integers(0, len(rn), size=size // 2 + 1)
            p = np.concatenate([np.stack([src[pick], rn[pick]], 1), rng.integers(0, n, size=(size - size // 2, 2))])
        keys = O.keys_from_pairs(p[:, 0], p[:, 1])
        keys = np.concatenate([keys, keys[: len(keys) // 4]])
        rng.shuffle(keys)
        (shadow.insert_batch if insert else shadow.remove_batch)(keys)
        batches.append(keys)
        ops.append(insert)
    got = G.update_stream(batches, ops)
    exp = [st.insert_batch(k) if ins else st.remove_batch(k) for k, ins in zip(batches, ops)]
    assert got.tolist() == exp
    _check(byo, O, G, st)
    G.close()


@pytest.mark.parametrize("container", ["pma", "pcsr", "vos"])
def test_random_mixed_stream(ctx, oracle_mod, container):
    """30 seeded ops through byo_graph_mixed_stream: 16-source queries between
    batches of 1-3000 pairs (unsorted with duplicates, removes half of present
    edges); every query's levels, every batch's count and the final contents
    against the oracle at that point of the stream."""
    import torch

    import byo_gb300 as byo
    O = oracle_mod
    lg = 14
    n = 1 << lg
    s, d = O.rmat_edges(121, lg, 1 << 16)
    off, nb = O.build_csr(n, s, d)
    G = byo.Graph.from_csr(ctx, off, nb, container=container)
    st = O.Store(off, nb)
    shadow = O.Store(off, nb)
    rng = np.random.default_rng(122)
    ops = []
    for i in range(30):
        if rng.integers(0, 3) == 0:
            ops.append(("query", rng.integers(0, n, 16).astype(np.uint32)))
            continue
        size = int(np.round(10.0 ** rng.uniform(0, np.log10(3000))))
        insert = bool(rng.integers(0, 2))
        if insert:
            p = rng.integers(0, n, size=(size, 2))
        else:
            ro, rn = shadow.export_csr()
            src = np.repeat(np.arange(n), np.diff(ro).astype(np.int64))
            pick = rng.integers(0, len(rn), size=size // 2 + 1)
            p = np.concatenate([np.stack([src[pick], rn[pick]], 1), rng.integers(0, n, size=(size - size // 2, 2))])
        keys = O.keys_from_pairs(p[:, 0], p[:, 1])
        keys = np.concatenate([keys, keys[: len(keys) // 4]])
        rng.shuffle(keys)
        (shadow.insert_batch if insert else shadow.remove_batch)(keys)
        ops.append(("insert" if insert else "remove", keys))
    nq = sum(1 for kind, _ in ops if kind == "query")
    levels = torch.full((max(nq, 1) * 16 * n,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    changed, _ = G.mixed_stream(ops, 16, levels)
    lev = levels.cpu().numpy().view(np.uint32).reshape(-1, 16, n)
    q = 0
    for i, (kind, x) in enumerate(ops):
        if kind == "query":
            so, sn = st.export_csr()
            for j, src in enumerate(x):
                assert np.array_equal(lev[q, j], O.bfs(so, sn, int(src))[1]), "op %d source %d" % (i, j)
            q += 1
        else:
            exp = st.insert_batch(x) if kind == "insert" else st.remove_batch(x)
            assert changed[i] == exp, "op %d" % i
    _check(byo, O, G, st)
    G.close()


@pytest.mark.parametrize("container", ["pma", "pcsr", "vos"])
def test_rejected_batches_every_size(ctx, oracle_mod, container):
    """A batch with one key out of range (src = n, dst = n, or both 2^32 - 1),
    or a batch passed as sorted that is not, is rejected with BYO_EINVAL at
    every size -- the one-CTA register sort (<= 4096 keys), the bucketed and
    two-level sorts (2^21 keys and more), the segment-list and full-leaf
    merges -- and leaves the contents, degrees and edge count unchanged; the
    same batch without the bad key then applies as the oracle's store says."""
    import byo_gb300 as byo
    O = oracle_mod
    lg = 14
    n = 1 << lg
    s, d = O.rmat_edges(151, lg, 1 << 17)
    off, nb = O.build_csr(n, s, d)
    G = byo.Graph.from_csr(ctx, off, nb, container=container)
    st = O.Store(off, nb)
    rng = np.random.default_rng(152)
    bads = ((n << 32) | 1, (3 << 32) | n, (0xFFFFFFFF << 32) | 0xFFFFFFFF)
    # 3000 pairs again at the end: by then the graph has more leaves than
    # keys, so the segment list meets the bucketed sort
    for size in (1, 100, 3000, 20000, 300000, 1 << 21, 3000, 100):
        p = rng.integers(0, n, size=(size, 2))
        keys = O.keys_from_pairs(p[:, 0], p[:, 1])
        m_before = G.M()
        for bad in bads:
            k = keys.copy()
            k[int(rng.integers(0, len(k)))] = bad
            for op in (G.insert_batch, G.remove_batch):
                with pytest.raises(byo.ByoError) as e:
                    op(k)
                assert e.value.code == byo._abi.BYO_EINVAL, (size, hex(bad))
                assert G.M() == m_before, (size, hex(bad))
        u = np.unique(keys)
        if len(u) > 1:
            j = int(rng.integers(0, len(u) - 1))
            u[j], u[j + 1] = u[j + 1], u[j]
            for op in (G.insert_batch, G.remove_batch):
                with pytest.raises(byo.ByoError) as e:
                    op(u, sorted=True)
                assert e.value.code == byo._abi.BYO_EINVAL, (size, "order")
        ro, rn = st.export_csr()
        go, gn = G.export_csr()
        assert np.array_equal(go, ro) and np.array_equal(gn, rn), (size, "changed by a rejected batch")
        assert np.array_equal(G.degrees(), np.diff(ro).astype(np.uint32)), size
        assert G.insert_batch(keys) == st.insert_batch(keys), size
        half = keys[: len(keys) // 2]
        assert G.remove_batch(half) == st.remove_batch(half), size
        assert G.M() == st.num_edges, size
    _check(byo, O, G, st)
    G.close()

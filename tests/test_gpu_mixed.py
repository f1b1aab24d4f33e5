"""Update batches and 64-source BFS queries drained by one persistent kernel
(byo_graph_mixed_stream), against the oracle after every op.

A PMA on RMAT 2^16 takes a stream of ops in order: queries of 64 seeded
sources (some repeated), small insert and remove batches (merged inside the
kernel), a batch too large for the kernel (finished by the host between two
launches) and a batch aimed at one vertex, whose merge overflows a leaf (the
kernel stops, the host redistributes, the kernel resumes with the next op).
Every query's levels must equal the oracle's single-source BFS levels
(benchmarks/BFS/NonDeterministicBFS/BFS.h:47-64) on the contents at that point
of the stream; every batch's changed count and the final contents must equal
the oracle's sorted-set store (gbbs/graph.h:3071-3124 semantics).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_mixed_stream_matches_oracle_after_every_op(ctx, oracle_mod):
    import torch

    import byo_gb300 as byo
    O = oracle_mod
    lg = 16
    n = 1 << lg
    s, d = O.rmat_edges(17, lg, 1 << 20)
    off, nb = O.build_csr(n, s, d)
    G = byo.Graph.from_csr(ctx, off, nb, container="pma")
    st = O.Store(off, nb)
    rng = np.random.default_rng(5)
    deg = np.diff(off.astype(np.int64))

    def batch(seed, pairs):
        us, ud = O.uniform_pairs(seed, n, pairs)
        return O.keys_from_pairs(us, ud)

    def query():
        q = rng.choice(np.nonzero(deg)[0], 64).astype(np.uint32)
        q[3] = q[2]  # a repeated source
        return q

    # 750 new neighbours of a vertex of degree 1, both directions: the
    # vertex's leaf overflows
    v = np.uint64(int(np.nonzero(deg == 1)[0][0]))
    dst = rng.choice(np.nonzero(np.arange(n) != int(v))[0], 750, replace=False).astype(np.uint64)
    dense = np.concatenate([(v << np.uint64(32)) | dst, (dst << np.uint64(32)) | v])
    b1, b2, b3 = batch(61, 300), batch(62, 1000), batch(63, 40)
    big = batch(64, 20000)  # 40000 keys: the host path
    ops = [("query", query()), ("insert", b1), ("query", query()), ("remove", b2), ("insert", big),
           ("query", query()), ("insert", b3), ("insert", dense), ("query", query()), ("remove", b1),
           ("remove", dense), ("query", query())]
    nq = sum(1 for kind, _ in ops if kind == "query")
    levels = torch.full((nq * 64 * n,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()  # the fill is done before the library's stream writes
    changed, times = G.mixed_stream(ops, 64, levels)
    lev = levels.cpu().numpy().view(np.uint32).reshape(nq, 64, n)
    q = 0
    for i, (kind, x) in enumerate(ops):
        if kind == "query":
            so, sn = st.export_csr()
            for j, src in enumerate(x):
                assert np.array_equal(lev[q, j], O.bfs(so, sn, int(src))[1]), "query %d source %d" % (q, j)
            q += 1
            assert times[i, 1] >= times[i, 0] > 0
        else:
            exp = st.insert_batch(x) if kind == "insert" else st.remove_batch(x)
            assert changed[i] == exp, "op %d" % i
    so, sn = st.export_csr()
    go, gn = G.export_csr()
    assert np.array_equal(go, so) and np.array_equal(gn, sn)
    assert times[4].tolist() == [0, 0]  # the large batch ran on the host path
    G.close()


@pytest.mark.parametrize("container", ["pcsr", "vos"])
def test_mixed_stream_other_containers(ctx, oracle_mod, container):
    """The same stream API on the packed CSR and the vector of runs, which run
    it op by op: every query's levels and every batch's count against the
    oracle at its point of the stream; op times stay 0 there."""
    import torch

    import byo_gb300 as byo
    O = oracle_mod
    lg = 14
    n = 1 << lg
    s, d = O.rmat_edges(18, lg, 1 << 17)
    off, nb = O.build_csr(n, s, d)
    G = byo.Graph.from_csr(ctx, off, nb, container=container)
    st = O.Store(off, nb)
    rng = np.random.default_rng(6)
    deg = np.diff(off.astype(np.int64))

    def batch(seed, pairs):
        us, ud = O.uniform_pairs(seed, n, pairs)
        return O.keys_from_pairs(us, ud)

    def query():
        return rng.choice(np.nonzero(deg)[0], 16).astype(np.uint32)

    b1, b2 = batch(71, 500), batch(72, 20000)
    ops = [("query", query()), ("insert", b1), ("insert", b2), ("query", query()), ("remove", b1),
           ("query", query()), ("remove", b2)]
    nq = 3
    levels = torch.full((nq * 16 * n,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    changed, times = G.mixed_stream(ops, 16, levels)
    lev = levels.cpu().numpy().view(np.uint32).reshape(nq, 16, n)
    q = 0
    for i, (kind, x) in enumerate(ops):
        if kind == "query":
            so, sn = st.export_csr()
            for j, src in enumerate(x):
                assert np.array_equal(lev[q, j], O.bfs(so, sn, int(src))[1]), "query %d source %d" % (q, j)
            q += 1
        else:
            exp = st.insert_batch(x) if kind == "insert" else st.remove_batch(x)
            assert changed[i] == exp, "op %d" % i
    assert not times.any()
    so, sn = st.export_csr()
    go, gn = G.export_csr()
    assert np.array_equal(go, so) and np.array_equal(gn, sn)
    G.close()

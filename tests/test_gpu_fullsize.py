"""Parity at the benchmarked sizes, through the C ABI, against the oracle.

C1 (the reference's run_csr case): CSR on RMAT(.57, .19, .19) with 2^20
vertices and 2^24 draws, symmetrised and deduplicated: BFS from 10 (levels and
min-id parents), CC labels (minimum vertex id), PageRank with eps 1e-6.
C2 (the dynamic case): RMAT with 2^22 vertices and 2^26 draws in each
updatable container (the packed-memory array, the packed CSR, the vector of
sorted runs); a batch of 10^7 uniform pairs (2*10^7 directed
keys, unsorted) inserted and then removed, plus 10^3 and 10^5 pair batches:
after every batch the sorted adjacency and the changed-key count equal the
oracle's sorted-set store (gbbs/graph.h:3071-3124 semantics), and BFS(10) and
CC are bit-exact on the updated graph; PageRank after the large insert.
Tolerances: integer results bit-exact; PageRank FP32-Kahan L1 <= 1e-6 and
FP64 L1 <= 1e-12 against the FP64 oracle (benchmarks/PageRank/PageRank.h:125-193).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PR_L1_FP32_KAHAN = 1e-6
PR_L1_FP64 = 1e-12


def _check_traversals(byo, O, G, off, nb, pagerank=True):
    par, lev = byo.BFS(G, 10, levels=True)
    opar, olev = O.bfs(off, nb, 10)
    assert np.array_equal(lev, olev), "BFS levels differ"
    assert np.array_equal(par, opar), "BFS parents differ"
    par_l = byo.BFS(G, 10, policy=byo._abi.POLICY_LEARNED)
    assert np.array_equal(par_l, opar), "BFS parents differ under the learned policy"
    assert np.array_equal(byo.SimpleUnionAsync(G), O.cc(off, nb)), "CC labels differ"
    if pagerank:
        op, oit, _ = O.pagerank(off, nb, 1e-6, 20)
        p, it, _ = byo.PageRank(G, 1e-6, 20, info=True)
        assert it == oit
        l1 = float(np.abs(p - op).sum())
        assert l1 <= PR_L1_FP32_KAHAN, "PageRank FP32-Kahan L1 %.3g" % l1
        return l1
    return None


def test_c1_csr_rmat20(ctx, oracle_mod):
    import byo_gb300 as byo
    O = oracle_mod
    s, d = O.rmat_edges(1, 20, 1 << 24)
    off, nb = O.build_csr(1 << 20, s, d)
    del s, d
    G = byo.Graph.generate(ctx, "rmat", seed=1, lg_n=20, draws=1 << 24)
    go, gn = G.export_csr()
    assert np.array_equal(go, off) and np.array_equal(gn, nb), "generated C1 graph differs from the oracle's"
    _check_traversals(byo, O, G, off, nb)
    op, _, _ = O.pagerank(off, nb, 1e-6, 100)
    p64 = byo.PageRank(G, 1e-6, 100, precision=byo._abi.PR_FP64)
    assert float(np.abs(p64 - op).sum()) <= PR_L1_FP64
    G.close()


@pytest.mark.parametrize("container", ["pma", "pcsr", "vos"])
def test_c2_rmat22_batches(ctx, oracle_mod, container):
    import byo_gb300 as byo
    O = oracle_mod
    s, d = O.rmat_edges(1, 22, 1 << 26)
    off, nb = O.build_csr(1 << 22, s, d)
    del s, d
    n = 1 << 22
    G = byo.Graph.generate(ctx, "rmat", seed=1, lg_n=22, draws=1 << 26, container=container)
    go, gn = G.export_csr()
    assert np.array_equal(go, off) and np.array_equal(gn, nb), "generated C2 graph differs from the oracle's"
    del go, gn
    st = O.Store(off, nb)
    for pairs, seed in ((10_000_000, 1001), (1_000, 7), (100_000, 8)):
        us, ud = O.uniform_pairs(seed, n, pairs)
        keys = O.keys_from_pairs(us, ud)
        rng = np.random.default_rng(seed)
        keys = keys[rng.permutation(len(keys))]  # unsorted, as the workload specifies
        assert G.insert_batch(keys) == st.insert_batch(keys)
        so, sn = st.export_csr()
        go, gn = G.export_csr()
        assert np.array_equal(go, so) and np.array_equal(gn, sn), "contents differ after inserting %d pairs" % pairs
        del go, gn
        _check_traversals(byo, O, G, so, sn, pagerank=pairs == 10_000_000)
        rng.shuffle(keys)  # the reference shuffles the batch before removing it
        assert G.remove_batch(keys) == st.remove_batch(keys)
        so, sn = st.export_csr()
        go, gn = G.export_csr()
        assert np.array_equal(go, so) and np.array_equal(gn, sn), "contents differ after removing %d pairs" % pairs
        del go, gn
        _check_traversals(byo, O, G, so, sn, pagerank=False)
    G.close()

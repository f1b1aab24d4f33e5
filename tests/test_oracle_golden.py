"""The oracle against the golden vectors: the reference's own unit-test
expectations (test_bfs.cc, test_cc.cc) and networkx / numpy answers on the
reference's input graphs (tests/golden/make_golden.py)."""
import numpy as np
import pytest

NONE = 0xFFFFFFFF


def _csr(g):
    return np.array(g["offsets"], np.uint64), np.array(g["nbrs"], np.uint32)


def test_reference_bfs_vectors(golden, oracle_mod):
    seen = 0
    for g in golden["graphs"]:
        if "reference_bfs" not in g:
            continue
        off, nb = _csr(g)
        for src, allowed in g["reference_bfs"].items():
            par, _ = oracle_mod.bfs(off, nb, int(src))
            for v, choices in enumerate(allowed):
                assert int(par[v]) in choices, (g["name"], src, v, par[v], choices)
            seen += 1
    assert seen == 3


def test_reference_cc_partition(golden, oracle_mod):
    for g in golden["graphs"]:
        if "reference_cc_partition" not in g:
            continue
        off, nb = _csr(g)
        lab = oracle_mod.cc(off, nb)
        for block in g["reference_cc_partition"]:
            assert len({int(lab[v]) for v in block}) == 1
        reps = [int(lab[b[0]]) for b in g["reference_cc_partition"]]
        assert len(set(reps)) == len(reps)


@pytest.mark.parametrize("idx", range(5))
def test_graph_answers(golden, oracle_mod, idx):
    g = golden["graphs"][idx]
    off, nb = _csr(g)
    for src, exp in g["bfs"].items():
        par, lev = oracle_mod.bfs(off, nb, int(src))
        assert lev.tolist() == exp["level"]
        assert par.tolist() == exp["parent"]
    assert oracle_mod.cc(off, nb).tolist() == g["cc"]
    assert oracle_mod.bfs_cc(off, nb).tolist() == g["cc"]
    assert oracle_mod.triangle_count(off, nb) == g["triangles"]
    for key, pr in g["pagerank"].items():
        p, it, _ = oracle_mod.pagerank(off, nb, pr["eps"], pr["max_iters"])
        assert it == pr["iters"], key
        np.testing.assert_allclose(p, pr["p"], rtol=0, atol=1e-15)


def test_update_sequence(golden, oracle_mod):
    u = golden["updates"]
    off, nb = np.array(u["offsets"], np.uint64), np.array(u["nbrs"], np.uint32)
    st = oracle_mod.Store(off, nb)
    for b in u["batches"]:
        keys = np.array(b["keys"], np.uint64)
        ch = st.insert_batch(keys) if b["op"] == "insert" else st.remove_batch(keys)
        assert ch == b["changed"]
        o2, n2 = st.export_csr()
        assert o2.tolist() == b["offsets"]
        assert n2.tolist() == b["nbrs"]

"""The algorithmic-byte formulas bench.py divides by kernel time for the
roofline, checked against direct counts on small graphs (no GPU)."""
import itertools
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _csr(n, pairs):
    adj = [set() for _ in range(n)]
    for a, b in pairs:
        if a != b:
            adj[a].add(b)
            adj[b].add(a)
    off = np.zeros(n + 1, np.uint64)
    off[1:] = np.cumsum([len(x) for x in adj])
    nb = np.array([v for x in adj for v in sorted(x)], np.uint32)
    return off, nb, adj


def test_tc_dag_bytes_matches_direct_count():
    """4 * sum over DAG edges (rank by degree, then id) of d+(u) + d+(v)."""
    import bench
    rng = np.random.default_rng(5)
    for n, e in ((6, 9), (40, 150), (200, 1500)):
        off, nb, adj = _csr(n, rng.integers(0, n, size=(e, 2)).tolist())
        deg = [len(x) for x in adj]
        rank = {v: r for r, v in enumerate(sorted(range(n), key=lambda v: (deg[v], v)))}
        dag = [(u, v) for u in range(n) for v in adj[u] if rank[v] > rank[u]]
        dplus = [sum(1 for v in adj[u] if rank[v] > rank[u]) for u in range(n)]
        want = 4 * sum(dplus[u] + dplus[v] for u, v in dag)
        assert bench.tc_dag_bytes(off, nb) == (want, len(dag))


def test_tc_dag_edges_orient_every_triangle_once():
    """Every triangle has exactly one vertex whose two DAG successors close
    it, which is what the wedge count relies on."""
    rng = np.random.default_rng(6)
    n = 30
    _, _, adj = _csr(n, rng.integers(0, n, size=(120, 2)).tolist())
    deg = [len(x) for x in adj]
    rank = {v: r for r, v in enumerate(sorted(range(n), key=lambda v: (deg[v], v)))}
    out = [{v for v in adj[u] if rank[v] > rank[u]} for u in range(n)]
    wedges = sum(1 for u in range(n) for v in out[u] for w in out[v] if w in out[u])
    tri = sum(1 for a, b, c in itertools.combinations(range(n), 3) if b in adj[a] and c in adj[a] and c in adj[b])
    assert wedges == tri


def test_pagerank_iteration_bytes():
    """ids once per slot, one 4-byte gather per edge, offsets, degrees, and
    p_curr read / p_next and p_div written (FP32)."""
    import bench
    n, m = 1000, 7000
    assert bench.pr_iteration_bytes(n, m, m) == 4 * m + 4 * m + 8 * (n + 1) + 4 * n + 4 * n + 4 * n + 4 * n
    # a gapped view reads its gaps too, but gathers only for edges
    assert bench.pr_iteration_bytes(n, m, m + 500) - bench.pr_iteration_bytes(n, m, m) == 4 * 500


def test_update_bytes_per_container():
    """Batch update bytes: 16 B per key (sort read + write) plus each element
    of a touched leaf read and written: the PMA's 8-byte (src, dst) entries,
    the packed CSR's 4-byte slots and sentinel bits."""
    import bench
    B, E = 2 * 10 ** 7, 96_645_293
    assert bench.update_bytes(B, E, "pma") == 16 * B + 16 * E
    assert bench.update_bytes(B, E, "pcsr") == 16 * B + 8.25 * E
    assert bench.update_bytes(B, 0) == 16 * B

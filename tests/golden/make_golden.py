"""Generate the golden fixtures in tests/golden/golden.json.

Run once in a checkout that has the BYO reference tree beside it:

    python tests/golden/make_golden.py --reference /path/to/BYO

Sources of truth, none of which is the oracle under test:
  * the reference's own unit tests, restated as data:
      benchmarks/BFS/NonDeterministicBFS/unit_tests/test_bfs.cc:16-51
        (edgeless 3-vertex graph, BFS(1); 7-vertex graph, BFS(1), BFS(2) with
        AnyOf alternatives for the nondeterministic parents)
      benchmarks/Connectivity/unit_tests/test_cc.cc:16-43
        (same graphs; only the partition is checked there)
  * the reference's input graphs inputs/rMatGraph_J_5_100, inputs/star.txt,
    inputs/triangles.txt (AdjacencyGraph text, gbbs/graph_io.cc:35-100),
    answered by networkx (BFS levels, components, triangles) and by a numpy
    restatement of PageRank.h:125-193 written here independently of oracle.c;
  * a short insert/delete sequence on triangles.txt whose expected contents
    follow from Python set arithmetic (Graph::insert_batch / remove_batch,
    gbbs/graph.h:3071-3124: sort, unique, then union / difference).

The fixture is committed; the tests never read the reference tree.
"""
import argparse
import json
import os

import networkx as nx
import numpy as np

NONE = 0xFFFFFFFF
HERE = os.path.dirname(os.path.abspath(__file__))


def parse_adj(path):
    tok = open(path).read().split()
    assert tok[0] == "AdjacencyGraph"
    n, m = int(tok[1]), int(tok[2])
    off = [int(x) for x in tok[3:3 + n]] + [m]
    nbrs = [int(x) for x in tok[3 + n:3 + n + m]]
    return n, off, nbrs


def csr_from_undirected(n, edges):
    adj = [set() for _ in range(n)]
    for a, b in edges:
        adj[a].add(b)
        adj[b].add(a)
    off, nb = [0], []
    for v in range(n):
        nb.extend(sorted(adj[v]))
        off.append(len(nb))
    return off, nb


def to_nx(n, off, nb):
    g = nx.Graph()
    g.add_nodes_from(range(n))
    for v in range(n):
        for j in range(off[v], off[v + 1]):
            g.add_edge(v, nb[j])
    return g


def bfs_answer(g, n, src):
    dist = nx.single_source_shortest_path_length(g, src)
    level = [dist.get(v, NONE) for v in range(n)]
    parent = []
    for v in range(n):
        if v not in dist:
            parent.append(NONE)
        elif v == src:
            parent.append(src)
        else:
            parent.append(min(u for u in g[v] if dist.get(u) == dist[v] - 1))
    return level, parent


def cc_answer(g, n):
    lab = [0] * n
    for comp in nx.connected_components(g):
        m = min(comp)
        for v in comp:
            lab[v] = m
    return lab


def pagerank_answer(n, off, nb, eps, max_iters):
    """PageRank.h:125-193 (Jacobi order), written with numpy."""
    off = np.asarray(off, np.int64)
    nb = np.asarray(nb, np.int64)
    deg = np.diff(off).astype(np.float64)
    with np.errstate(divide="ignore"):
        p_curr = np.full(n, 1.0 / n)
        p_div = (1.0 / n) / deg
    added = (1 - 0.85) * (1 / n)
    it = 0
    while it < max_iters:
        it += 1
        p_next = np.empty(n)
        for v in range(n):
            s = 0.0
            for j in range(off[v], off[v + 1]):
                s += p_div[nb[j]]
            p_next[v] = 0.85 * s + added
        l1 = float(np.sum(np.abs(p_curr - p_next)))
        with np.errstate(divide="ignore"):
            p_div = p_next / deg
        if l1 < eps:
            break
        p_curr = p_next
    return [float(x) for x in p_next], it


def graph_entry(name, n, off, nb, sources, expect_bfs=None, expect_cc_partition=None):
    g = to_nx(n, off, nb)
    e = {"name": name, "n": n, "offsets": off, "nbrs": nb, "bfs": {}}
    for s in sources:
        level, parent = bfs_answer(g, n, s)
        e["bfs"][str(s)] = {"level": level, "parent": parent}
    e["cc"] = cc_answer(g, n)
    e["triangles"] = sum(nx.triangles(g).values()) // 3
    pr = {}
    for eps, iters in ((1e-6, 100), (1e-4, 20)):
        p, it = pagerank_answer(n, off, nb, eps, iters)
        pr[f"{eps:g}/{iters}"] = {"eps": eps, "max_iters": iters, "iters": it, "p": p}
    e["pagerank"] = pr
    if expect_bfs:
        e["reference_bfs"] = expect_bfs
    if expect_cc_partition:
        e["reference_cc_partition"] = expect_cc_partition
    return e


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="root of the BYO source tree")
    args = ap.parse_args()
    graphs = []

    # test_bfs.cc:16-24 / test_cc.cc:16-24: edgeless graph on 3 vertices
    off, nb = csr_from_undirected(3, [])
    graphs.append(graph_entry(
        "test_bfs_edgeless", 3, off, nb, [1],
        expect_bfs={"1": [[NONE], [1], [NONE]]},
        expect_cc_partition=[[0], [1], [2]]))
    # test_bfs.cc:26-50 / test_cc.cc:26-42: 0-1  2-3-4, 3-5, 4-5, 5-6
    edges = [(0, 1), (2, 3), (3, 4), (3, 5), (4, 5), (5, 6)]
    off, nb = csr_from_undirected(7, edges)
    graphs.append(graph_entry(
        "test_bfs_basic", 7, off, nb, [1, 2],
        expect_bfs={
            "1": [[1], [1], [NONE], [NONE], [NONE], [NONE], [NONE]],
            "2": [[NONE], [NONE], [2], [2], [3, 5], [3, 4], [5]],
        },
        expect_cc_partition=[[0, 1], [2, 3, 4, 5, 6]]))

    for fname, srcs in (("rMatGraph_J_5_100", [0, 10, 77]), ("star.txt", [0, 3]),
                        ("triangles.txt", [0, 4])):
        n, off, nb = parse_adj(os.path.join(args.reference, "inputs", fname))
        graphs.append(graph_entry("inputs/" + fname, n, off, nb, srcs))

    # update sequence on triangles.txt
    n, off, nb = parse_adj(os.path.join(args.reference, "inputs", "triangles.txt"))
    cur = {(v, nb[j]) for v in range(n) for j in range(off[v], off[v + 1])}
    seq = []
    batches = [
        ("insert", [(0, 3), (3, 0), (0, 3), (1, 1), (4, 0), (0, 4)]),   # dup + self loop
        ("insert", [(2, 3), (1, 4), (4, 1)]),                          # (2,3) already present
        ("remove", [(0, 3), (0, 3), (2, 4), (3, 3)]),                  # (3,3) absent
        ("remove", [(0, 1), (1, 0), (1, 2), (2, 1), (0, 2), (2, 0)]),
        ("insert", []),
    ]
    for op, pairs in batches:
        keys = [(a << 32) | b for a, b in pairs]
        if op == "insert":
            changed = len(set(pairs) - cur)
            cur |= set(pairs)
        else:
            changed = len(set(pairs) & cur)
            cur -= set(pairs)
        o2, n2 = [0], []
        for v in range(n):
            n2.extend(sorted(b for a, b in cur if a == v))
            o2.append(len(n2))
        seq.append({"op": op, "keys": keys, "changed": changed, "offsets": o2, "nbrs": n2})
    updates = {"graph": "inputs/triangles.txt", "n": n, "offsets": off, "nbrs": nb, "batches": seq}

    out = {"generated_by": "tests/golden/make_golden.py", "graphs": graphs, "updates": updates}
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote", os.path.join(HERE, "golden.json"))


if __name__ == "__main__":
    main()

"""Graph files in the reference's formats (gbbs/graph_io.cc:35-95): the
library's host parser against files written here from the golden graphs,
both layouts, and malformed files.  No device is needed."""
import numpy as np
import pytest


def _write_text(path, off, nb):
    with open(path, "w") as f:
        f.write("AdjacencyGraph\n%d\n%d\n" % (len(off) - 1, len(nb)))
        f.write("".join("%d\n" % x for x in off[:-1]))
        f.write("".join("%d\n" % x for x in nb))


def _write_binary(path, off, nb):
    n, m = len(off) - 1, len(nb)
    with open(path, "wb") as f:
        f.write(np.array([n, m, 24 + 8 * (n + 1) + 4 * m], np.int64).tobytes())
        f.write(np.asarray(off, np.uint64).tobytes())
        f.write(np.asarray(nb, np.uint32).tobytes())


@pytest.fixture(scope="module")
def lib_built():
    from byo_gb300 import build as nb
    nb.build()


def test_golden_graphs_both_layouts(golden, tmp_path, lib_built):
    from byo_gb300.graph import read_adj_host
    for g in golden["graphs"]:
        off = np.array(g["offsets"], np.uint64)
        nb = np.array(g["nbrs"], np.uint32)
        t = tmp_path / "g.adj"
        b = tmp_path / "g.bin"
        _write_text(t, off, nb)
        _write_binary(b, off, nb)
        for path, binary in ((t, False), (b, True)):
            o2, n2 = read_adj_host(str(path), binary)
            assert np.array_equal(o2, off) and np.array_equal(n2, nb)


def test_large_text_parses_in_parallel(oracle_mod, tmp_path, lib_built):
    """Above a megabyte the text is parsed by several threads."""
    from byo_gb300.graph import read_adj_host
    s, d = oracle_mod.rmat_edges(5, 16, 1 << 19)
    off, nb = oracle_mod.build_csr(1 << 16, s, d)
    t = tmp_path / "big.adj"
    with open(t, "w") as f:  # irregular whitespace between tokens
        f.write("AdjacencyGraph  %d\r\n%d\n" % (len(off) - 1, len(nb)))
        f.write(" ".join("%d" % x for x in off[:-1]) + "\n\t")
        f.write("\n".join("%d" % x for x in nb) + "\n\n")
    assert t.stat().st_size > (1 << 20)
    o2, n2 = read_adj_host(str(t))
    assert np.array_equal(o2, off) and np.array_equal(n2, nb)


@pytest.mark.parametrize("body", ["WeightedAdjacencyGraph\n1\n0\n0\n", "AdjacencyGraph\n2\n", "AdjacencyGraph\n2\n2\n0\n",
                                  "AdjacencyGraph\n2\n2\n0\n1\n1\nx\n", "AdjacencyGraph\n2\n2\n0\n1\n1\n2\n",
                                  "AdjacencyGraph\n2\n2\n1\n1\n1\n0\n", "AdjacencyGraph\n2\n1\n0\n2\n1\n"])
def test_malformed_text(tmp_path, body, lib_built):
    from byo_gb300 import ByoError
    from byo_gb300.graph import read_adj_host
    p = tmp_path / "bad.adj"
    p.write_text(body)
    with pytest.raises(ByoError):
        read_adj_host(str(p))


def test_malformed_binary(tmp_path, lib_built):
    from byo_gb300 import ByoError
    from byo_gb300.graph import read_adj_host
    p = tmp_path / "bad.bin"
    p.write_bytes(np.array([4, 10, 0], np.int64).tobytes() + np.zeros(5, np.uint64).tobytes())
    with pytest.raises(ByoError):
        read_adj_host(str(p), True)
    with pytest.raises(ByoError):
        read_adj_host(str(tmp_path / "missing.bin"), True)

"""byte-PD compressed graphs (gbbs/encodings/byte_pd_amortized.h): the GPU
encoder is byte-identical to the oracle's restatement, the GPU decoder
inverts it for every block size, the reference's file layout round-trips,
and malformed data is rejected without a fault."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _graphs(byo, ctx):
    return [byo.Graph.generate(ctx, "rmat", seed=51, lg_n=16, draws=1 << 20),
            byo.Graph.generate(ctx, "grid", n=40, draws=50),
            byo.Graph.generate(ctx, "rmat", seed=52, lg_n=13, draws=1 << 16, container="pma")]


def test_encode_matches_oracle_and_decodes(ctx, oracle_mod):
    import byo_gb300 as byo
    O = oracle_mod
    for G in _graphs(byo, ctx):
        off, nb = G.export_csr()
        assert int(np.diff(off).max()) > 0
        for P in (1000, 256, 7, 1):
            bo, dg, data = G.to_bytepd(P)
            obo, odg, odata = O.bytepd_encode(off, nb, P)
            assert np.array_equal(bo, obo) and np.array_equal(dg, odg) and bytes(data) == bytes(odata), P
            for cont in ("csr", "pma", "pcsr"):
                H = byo.Graph.from_bytepd(ctx, obo, odg, odata, block=P, container=cont)
                o2, n2 = H.export_csr()
                assert np.array_equal(o2, off) and np.array_equal(n2, nb), (P, cont)
                H.close()
        G.close()


def test_hub_blocks_and_bfs(ctx, oracle_mod):
    """A vertex with more than 1000 neighbours spans several blocks; BFS on
    the decoded graph equals the oracle's."""
    import byo_gb300 as byo
    O = oracle_mod
    n = 5000
    src = np.concatenate([np.full(4000, 17), np.arange(0, 4999)])
    dst = np.concatenate([np.arange(1000, 5000), np.arange(1, 5000)])
    off, nb = O.build_csr(n, src, dst)
    assert int(np.diff(off).max()) > 3000
    bo, dg, data = O.bytepd_encode(off, nb, 1000)
    G = byo.Graph.from_bytepd(ctx, bo, dg, data)
    o2, n2 = G.export_csr()
    assert np.array_equal(o2, off) and np.array_equal(n2, nb)
    opar, olev = O.bfs(off, nb, 17)
    par, lev = byo.BFS(G, 17, levels=True)
    assert np.array_equal(par, opar) and np.array_equal(lev, olev)
    G.close()


def test_file_round_trip(ctx, oracle_mod, tmp_path):
    import byo_gb300 as byo
    O = oracle_mod
    G = byo.Graph.generate(ctx, "rmat", seed=53, lg_n=14, draws=1 << 17)
    off, nb = G.export_csr()
    path = os.fspath(tmp_path / "g.bytepda")
    G.write_bytepd(path)
    # the reference's layout: int64 n, m, bytes; uint64 offsets; uint32 degrees; bytes
    raw = open(path, "rb").read()
    n, m, total = np.frombuffer(raw[:24], np.int64)
    bo, dg, data = O.bytepd_encode(off, nb, 1000)
    assert (n, m, total) == (len(off) - 1, len(nb), len(data))
    assert raw[24:24 + 8 * (n + 1)] == bo.tobytes() and raw[24 + 8 * (n + 1):24 + 8 * (n + 1) + 4 * n] == dg.tobytes()
    assert raw[24 + 12 * n + 8:] == bytes(data)
    for cont in ("csr", "pma", "pcsr"):
        H = byo.Graph.read_bytepd(ctx, path, container=cont)
        o2, n2 = H.export_csr()
        assert np.array_equal(o2, off) and np.array_equal(n2, nb)
        H.close()
    G.close()


def test_malformed_rejected(ctx, oracle_mod, tmp_path):
    import byo_gb300 as byo
    O = oracle_mod
    s, d = O.rmat_edges(54, 10, 1 << 13)
    off, nb = O.build_csr(1 << 10, s, d)
    bo, dg, data = O.bytepd_encode(off, nb, 1000)
    cases = []
    cases.append((bo, dg, data[:-3]))                        # bytes shorter than the offsets say
    bad = dg.copy()
    v = int(np.flatnonzero(bad)[0])
    bad[v] += 1
    cases.append((bo, bad, data))                            # degree header mismatch
    junk = data.copy()
    junk[int(bo[v]) + 8:int(bo[v + 1])] = 0xFF              # an integer that never ends
    cases.append((bo, dg, junk))
    zero = data.copy()
    zero[int(bo[v]) + 8:int(bo[v + 1])] = 0x00              # zero differences (no such encoding)
    cases.append((bo, dg, zero))
    for b_, d_, x_ in cases:
        with pytest.raises(byo.ByoError) as e:
            byo.Graph.from_bytepd(ctx, b_, d_, x_)
        assert e.value.code == byo._abi.BYO_EINVAL
    p = os.fspath(tmp_path / "short.bytepda")
    open(p, "wb").write(np.array([len(dg), len(nb), len(data)], np.int64).tobytes() + bo.tobytes())
    with pytest.raises(byo.ByoError):
        byo.Graph.read_bytepd(ctx, p)
    # the context stays usable
    G = byo.Graph.from_bytepd(ctx, bo, dg, data)
    assert G.M() == len(nb)
    G.close()

"""Where FP32-Kahan PageRank matters: a hub of degree 2^26.

The PageRank pull sums a vertex's gathered p/deg values in a fixed blocked
order (512-slot chunks, 16 values per lane, a warp tree, then the chunk
partials 32-strided and a warp tree).  On the benchmark graphs the FP32 error
is set by storing p in FP32 (L1 ~1e-7 with or without compensation).  A star
whose centre has 2^26 leaves makes the centre's sum long enough (131072
chunks, 4096 partials per lane) for uncompensated FP32 rounding to build up:
all leaves hold the same value, so the rounding errors do not cancel.  Plain
FP32 then misses the 1e-6 L1 bound against the FP64 oracle
(benchmarks/PageRank/PageRank.h:125-193, 20 iterations) while the compensated
(TwoSum) sums stay inside it (measured on GB300: FP32 5.6e-5, FP32-Kahan
1.5e-7, FP64 1.5e-10).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_kahan_holds_where_plain_fp32_fails(ctx, oracle_mod):
    import byo_gb300 as byo
    from byo_gb300 import _abi
    O = oracle_mod
    D = 1 << 26
    n = D + 1
    off = np.empty(n + 1, np.uint64)
    off[0] = 0
    off[1:] = D + np.arange(n, dtype=np.uint64)  # centre: D slots; each leaf: 1
    nb = np.empty(2 * D, np.uint32)
    nb[:D] = np.arange(1, n, dtype=np.uint32)
    nb[D:] = 0
    op, oit, _ = O.pagerank(off, nb, 0.0, 20)
    G = byo.Graph.from_csr(ctx, off, nb)
    del nb
    l1 = {}
    for name, prec in (("fp32", _abi.PR_FP32), ("fp32_kahan", _abi.PR_FP32_KAHAN), ("fp64", _abi.PR_FP64)):
        p, it, _ = byo.PageRank(G, 0.0, 20, precision=prec, info=True)
        assert it == oit == 20
        l1[name] = float(np.abs(p - op).sum())
    print("star 2^26: L1 vs FP64 oracle", l1)
    # the oracle's own left-to-right FP64 sum of 2^26 equal terms carries up to
    # ~2^26 * 2^-53 relative error, so FP64 agrees only to ~1e-9 here
    assert l1["fp64"] <= 1e-8
    assert l1["fp32_kahan"] <= 1e-6
    assert l1["fp32"] > 1e-6
    G.close()

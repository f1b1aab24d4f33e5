"""The bounded device waits' error path, made to run out on purpose.

The persistent kernels (runs of small BFS push rounds, the 64-source bit-lane
BFS, the update stream) separate their phases with a grid barrier that gives
up after a time limit, sets an error word and returns, so a wait that cannot
complete never hangs the GPU.  byo_ctx_set_barrier_test shortens the limit to
1 ms and makes every barrier wait for one more block than was launched: no
barrier can complete, every block leaves after 1 ms, and the call must return
BYO_ETIMEDOUT.  Afterwards, with the default restored, the same context must
give the oracle's answers (the context survived) and an update stream that
timed out before its first merge must have left the container unchanged.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _barrier_test(ctx, limit_ms, extra):
    from byo_gb300 import _abi
    _abi.check(_abi.lib().byo_ctx_set_barrier_test(ctx.h, limit_ms, extra), ctx.h)


def test_barrier_timeout_reports_and_context_survives(ctx, oracle_mod):
    import byo_gb300 as byo
    from byo_gb300 import _abi
    O = oracle_mod
    # a 64 x 64 grid: every BFS round is small, so the rounds run in the
    # persistent small-round kernel
    G = byo.Graph.generate(ctx, "grid", n=64, draws=64)
    off, nb = G.export_csr()
    exp_par, exp_lev = O.bfs(off, nb, 0)
    P = byo.Graph.generate(ctx, "rmat", seed=3, lg_n=16, draws=1 << 19, container="pma")
    po, pn = P.export_csr()
    batches = [O.keys_from_pairs(*O.uniform_pairs(40 + i, 1 << 16, 50 + 30 * i)) for i in range(3)]
    try:
        # out-of-range settings are refused
        assert _abi.lib().byo_ctx_set_barrier_test(ctx.h, 5000, 0) == _abi.BYO_EINVAL
        assert _abi.lib().byo_ctx_set_barrier_test(ctx.h, 1, 2) == _abi.BYO_EINVAL
        _barrier_test(ctx, 1, 1)
        with pytest.raises(_abi.ByoError) as e:
            byo.BFS(G, 0)
        assert e.value.code == _abi.BYO_ETIMEDOUT
        with pytest.raises(_abi.ByoError) as e:
            byo.BFS_multi(G, [0, 5, 4095])
        assert e.value.code == _abi.BYO_ETIMEDOUT
        with pytest.raises(_abi.ByoError) as e:
            P.update_stream(batches, [True, True, False])
        assert e.value.code == _abi.BYO_ETIMEDOUT
    finally:
        _barrier_test(ctx, 0, 0)
    # the context is usable and the results are the oracle's
    par, lev = byo.BFS(G, 0, levels=True)
    assert np.array_equal(par, exp_par) and np.array_equal(lev, exp_lev)
    lv = byo.BFS_multi(G, [0, 5, 4095])
    for i, s in enumerate([0, 5, 4095]):
        assert np.array_equal(lv[i], O.bfs(off, nb, s)[1])
    # the stream stopped at its first barrier, before any merge
    qo, qn = P.export_csr()
    assert np.array_equal(qo, po) and np.array_equal(qn, pn)
    st = O.Store(po, pn)
    exp = [st.insert_batch(batches[0]), st.insert_batch(batches[1]), st.remove_batch(batches[2])]
    assert P.update_stream(batches, [True, True, False]).tolist() == exp
    so, sn = st.export_csr()
    qo, qn = P.export_csr()
    assert np.array_equal(qo, so) and np.array_equal(qn, sn)
    G.close()
    P.close()

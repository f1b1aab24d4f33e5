"""The allocation-free BFS entry point (byo_bfs_csr_noalloc) against the oracle.

Callers whose memory manager owns the whole GPU and hands out sub-ranges
itself cannot let a library call cudaMalloc; they get a BFS whose state lives
in a fixed static device array.  This test calls it through the C ABI on CSRs
the test placed on the device, several times in a row (a call must not see
the previous call's leftovers in the shared array), and checks parents and
levels against the CPU oracle bit for bit, and against the allocating entry
point.  Cases: a graph at the array's full capacity (2^20 vertices), a small
graph whose vertex count is not a multiple of 32 (partial last bitmap word),
an isolated source (degree 0: the first round finds nothing), and the
rejection of src >= n and n beyond the capacity.  It sits in its own file,
named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(L, off_t, nb_t, n, m, src, par_t, lev_t, stream):
    rounds = ctypes.c_uint32(0)
    rc = L.byo_bfs_csr_noalloc(off_t.data_ptr(), nb_t.data_ptr(), n, m, src, par_t.data_ptr(),
                               lev_t.data_ptr(), stream, ctypes.byref(rounds))
    return rc, rounds.value


def _to_device(torch, off, nb):
    off_t = torch.from_numpy(off.view(np.int64).copy()).cuda()
    nb_t = torch.from_numpy(nb.view(np.int32).copy()).cuda() if len(nb) else torch.zeros(1, dtype=torch.int32,
                                                                                         device="cuda")
    return off_t, nb_t


def test_noalloc_bfs_matches_oracle(ctx, oracle_mod):
    import torch

    import byo_gb300 as byo
    from byo_gb300 import _abi
    O = oracle_mod
    L = _abi.lib()
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream().cuda_stream

    # the array's full capacity: RMAT 2^20
    s, d = O.rmat_edges(21, 20, 1 << 23)
    off, nb = O.build_csr(1 << 20, s, d)
    n, m = len(off) - 1, len(nb)
    assert n == _abi.NOALLOC_MAX_VERTICES
    off_t, nb_t = _to_device(torch, off, nb)
    par_t = torch.empty(n, dtype=torch.int32, device="cuda")
    lev_t = torch.empty(n, dtype=torch.int32, device="cuda")
    deg = np.diff(off.astype(np.int64))
    hub = int(np.argmax(deg))
    G = byo.Graph.from_csr(ctx, off, nb)
    for src in (10, hub):  # two calls in a row on the shared scratch
        rc, rounds = _noalloc(L, off_t, nb_t, n, m, src, par_t, lev_t, stream)
        assert rc == _abi.BYO_OK
        exp_par, exp_lev = O.bfs(off, nb, src)
        got_par = par_t.cpu().numpy().view(np.uint32)
        got_lev = lev_t.cpu().numpy().view(np.uint32)
        assert np.array_equal(got_par, exp_par)
        assert np.array_equal(got_lev, exp_lev)
        # and the allocating entry point agrees
        a_par, a_lev = byo.BFS(G, src, levels=True)
        assert np.array_equal(got_par, a_par) and np.array_equal(got_lev, a_lev)
        assert rounds > 0
    G.close()
    # n beyond the static capacity, and a source outside the graph, are refused
    rc, _ = _noalloc(L, off_t, nb_t, n + 1, m, 0, par_t, lev_t, stream)
    assert rc == _abi.BYO_EINVAL
    rc, _ = _noalloc(L, off_t, nb_t, n, m, n, par_t, lev_t, stream)
    assert rc == _abi.BYO_EINVAL

    # a vertex count that is not a multiple of 32, with isolated vertices;
    # run right after the large graph, so stale bitmap words would show
    n2 = 1000 + 13
    s2, d2 = O.uniform_pairs(33, 900, 2500)  # vertices 900.. have no edges
    off2, nb2 = O.build_csr(n2, s2, d2)
    off2_t, nb2_t = _to_device(torch, off2, nb2)
    par2 = torch.empty(n2, dtype=torch.int32, device="cuda")
    lev2 = torch.empty(n2, dtype=torch.int32, device="cuda")
    deg2 = np.diff(off2.astype(np.int64))
    isolated = int(np.nonzero(deg2 == 0)[0][-1])
    assert isolated >= 900
    for src in (5, n2 - 1, isolated, 7):
        rc, rounds = _noalloc(L, off2_t, nb2_t, n2, len(nb2), src, par2, lev2, stream)
        assert rc == _abi.BYO_OK
        exp_par, exp_lev = O.bfs(off2, nb2, src)
        assert np.array_equal(par2.cpu().numpy().view(np.uint32), exp_par)
        assert np.array_equal(lev2.cpu().numpy().view(np.uint32), exp_lev)
        if deg2[src] == 0:
            assert int((exp_par != O.NONE).sum()) == 1
    rc, _ = _noalloc(L, off2_t, nb2_t, n2, len(nb2), n2, par2, lev2, stream)
    assert rc == _abi.BYO_EINVAL

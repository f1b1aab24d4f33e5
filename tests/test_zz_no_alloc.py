"""The allocation-free BFS entry point (byo_bfs_csr_noalloc) against byo_bfs.

Callers that cannot let a library allocate device memory (a host whose memory
manager owns the whole GPU, or code issuing work during stream capture) get a
BFS whose state lives in a fixed static device array.  This test calls it
through the C ABI on a CSR the test placed on the device, twice in a row (the
second call must not see the first call's leftovers), and checks parents and
levels against the allocating entry point bit for bit.  It sits in its own file
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


def test_noalloc_bfs_matches_bfs(ctx):
    import torch

    import byo_gb300 as byo
    from byo_gb300 import _abi
    L = _abi.lib()
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream().cuda_stream
    G = byo.Graph.generate(ctx, "rmat", seed=21, lg_n=20, draws=1 << 23)
    off, nb = G.export_csr()
    n, m = len(off) - 1, len(nb)
    assert n == _abi.NOALLOC_MAX_VERTICES
    off_t = torch.from_numpy(off.view(np.int64)).cuda()
    nb_t = torch.from_numpy(nb.view(np.int32)).cuda()
    par_t = torch.empty(n, dtype=torch.int32, device="cuda")
    lev_t = torch.empty(n, dtype=torch.int32, device="cuda")
    hub = int(np.argmax(np.diff(off.astype(np.int64))))
    for src in (10, hub):  # two calls in a row on the shared scratch
        rc, rounds = _noalloc(L, off_t, nb_t, n, m, src, par_t, lev_t, stream)
        assert rc == _abi.BYO_OK
        exp_par, exp_lev = byo.BFS(G, src, levels=True)
        assert np.array_equal(par_t.cpu().numpy().view(np.uint32), exp_par)
        assert np.array_equal(lev_t.cpu().numpy().view(np.uint32), exp_lev)
        assert rounds > 0
    # n beyond the static capacity is refused
    rc, _ = _noalloc(L, off_t, nb_t, n + 1, m, 0, par_t, lev_t, stream)
    assert rc == _abi.BYO_EINVAL
    G.close()

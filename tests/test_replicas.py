"""The N-GPU path of bench.py is N independent replicas: the job's time is the
slowest rank's and its rate counts every rank's work.  Checked here with two
gloo ranks on the CPU (127.0.0.1)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        ms = 10.0 + 5.0 * rank           # rank 1 is the slow one
        got = bench.max_over_ranks(ms, world)
        q.put((rank, got, bench.replica_value(3e9, world, got)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, val in out:
        assert got == 15.0
        assert val == pytest.approx(2 * 3e9 / 0.015 / 1e9)


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(7.5, 1) == 7.5
    assert bench.replica_value(1e9, 1, 1000.0) == pytest.approx(1.0)

"""Multi-GPU coordination on the CPU: two gloo ranks (one process each, as torchrun starts them).

The path runs replicas only (independent images per rank, no data-path
collective); what crosses ranks is the timing: max over ranks of each rank's
timed region, and the whole-job rate computed from it.
"""
import os
import socket

import pytest

from pymoresane_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = [10.0 + rank, 5.0 * (world - rank), float(rank)]
        dist.barrier()
        got = replicas.reduce_max(local, dist, "cpu")
        dist.barrier()
        q.put((rank, got, replicas.whole_job_rate(3, world, got[0]),
               replicas.rank_seed(1000, rank)))
    finally:
        dist.destroy_process_group()


def test_reduce_max_and_rate_over_two_gloo_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(q.get(timeout=10) for _ in procs)
    for rank, got, rate, seed in res:
        assert got == [11.0, 10.0, 1.0]          # element-wise max of both ranks' values
        assert rate == pytest.approx(2 * 3 / 11.0)
    assert res[0][3] != res[1][3]                # each rank deconvolves its own images


def test_single_process_is_local():
    assert replicas.reduce_max([1.5, 2.0]) == [1.5, 2.0]
    assert replicas.whole_job_rate(4, 1, 2.0) == 2.0

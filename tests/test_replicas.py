"""Replica aggregation across ranks (world size 2, gloo on CPU): the job rate
is everything the ranks completed over the slowest rank's time."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, counts, times, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from pyvr_gb300.replicas import barrier, job_rate
        barrier()
        r = job_rate(counts[rank], times[rank])
        barrier()
        out[rank] = r
    finally:
        dist.destroy_process_group()


def _vote_worker(rank, world, port, flags, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from pyvr_gb300.replicas import all_ok
        out[rank] = (all_ok(flags[rank]), all_ok(True))
    finally:
        dist.destroy_process_group()


def test_ranks_decide_together():
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    mp.start_processes(_vote_worker, args=(2, _free_port(), [True, False], out), nprocs=2,
                       start_method="spawn")
    assert out[0] == (False, True) and out[1] == (False, True)


def test_job_rate_over_two_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    counts, times = [120, 80], [1.5, 2.0]
    mp.start_processes(_worker, args=(2, _free_port(), counts, times, out), nprocs=2, start_method="spawn")
    want = sum(counts) / max(times)
    assert out[0] == pytest.approx(want) and out[1] == pytest.approx(want)


def test_single_process_rate():
    from pyvr_gb300.replicas import job_rate
    assert job_rate(50, 2.0) == 25.0
    assert job_rate(5, 0.0) == 0.0

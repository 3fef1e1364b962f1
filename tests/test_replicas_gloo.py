"""The bench's multi-GPU form is replicas only (the path does not shard): every
rank runs the whole step on its own GPU, rank 0 reports the slowest rank's
time and the whole job's throughput.  This checks that host logic with two
gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(times[rank], world, "cpu")
        out[rank] = (ms, bench.whole_job_value(1_000_000_000, world, ms))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    world, port = 2, _free_port()
    times = [12.5, 14.0]   # ms per step on each rank
    with mp.get_context("spawn").Manager() as m:   # no fork of a threaded process
        out = m.dict()
        mp.spawn(_rank, args=(world, port, times, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        ms, value = res[r]
        assert ms == pytest.approx(14.0)
        # 2 ranks x 1e9 edges in 14 ms
        assert value == pytest.approx(2 * 1e9 / 14e-3 / 1e9)


def test_single_rank_needs_no_process_group():
    assert bench.max_over_ranks(3.25, 1, "cpu") == 3.25
    assert bench.whole_job_value(5e8, 1, 10.0) == pytest.approx(50.0)

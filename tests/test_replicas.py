"""The bench's replica timing (one process per GPU, no exchange in the data path): every rank
times its own steps, the job's time is the slowest rank's (all_reduce MAX) and the rate counts
the rays of all ranks.  Two gloo ranks on the CPU stand in for two GPUs."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    dist.barrier()
    ms = 100.0 + 25.0 * rank                       # rank 1 is the slow replica
    job_ms = bench.max_over_ranks(ms, dist, torch.device("cpu"))
    rate = bench.whole_job_rate(world, 1000, 4, job_ms)
    out[rank] = (job_ms, rate)
    dist.destroy_process_group()


def test_two_replicas_time_the_slowest_rank():
    world = 2
    out = mp.get_context("spawn").Manager().dict()     # spawn: no fork of a threaded process
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        job_ms, rate = out[r]
        assert job_ms == 125.0
        assert rate == pytest.approx(world * 1000 * 4 / 0.125)


def test_single_process_needs_no_collective():
    import bench
    assert bench.max_over_ranks(42.0, None, torch.device("cpu")) == 42.0
    assert bench.whole_job_rate(1, 1_000_000, 100, 10_000.0) == pytest.approx(1e7)

"""Multi-GPU path of bench.py: replicas only (every rank serves the stream on
its own graph replica, no data-path collective).  The timing reduction it
does use — the slowest rank's time by a MAX all-reduce, whole-job throughput
= all ranks' units over that time — runs here as two gloo ranks on CPU."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int) -> None:
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seconds = 1.5 + rank  # rank 1 is the slower one
        slowest = bench.max_over_ranks(seconds, world, "cpu")
        assert slowest == 2.5
        assert bench.replica_throughput(30, world, slowest) == pytest.approx(24.0)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_timing_reduction():
    mp.spawn(_rank, args=(2, _free_port()), nprocs=2, join=True)


def test_single_rank_needs_no_process_group():
    assert bench.max_over_ranks(3.0, 1, "cpu") == 3.0
    assert bench.replica_throughput(15, 1, 0.5) == 30.0

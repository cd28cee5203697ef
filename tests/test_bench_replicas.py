"""The multi-GPU path of bench.py is independent replicas: each rank times its
own problem, the job's time is the slowest rank's (a MAX all-reduce, the only
collective), and the value is every rank's units over that time. Two gloo
ranks on the CPU run the same helpers the benchmark calls."""
import os
import socket
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, ms_by_rank, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(ms_by_rank[rank], world)
        out[rank] = (ms, bench.replica_throughput(10, world, ms))
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    ms_by_rank = [1500.0, 2100.0]
    # the manager's server process is spawned, not forked: this process may already run
    # the CPU oracle's OpenMP threads
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), ms_by_rank, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        ms, value = res[r]
        assert ms == max(ms_by_rank)
        assert value == pytest.approx(10 * world / (max(ms_by_rank) / 1e3))


def test_single_rank_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(123.5, 1) == 123.5
    assert bench.replica_throughput(10, 1, 2000.0) == pytest.approx(5.0)

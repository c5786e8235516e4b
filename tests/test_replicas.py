"""The multi-GPU form of bench.py is independent replicas (one field per rank,
no collective on the data path): the whole-job rate is the sum over ranks of
the units processed, divided by the slowest rank's time.  Two gloo ranks on
CPU check the max-over-ranks timing and the aggregate."""
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


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 100.0 * (rank + 1)                     # rank 1 is the slow one
        slow = bench.max_over_ranks(ms, dist, "cpu")
        out[rank] = (slow, bench.replica_rate(world, 1.0e9, 4, slow))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:   # no fork of this (threaded) process
        out = m.dict()
        mp.start_processes(_rank, args=(world, port, out), nprocs=world, start_method="spawn")
        res = dict(out)
    for r in range(world):
        slow, rate = res[r]
        assert slow == 200.0
        assert rate == pytest.approx(2 * 1.0e9 * 4 / 0.2)


def test_single_process_needs_no_group():
    assert bench.max_over_ranks(12.5, None, "cpu") == 12.5
    assert bench.replica_rate(1, 1e6, 2, 1000.0) == pytest.approx(2e6)

"""The multi-GPU host logic of bench.py on CPU: world_size 2 over gloo.  Each rank steps its own
seeded system (no collective on the data path); the timings meet in a max over ranks, the atom
counts in a sum, and the whole-job value is all atoms x steps / the slowest rank's time."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seconds = 1.0 + rank  # rank 1 is the slower one
        atoms = 1000.0 * (rank + 1)
        t_max = bench.over_ranks(dist, seconds, "max", "cpu")
        n_all = bench.over_ranks(dist, atoms, "sum", "cpu")
        out[rank] = (t_max, n_all, bench.job_value(n_all, 10, t_max))
    finally:
        dist.destroy_process_group()


def test_two_ranks_reduce_over_gloo():
    world = 2
    with mp.get_context("spawn").Manager() as m:  # no fork of this (threaded) test process
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        t_max, n_all, value = res[rank]
        assert t_max == 2.0 and n_all == 3000.0
        assert value == pytest.approx(3000.0 * 10 / 2.0)


def test_one_rank_needs_no_process_group():
    assert bench.over_ranks(None, 2.5, "max", "cpu") == 2.5
    assert bench.job_value(45546.0, 200, 0.0172) == pytest.approx(45546.0 * 200 / 0.0172)


def test_ranks_step_independent_systems():
    """Rank r's workload has its own seed: the same size class, different atoms."""
    p0, r0, _ = bench.workload(0)
    p1, r1, _ = bench.workload(1)
    assert p0.nMol > 40000 and p1.nMol > 40000
    assert p0.nMol != p1.nMol or not np.array_equal(r0, r1)

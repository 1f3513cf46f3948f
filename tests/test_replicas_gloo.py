"""Multi-rank host logic of the benchmark (replicas, no data-path collective),
run as two gloo ranks on the CPU: each rank takes a disjoint slice of one
seeded candidate stream, and the job time is the maximum over ranks."""
from __future__ import annotations

import os
import socket
import sys

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out: dict):
    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    cands = bench.rank_candidates(1, 3, world, rank, 8)
    times = bench.max_over_ranks([1.0 + rank, 10.0 - rank], dist, "cpu")
    out[rank] = (cands, times)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_disjoint_candidates_and_max_time():
    port = _free_port()
    with mp.get_context("spawn").Manager() as mgr:   # no fork of this (threaded) process
        out = mgr.dict()
        mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    sys.path.insert(0, REPO)
    import bench
    from tomography_gb300 import workloads as W

    allc = W.candidate_batch(1, 6, 8)
    np.testing.assert_array_equal(np.concatenate([res[0][0], res[1][0]]), allc)
    assert not np.array_equal(res[0][0], res[1][0])
    assert res[0][1] == res[1][1] == [2.0, 10.0]
    assert bench.max_over_ranks([3.0, 4.0]) == [3.0, 4.0]   # one process: unchanged

"""Multi-rank host logic on CPU (gloo, world size 2): the shards of the batch
workload are disjoint and the timing reduction takes the slowest rank's time
and the sum of the trajectory-steps of all ranks (the only collective)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t, done = bench.reduce_over_ranks(1.0 + rank, 10.0 * (rank + 1), world, "cpu")
    out[rank] = (t, done)
    dist.destroy_process_group()


def test_reduce_over_two_gloo_ranks():
    world, port = 2, _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        assert out[r] == (2.0, 30.0)


def test_rank_shards_are_disjoint():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    a, b = bench.workload(0, 8), bench.workload(1, 8)
    key = lambda m: (tuple(m["Z"]), round(float(np.asarray(m["xyz"]).sum()), 6))
    assert not set(map(key, a)) & set(map(key, b))

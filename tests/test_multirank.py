"""Multi-rank host logic on CPU (gloo, world size 2): the shards of the batch
workload are disjoint and the timing reduction takes the slowest rank's time
and the sum of the trajectory-steps of all ranks (the only collective); the
production driver splits an ensemble over ranks by nao^3 (every trajectory in
one shard, the heaviest rank within one trajectory of the mean) and merges the
ranks' result records in trajectory order."""
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


def _gather_worker(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from qcxms_gb300 import driver
    # each rank holds the records of its own shard, in its own order
    mine = [{"itrj": t, "rank": rank} for t in (range(5, 0, -2) if rank == 0 else (6, 2, 4))]
    out[rank] = driver.gather_results(mine, world)
    dist.destroy_process_group()


def test_sharded_ensemble_records_merge_over_two_gloo_ranks():
    world, port = 2, _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_gather_worker, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        assert [t["itrj"] for t in out[r]] == [1, 2, 3, 4, 5, 6]
        assert [t["rank"] for t in out[r]] == [0, 1, 0, 1, 0, 1]


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_ensemble_shards_partition_and_balance(world):
    from qcxms_gb300 import basis, driver, molgen
    mols = molgen.batch_workload(256, 5, 40)
    shards = driver.shard_ensemble(mols, world)
    assert len(shards) == world
    flat = sorted(i for s in shards for i in s)
    assert flat == list(range(len(mols)))
    assert all(s == sorted(s) for s in shards)
    assert driver.shard_ensemble(mols, world) == shards  # every rank computes the same split
    cost = np.array([float(basis.nao_of(m["Z"])) ** 3 for m in mols])
    load = np.array([cost[s].sum() for s in shards])
    # greedy bound: the heaviest rank carries at most the mean plus one trajectory
    assert load.max() <= cost.sum() / world + cost.max() + 1e-6
    if world > 1:
        # and far better than consecutive blocks of the ensemble
        blocks = np.array_split(np.arange(len(mols)), world)
        assert load.max() <= max(cost[b].sum() for b in blocks)
        assert load.max() / load.mean() < 1.02


def test_more_ranks_than_trajectories():
    from qcxms_gb300 import driver, molgen
    mols = molgen.batch_workload(3, 5, 10)
    shards = driver.shard_ensemble(mols, 5)
    assert sorted(i for s in shards for i in s) == [0, 1, 2]
    assert sum(1 for s in shards if not s) == 2
    with pytest.raises(ValueError):
        driver.shard_ensemble(mols, 0)


def _driver_main_worker(rank, world, port, out_json, res_path):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from qcxms_gb300 import driver

    def fake_run(root, *a, rank=0, world=1, **k):
        # this rank's shard of a 5-trajectory ensemble: two records of rank 0, three of rank 1
        mine = [1, 4] if rank == 0 else [0, 2, 3]
        return [{"itrj": i, "mdok": True, "fragstate": 1, "nstep": 10 * i, "nfrag": 2, "formula": ["H2O1"],
                 "res_lines": ["line %d" % i]} for i in mine]

    driver.run_ensemble = fake_run
    sys.argv = ["driver", "ENSEMBLE", "--out", out_json, "--res", res_path]
    driver.main()


def test_driver_main_merges_the_ranks_records(tmp_path):
    world, port = 2, _free_port()
    out_json, res_path = str(tmp_path / "res.json"), str(tmp_path / "qcxms.res")
    mp.spawn(_driver_main_worker, args=(world, port, out_json, res_path), nprocs=world, join=True)
    import json
    with open(out_json) as f:
        recs = json.load(f)
    assert [r["itrj"] for r in recs] == [0, 1, 2, 3, 4]
    with open(res_path) as f:
        assert f.read().split("\n")[:5] == ["line %d" % i for i in range(5)]


def test_run_ensemble_takes_its_ranks_shard(monkeypatch):
    import sys
    sys.path.insert(0, ROOT)
    from qcxms_gb300 import driver, molgen
    mols = molgen.batch_workload(12, 5, 30)
    for i, m in enumerate(mols):
        m["itrj"] = i
    monkeypatch.setattr(driver, "read_ensemble", lambda root, charge=1: [dict(m) for m in mols])

    class Seen(Exception):
        pass

    def fake_batch(ms, etemp=300.0):
        raise Seen([m["itrj"] for m in ms])

    monkeypatch.setattr(driver, "Batch", fake_batch)
    shards = driver.shard_ensemble(mols, 3)
    for rank in range(3):
        with pytest.raises(Seen) as e:
            driver.run_ensemble("ENSEMBLE", rank=rank, world=3)
        assert e.value.args[0] == shards[rank]
    # one rank: the whole ensemble in order
    with pytest.raises(Seen) as e:
        driver.run_ensemble("ENSEMBLE")
    assert e.value.args[0] == list(range(12))

"""Host-side measurement logic of bench.py, on CPU: the SCC FLOP convention of
the roofline, the size-stratified samples, the CPU baseline's timing of the
oracle (busy-time rate, accepted steps only) and the reference arm's JSON line
(the keys the run's consumers read)."""
import argparse
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_scc_flop_convention():
    # per molecule: iterations * 11 n^3 (9 n^3 eigensolve, 2 n^3 density) + 2 n^3 (W)
    nao = np.array([10, 20])
    iters = np.array([3, 5])
    assert bench.scc_flops(nao, iters) == 3 * 11 * 1000 + 2 * 1000 + 5 * 11 * 8000 + 2 * 8000
    assert bench.scc_flops(np.array([7]), np.array([0])) == 2 * 343


def test_stratified_sample_spans_the_sizes():
    mols = bench.workload(0)
    nat = np.array([len(m["Z"]) for m in mols])
    s = bench.stratified(mols, 32)
    sn = [len(m["Z"]) for m in s]
    assert len(s) == 32
    assert sn[0] == nat.max() and sn[-1] == nat.min()
    assert all(a >= b for a, b in zip(sn, sn[1:]))
    everything = bench.stratified(mols[:5], 10)
    assert sorted(len(m["Z"]) for m in everything) == sorted(len(m["Z"]) for m in mols[:5])


def test_workload_is_deterministic_per_rank():
    a, b = bench.workload(0, 6), bench.workload(0, 6)
    for x, y in zip(a, b):
        assert np.array_equal(x["Z"], y["Z"]) and np.array_equal(np.asarray(x["xyz"]), np.asarray(y["xyz"]))


def test_cpu_baseline_counts_accepted_steps_over_busy_time(oracle_lib):
    mols = bench.stratified(bench.workload(0), 4)[-2:]  # the two smallest of four
    v, calls, el, done, wall = bench.cpu_sample(mols, 0.01, 1, chunk=2)
    assert calls == 1 and done == 2 * len(mols)  # one call of 2 steps, every trajectory accepted
    # one thread: its busy time is within the call's wall time, so the busy-time
    # rate is at least the wall-clock rate
    assert v >= wall > 0 and el > 0


def test_reference_arm_line(monkeypatch, capsys):
    # the sample timing is replaced by fixed figures: the line's keys and the
    # median over steps are what is checked here
    figures = iter([(100.0, 3, 12.0, 1200, 50.0), (300.0, 3, 12.0, 1200, 50.0), (200.0, 3, 12.0, 1200, 50.0)])
    monkeypatch.setattr(bench, "cpu_sample", lambda *a, **k: next(figures))
    monkeypatch.delenv("RANK", raising=False)
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    bench.run_reference(argparse.Namespace(steps=3, warmup=3, gpus=1))
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] == 200.0
    for key in ("metric", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["e2e"] == {"value": 200.0, "unit": line["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert line["cpu_baseline"]["value"] == 200.0 and line["cpu_baseline"]["kind"] == "port"
    assert line["higher_is_better"] is True and line["config"]["workload"] == bench.WORKLOAD_NAMES["batch"]


def test_reference_arm_other_ranks_do_no_work(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(bench, "cpu_sample", lambda *a, **k: pytest.fail("rank 1 must not time anything"))
    bench.run_reference(argparse.Namespace(steps=1, warmup=0, gpus=2))
    assert capsys.readouterr().out == ""

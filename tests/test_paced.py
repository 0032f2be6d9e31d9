"""Size-bucketed stepping: molecule groups step from their own graphs.

qcx_batch_step_groups advances group g by nsteps[g] MD steps; every group
replays its own captured graph on its own stream. qcx_batch_step_paced gives
the largest molecules' group one step and every other group as many as fit
into the same time. Trajectories are independent, so every trajectory's
sequence of steps must be the one of plain whole-batch stepping, to the SCC
tolerances.

GPU: step counts per group; positions after k steps against the whole-batch
path; paced stepping with the SCC budget; the device MD rules in groups.
"""
import numpy as np
import pytest

import qcxms_gb300 as qg
from qcxms_gb300 import constants, molgen

pytestmark = pytest.mark.gpu
DT = 0.5 * constants.FSTOAU


def _path(mols, nsteps):
    a = qg.Batch(mols)
    a.egrad()
    path = [a.get()["xyz"].copy()]
    for _ in range(nsteps):
        a.step(1, DT)
        path.append(a.get()["xyz"].copy())
    act, steps = a.progress()
    a.close()
    return path, act, steps


def test_step_groups_follow_the_whole_batch_path(gpu):
    mols = molgen.batch_workload(16, 6, 24, seed0=300)
    path, act_a, steps_a = _path(mols, 8)
    b = qg.Batch(mols)
    b.egrad()
    grp, _, _ = b.group_info()
    assert grp.max() == 7 and np.all(np.bincount(grp) == 2)
    nsteps = np.array([1, 1, 2, 2, 3, 4, 6, 8], dtype=np.int32)
    _, s0 = b.progress()
    b.step_groups(nsteps, DT)
    r = b.get()
    act, s1 = b.progress()
    off = b.offsets
    compared = 0
    for i in range(b.nmol):
        k = int(nsteps[grp[i]])
        if not (act[i] and act_a[i] and steps_a[i] - 1 >= k):
            continue
        assert s1[i] - s0[i] == k
        sl = slice(off[i], off[i + 1])
        assert np.abs(r["xyz"][sl] - path[k][sl]).max() < 1e-6, (i, k)
        compared += 1
    assert compared >= 12
    _, gn, _ = b.group_info()
    assert list(gn) == list(nsteps)
    b.close()


def test_step_paced_with_budget_follows_the_path(gpu):
    mols = molgen.batch_workload(24, 6, 30, seed0=500)
    path, act_a, steps_a = _path(mols, 12)
    b = qg.Batch(mols)
    b.set_scc_budget(10)
    b.egrad()
    base = b.progress()[1].copy()
    seen = base.copy()
    off = b.offsets
    compared = 0
    # budget 10 for each group's largest molecule (the budget scales per group):
    # most SCCs need two or three calls, so six calls give every group steps
    for _ in range(6):
        b.step_paced(1, DT)
        r = b.get()
        act, steps = b.progress()
        pend = (r["status"] & qg.STATUS_SCC_PENDING) != 0
        for i in range(b.nmol):
            k = int(steps[i] - base[i])
            if steps[i] > seen[i] and not pend[i] and k <= 12 and act[i] and act_a[i] and steps_a[i] - 1 >= k:
                sl = slice(off[i], off[i + 1])
                assert np.abs(r["xyz"][sl] - path[k][sl]).max() < 1e-5, (i, k)
                compared += 1
            seen[i] = steps[i]
    _, gn, gms = b.group_info()
    # the largest molecules' group takes one step per call, the others at least one
    assert gn[0] == 1 and np.all(gn >= 1) and np.all(gms > 0)
    assert compared >= 20
    b.close()


def test_md_rules_in_groups(gpu):
    """Grouped steps run the device MD rules per group: nstep - steps_done is the
    same for every running trajectory and the same as with whole-batch steps."""
    mols = molgen.batch_workload(16, 8, 24, seed0=700)

    def offsets(b):
        st = b.md_state()
        act, steps = b.progress()
        return (st["nstep"] - steps)[st["done"] == 0]

    a = qg.Batch(mols)
    a.egrad()
    a.set_md_rules(6, 250, 100000)
    a.step(2, DT)
    ref = offsets(a)
    a.close()
    b = qg.Batch(mols)
    b.egrad()
    b.set_md_rules(6, 250, 100000)
    b.step_groups(np.array([1, 2, 3, 4, 5, 6, 7, 8], dtype=np.int32), DT)
    d = offsets(b)
    assert len(ref) > 0 and len(d) > 0 and np.all(d == ref[0])
    b.close()


def test_budget_autotuner(gpu):
    """The autotuner measures every candidate on the batch's own paced steps,
    keeps the fastest and leaves the batch stepping with it."""
    mols = molgen.batch_workload(24, 6, 30, seed0=900)
    b = qg.Batch(mols)
    b.egrad()
    _, s0 = b.progress()
    (best, per_group), rates = b.autotune_budget((0, 8, 30), calls=2, tstep=DT)
    # every candidate with both budget scales (each group's largest molecule,
    # the batch's largest)
    assert best in (0, 8, 30) and per_group in (0, 1)
    assert set(rates) == {(k, g) for k in (0, 8, 30) for g in (0, 1)}
    assert all(v > 0 for v in rates.values()) and rates[(best, per_group)] == max(rates.values())
    _, s1 = b.progress()
    assert np.sum(s1 - s0) > 0  # the measured steps advanced the trajectories
    b.step_paced(1, DT)
    b.close()


def test_group_graphs_take_new_scc_settings(gpu):
    # the group graphs hold the SCC settings as kernel arguments: after
    # set_scc they are captured again, so a 2-iteration limit set between two
    # grouped steps stops every SCC of the second one
    mols = molgen.batch_workload(16, 6, 24, seed0=300)
    b = qg.Batch(mols)
    b.egrad()
    ones = np.ones(8, dtype=np.int32)
    b.step_groups(ones, DT)
    st, _ = b.status_iters()
    assert (st == 0).sum() >= len(st) - 1
    act = b.progress()[0] > 0
    b.set_scc(max_iter=2)
    b.step_groups(ones, DT)
    st, it = b.status_iters()
    assert np.all(st != 0) and np.all(it[act] <= 2), (st, it)
    b.close()

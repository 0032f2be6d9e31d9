"""Per-step SCC budget (qcx_batch_set_scc_budget): trajectories at their own pace.

QCxMS runs every trajectory as its own process (bin/pqcxms), so a slow SCC
delays only its own trajectory. With a budget, an SCC that needs more
iterations than one step grants stops (status QCX_STATUS_SCC_PENDING) and the
next step continues it at the same coordinates; the trajectory neither moves
nor counts a step meanwhile. Each trajectory's sequence of steps must be the
one without a budget, to the SCC tolerances.

GPU: the same batch stepped with and without a small budget: after its k-th
completed step every trajectory of the budgeted batch sits where the
unbudgeted one was after step k; pending trajectories do not move; steps
count only on completion; qcx_batch_egrad completes suspended SCCs; FP64 and
mixed precision; the device MD rules skip pending steps.
"""
import numpy as np
import pytest

import qcxms_gb300 as qg
from qcxms_gb300 import constants, molgen

pytestmark = pytest.mark.gpu
DT = 0.5 * constants.FSTOAU


def _mols(n=10, seed=40):
    return molgen.batch_workload(n, 8, 30, seed0=seed)


def _reference_path(mols, precision, nsteps):
    a = qg.Batch(mols)
    a.set_precision(precision)
    a.egrad()
    path = [a.get()["xyz"].copy()]
    for _ in range(nsteps):
        a.step(1, DT)
        path.append(a.get()["xyz"].copy())
    act, steps = a.progress()
    a.close()
    return path, act, steps


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_budgeted_steps_follow_the_unbudgeted_path(gpu, precision):
    mols = _mols()
    nsteps = 3
    path, act_a, steps_a = _reference_path(mols, precision, nsteps)
    b = qg.Batch(mols)
    b.set_precision(precision)
    b.set_scc_budget(6 if precision == "mixed" else 12)
    b.egrad()
    r0 = b.get()
    assert not np.any(r0["status"] & qg.STATUS_SCC_PENDING)  # egrad completes every SCC
    off = b.offsets
    seen = b.progress()[1].copy()  # the start's evaluation counts one
    base = seen.copy()
    pending_seen = 0
    for tick in range(150):
        b.step(1, DT)
        r = b.get()
        act, steps = b.progress()
        pend = (r["status"] & qg.STATUS_SCC_PENDING) != 0
        for i in range(b.nmol):
            sl = slice(off[i], off[i + 1])
            if pend[i]:
                pending_seen += 1
                assert steps[i] == seen[i]  # no step counted while pending
            if steps[i] > seen[i]:
                assert steps[i] == seen[i] + 1
                seen[i] = steps[i]
                k = int(steps[i] - base[i])
                if k <= nsteps and act_a[i] and steps_a[i] - 1 >= k:
                    assert np.abs(r["xyz"][sl] - path[k][sl]).max() < 1e-5, (i, k)
        if np.all((seen - base >= nsteps) | (act == 0)):
            break
    assert pending_seen > 0  # the budget suspended some SCCs
    assert np.all((seen - base >= nsteps) | (act == 0))
    # a pending trajectory stays put for the ticks it waits
    b.step(1, DT)
    r1 = b.get()
    pend = (r1["status"] & qg.STATUS_SCC_PENDING) != 0
    x_before = r1["xyz"].copy()
    b.step(1, DT)
    r2 = b.get()
    for i in np.where(pend)[0]:
        sl = slice(off[i], off[i + 1])
        assert np.array_equal(r2["xyz"][sl], x_before[sl])
    # egrad completes every suspended SCC at the current coordinates
    b.egrad()
    r3 = b.get()
    assert not np.any(r3["status"] & qg.STATUS_SCC_PENDING)
    c = qg.Batch([{"Z": m["Z"], "xyz": r3["xyz"][off[i]:off[i + 1]], "charge": m["charge"]}
                  for i, m in enumerate(mols)])
    c.set_precision(precision)
    c.egrad()
    rc = c.get()
    ok = (r3["status"] == 0) & (rc["status"] == 0) & (act > 0)
    assert ok.sum() >= b.nmol // 2
    assert np.abs(r3["energy"][ok] - rc["energy"][ok]).max() < 1e-6
    c.close()
    b.close()


def test_md_rules_skip_pending_steps(gpu):
    """With the device MD rules on, a budgeted batch advances the rule state
    (nstep) only with completed steps: nstep - steps_done is the same for every
    running trajectory and the same as without a budget."""
    mols = _mols(8, seed=77)

    def offsets(b):
        st = b.md_state()
        act, steps = b.progress()
        run = st["done"] == 0
        return (st["nstep"] - steps)[run]

    a = qg.Batch(mols)
    a.egrad()
    a.set_md_rules(6, 250, 100000)
    a.step(2, DT)
    ref = offsets(a)
    assert len(ref) > 0 and np.all(ref == ref[0])
    a.close()
    b = qg.Batch(mols)
    b.set_scc_budget(5)
    b.egrad()
    b.set_md_rules(6, 250, 100000)
    pend = 0
    for _ in range(12):
        b.step(1, DT)
        pend += int(np.sum((b.status_iters()[0] & qg.STATUS_SCC_PENDING) != 0))
    d = offsets(b)
    assert pend > 0 and len(d) > 0 and np.all(d == ref[0])
    b.close()

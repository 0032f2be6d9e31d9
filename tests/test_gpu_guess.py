"""SCC starting point across MD steps (qcx_batch_set_guess).

The default starts every SCC from zero moments, as the reference creates a
fresh wavefunction on every call (src/tblite.f90:133). The opt-in warm start
reuses a trajectory's converged moments from its previous geometry: it must
reach the same solution to the SCC tolerances with fewer iterations."""
import numpy as np
import pytest

import qcxms_gb300 as qg
from qcxms_gb300 import constants, molgen

pytestmark = pytest.mark.gpu


def _run(guess, nsteps=6):
    mols = molgen.batch_workload(12, 8, 30, seed0=7)
    b = qg.Batch(mols, etemp=300.0)
    b.set_precision("mixed")
    b.set_scc(100, 1e-9, 1e-8, 0.25)
    b.set_guess(guess)
    b.egrad()
    iters = []
    energies = []
    for _ in range(nsteps):
        b.step(1, 0.5 * constants.FSTOAU)
        r = b.get()
        iters.append(r["iters"].copy())
        energies.append(r["energy"].copy())
    r = b.get()
    active, _ = b.progress()
    return np.array(energies), np.array(iters), r, active


def test_warm_start_same_trajectory_fewer_iterations(gpu):
    e0, it0, r0, a0 = _run("zero")
    e1, it1, r1, a1 = _run("previous")
    ok = (a0 > 0) & (a1 > 0)
    assert ok.sum() >= 6
    # same solution to well inside the SCC tolerances over six steps
    assert np.abs(e0[:, ok] - e1[:, ok]).max() < 1e-6
    at = np.repeat(ok, [len(m["Z"]) for m in molgen.batch_workload(12, 8, 30, seed0=7)])
    assert np.abs(r0["xyz"][at] - r1["xyz"][at]).max() < 1e-6
    assert np.abs(r0["grad"][at] - r1["grad"][at]).max() < 1e-5
    # after the first step the warm start needs clearly fewer iterations
    assert it1[1:, ok].mean() < 0.8 * it0[1:, ok].mean()


def test_guess_switch(gpu):
    mols = molgen.batch_workload(4, 8, 20, seed0=3)
    b = qg.Batch(mols, etemp=300.0)
    b.set_precision("mixed")
    b.egrad()
    r = b.get()
    it_fresh, e_fresh, ok = r["iters"].copy(), r["energy"].copy(), r["status"] == 0
    assert ok.sum() >= 3
    b.set_guess("previous")
    b.egrad()  # same geometry: starts from the converged moments
    r = b.get()
    it_warm = r["iters"].copy()
    assert (it_warm[ok] < it_fresh[ok]).all()
    assert np.abs(r["energy"][ok] - e_fresh[ok]).max() < 1e-6
    b.set_guess("zero")
    b.egrad()
    r = b.get()
    # back to the zero start: as many iterations as the first evaluation, to
    # within the run-to-run spread of the SCC path (the pair sums of the
    # potentials use atomics), far more than the warm start needed
    assert r["iters"][ok].mean() > 1.5 * it_warm[ok].mean()
    assert np.abs(r["energy"][ok] - e_fresh[ok]).max() < 1e-6

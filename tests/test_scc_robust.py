"""SCC convergence on hard geometries: the FP64 GPU path converges where the
oracle converges, in about as many iterations, to the same energy; the mixed
path converges on nearly all of them.

The geometries are MD snapshots of hot random cations of the default workload
(taken with the oracle's own MD) whose SCC needs many iterations: clusters of
orbitals 1e-3 Eh apart at the Fermi level make the first-order eigenvector
refinement hand over to Jacobi often. A refinement that leaves the
coefficient rows slightly non-orthonormal in the overlap metric turns the next
eigenproblem into the wrong one (eigenvalue errors of 3e-4 Eh were seen), and
the SCC then needs several times the oracle's iterations or stops at the
iteration limit. Both sides use the default thresholds (1e-7 Eh, 1e-6)."""
import numpy as np
import pytest

import qcxms_gb300 as qg
from qcxms_gb300 import constants, molgen

pytestmark = pytest.mark.gpu
KT = 300.0 * constants.KB_AU
DT = 0.5 * constants.FSTOAU
# (molecule of the 256-trajectory workload, MD step of the snapshot)
CASES = [(101, 6), (118, 26), (174, 8), (182, 10), (208, 20), (231, 1)]


@pytest.fixture(scope="module")
def snapshots(oracle_lib):
    mols = molgen.batch_workload(256, 5, 40)
    out = []
    for i, ns in CASES:
        m = mols[i]
        rc, e, g, q = oracle_lib.egrad_batch([m], KT, nthreads=1)
        fails, xyz, vel, grad, ep, its = oracle_lib.md_batch([m], ns, DT, g, KT, nthreads=1)
        assert fails == 0
        r, e, g, q, info = oracle_lib.egrad(m["Z"], xyz, 1, kT=KT)
        assert r == 0 and info["converged"] == 1
        out.append((m, xyz, e, info["iterations"]))
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_hard_geometries_converge_like_the_oracle(gpu, snapshots, precision):
    b = qg.Batch([dict(m, xyz=xyz) for m, xyz, _, _ in snapshots], etemp=300.0)
    b.set_precision(precision)
    b.egrad()
    r = b.get()
    e_orc = np.array([e for _, _, e, _ in snapshots])
    it_orc = np.array([it for _, _, _, it in snapshots])
    st, it = b.status_iters()
    ok = st == 0
    if precision == "fp64":
        # the FP64 path follows the oracle's SCC path (the same iterates to
        # rounding): every SCC converges in about as many iterations
        assert np.all(ok), (st, it, it_orc)
        assert np.all(it <= 1.25 * it_orc + 10), (it, it_orc)
        assert np.abs(r["energy"] - e_orc).max() < 1e-7
    else:
        # the FP32 iterations take their own path (FP32 rounding, eigenvectors
        # to the FP32 tolerance); on these near-degenerate cases that path is
        # sensitive to every rounding, so one of them may need the iteration
        # limit. The others converge to the oracle's energy.
        assert ok.sum() >= len(ok) - 1, (st, it, it_orc)
        assert np.mean(it[ok]) <= 2.0 * np.mean(it_orc[ok]) + 10, (it, it_orc)
        assert np.abs(r["energy"][ok] - e_orc[ok]).max() < 1e-6

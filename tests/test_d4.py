"""D4 dispersion anchored to QCxMS's own D4 data and algorithm.

QCxMS ships a D4 model in src/dftd4.f90 with its reference data in
include/param_d4.fh. The library and the oracle build their reference C6 from
that data (converted to qcx_d4ref.h by qcxms_gb300/params/gen_d4_reference.py)
by the reference's steps: polarisabilities of d4dim, Casimir-Polder C6 by
trapzd, covalent CN, Gaussian weights with refc Gaussians, charge scaling zeta.

CPU: the oracle's C6 against tests/golden/d4_c6.json, which
tests/golden/make_d4_golden.py computed with an independent numpy restatement
that parses the two reference files itself; the converted header against the
same fixture's raw values; the dispersion gradient against finite differences.
GPU: energies and gradients of the CUDA path against the oracle (the parity
tests cover the full energy; here molecules where dispersion matters: a
stretched dimer and a cation next to an Ar atom).
"""
import json
import os

import numpy as np
import pytest

from qcxms_gb300 import constants

HERE = os.path.dirname(os.path.abspath(__file__))
KT = 300.0 * constants.KB_AU


def _golden():
    return json.load(open(os.path.join(HERE, "golden", "d4_c6.json")))


def test_reference_pair_c6_match_independent_restatement(oracle_lib):
    for za, i, zb, j, v in _golden()["c6ref"]:
        assert abs(oracle_lib.d4_c6ref(za, i, zb, j) - v) <= 1e-13 * abs(v), (za, i, zb, j)
        assert oracle_lib.d4_c6ref(za, i, zb, j) == oracle_lib.d4_c6ref(zb, j, za, i)
    # Ar-Ar from the free-atom reference: a sanity value of the right size (about 64 a.u.)
    assert 60.0 < oracle_lib.d4_c6ref(18, 0, 18, 0) < 70.0
    assert oracle_lib.d4_c6ref(1, 5, 1, 0) == -1.0  # H has two references


def test_molecular_c6_match_independent_restatement(oracle_lib):
    for m in _golden()["molecules"]:
        c0 = oracle_lib.d4_c6(m["Z"], m["xyz"])
        cq = oracle_lib.d4_c6(m["Z"], m["xyz"], m["q"])
        ref0, refq = np.array(m["c6_q0"]), np.array(m["c6_q"])
        assert np.abs(c0 - ref0).max() <= 1e-13 * np.abs(ref0).max(), m["name"]
        assert np.abs(cq - refq).max() <= 1e-13 * np.abs(refq).max(), m["name"]
        # charge scaling: positive charges shrink C6, negative ones grow it
        assert not np.allclose(c0, cq)


def test_d4_gradient_finite_differences(oracle_lib):
    """A stretched water dimer cation and NH3+ next to Ar and S: analytic
    gradient (dispersion included) against central differences, h = 1e-4 Bohr."""
    m = _golden()["molecules"][3]
    Z, xyz = np.array(m["Z"]), np.array(m["xyz"])
    o = oracle_lib.default_opts(econv=1e-12, pconv=1e-10)
    rc, e, g, q, info = oracle_lib.egrad(Z, xyz, 1, kT=KT, opts=o)
    assert rc == 0 and info["e_disp"] < 0.0 and info["e_atm"] != 0.0
    h = 1e-4
    for a in (0, 4, 5):
        for k in range(3):
            xp, xm = xyz.copy(), xyz.copy()
            xp[a, k] += h
            xm[a, k] -= h
            ep = oracle_lib.egrad(Z, xp, 1, kT=KT, opts=o)[1]
            em = oracle_lib.egrad(Z, xm, 1, kT=KT, opts=o)[1]
            assert abs((ep - em) / (2 * h) - g[a, k]) < 1e-6, (a, k)


def test_header_holds_the_reference_literals():
    """qcx_d4ref.h holds the single-precision literals of the reference files
    (a spot check of values the fixture script parsed independently)."""
    txt = open(os.path.join(HERE, "..", "qcxms_gb300", "csrc", "qcx_d4ref.h")).read()
    assert "static const int qcx_d4_refn[19] = {0, 2, 1, 2, 3, 5, 7, 5, 4, 2, 1, 2, 3, 4, 5, 4, 3, 2, 1};" in txt
    # r4r2 of H, 2.00734898 in src/dftd4.f90, as Fortran stores it
    assert repr(float(np.float32(2.00734898))) in txt


@pytest.mark.gpu
def test_gpu_dispersion_matches_oracle(gpu, oracle_lib):
    import qcxms_gb300 as qg
    g = _golden()
    # the fixture geometries are symmetric (CH4 is tetrahedral: a threefold
    # degenerate level of the cation); jitter them so that no exact degeneracy
    # is left at the Fermi level
    rng = np.random.default_rng(11)
    mols = [(np.array(m["Z"]), np.array(m["xyz"]) + rng.normal(scale=0.05, size=(len(m["Z"]), 3)), 1)
            for m in g["molecules"]]
    b = qg.Batch([{"Z": Z, "xyz": x, "charge": c} for Z, x, c in mols])
    b.set_scc(100, 1e-11, 1e-9, 0.25)
    b.egrad()
    r = b.get()
    grads = b.split(r["grad"])
    o = oracle_lib.default_opts(econv=1e-11, pconv=1e-9)
    both = 0
    for i, (Z, x, c) in enumerate(mols):
        rc, e, gr, q, info = oracle_lib.egrad(Z, x, c, kT=KT, opts=o)
        t = b.energy_terms(i)
        if rc != 0 or r["status"][i] not in (0, qg.STATUS_CHECKQC):
            continue
        both += 1
        assert abs(t["disp"] - info["e_disp"]) < 1e-10 and abs(t["atm"] - info["e_atm"]) < 1e-9
        assert np.abs(grads[i] - gr).max() < 1e-7
    assert both >= 3

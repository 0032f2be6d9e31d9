"""The differentiation, precision and collision configurations at full size.

- differentiation: all 64 seeded 30-atom C/H/O cations; two random gradient
  components of each against central finite differences (h = 1e-4 Bohr) of GPU
  energies, all displaced structures in one batch, tolerance 1e-5 Eh/Bohr; and
  the GPU gradients of 16 of them against the CPU oracle's;
- precision: all 1024 seeded 60-atom C/H/N/O cations (about 150 atomic
  orbitals), the mixed path against the FP64 oracle: energies within 1e-6 Eh,
  gradients within 1e-5 Eh/Bohr;
- collision-induced dissociation: 64 ions of 60-80 C/H/N/O/S atoms next to an
  Ar atom, the mixed path against the FP64 oracle.
Each test prints its summary line (max errors, fractions within the contract).
"""
import json
import os

import numpy as np
import pytest

import qcxms_gb300 as qg
from qcxms_gb300 import constants, molgen

pytestmark = pytest.mark.gpu
KT = 300.0 * constants.KB_AU
NCPU = os.cpu_count() or 1


def _oracle_batch(oracle_lib, mols, opts=None):
    return oracle_lib.egrad_batch([{"Z": m["Z"], "xyz": m["xyz"], "charge": m["charge"]} for m in mols], KT,
                                  opts=opts, nthreads=NCPU)


def test_differentiation_64_cations_fd(gpu, oracle_lib):
    mols = []
    for s in range(64):
        Z, xyz = molgen.random_cho(30, s)
        mols.append({"Z": Z, "xyz": np.asarray(xyz, dtype=np.float64).reshape(-1, 3), "charge": 1})
    tight = (100, 1e-10, 1e-8, 0.25)
    b = qg.Batch(mols)
    b.set_scc(*tight)
    b.egrad()
    r = b.get()
    grads = b.split(r["grad"])
    rng = np.random.default_rng(64)
    h = 1e-4
    picks, disp = [], []
    for i, m in enumerate(mols):
        for _ in range(2):
            a, k = int(rng.integers(0, 30)), int(rng.integers(0, 3))
            picks.append((i, a, k))
            for sgn in (1.0, -1.0):
                x = m["xyz"].copy()
                x[a, k] += sgn * h
                disp.append({"Z": m["Z"], "xyz": x, "charge": 1})
    bd = qg.Batch(disp)
    bd.set_scc(*tight)
    bd.egrad()
    rd = bd.get()
    err, n_ok = [], 0
    for p, (i, a, k) in enumerate(picks):
        if r["status"][i] or rd["status"][2 * p] or rd["status"][2 * p + 1]:
            continue
        fd = (rd["energy"][2 * p] - rd["energy"][2 * p + 1]) / (2 * h)
        err.append(abs(fd - grads[i][a, k]))
        n_ok += 1
    err = np.array(err)
    # the GPU FP64 gradient against the oracle's for 16 of them
    o = oracle_lib.default_opts(econv=1e-10, pconv=1e-8)
    rc, e_o, g_o, _ = _oracle_batch(oracle_lib, mols[:16], o)
    dg = [np.abs(grads[i] - g_o[i]).max() for i in range(16) if rc[i] == 0 and r["status"][i] == 0]
    print(json.dumps({"config": "differentiation", "molecules": 64, "components": n_ok,
                      "max_fd_error": float(err.max()), "max_dg_vs_oracle": float(max(dg))}))
    assert n_ok >= 110 and err.max() < 1e-5
    assert len(dg) >= 14 and max(dg) < 1e-7


def _mixed_vs_oracle(oracle_lib, mols, label):
    b = qg.Batch(mols)
    b.set_precision("mixed")
    b.egrad()
    r = b.get()
    grads = b.split(r["grad"])
    rc, e_o, g_o, _ = _oracle_batch(oracle_lib, mols)
    ok = [i for i in range(len(mols)) if rc[i] == 0 and r["status"][i] == 0]
    dE = np.array([abs(r["energy"][i] - e_o[i]) for i in ok])
    dg = np.array([np.abs(grads[i] - g_o[i]).max() for i in ok])
    res = {"config": label, "molecules": len(mols), "both_converged": len(ok),
           "max_abs_dE": float(dE.max()), "median_abs_dE": float(np.median(dE)), "max_abs_dg": float(dg.max()),
           "frac_dE_le_1e-6": float(np.mean(dE <= 1e-6)), "frac_dg_le_1e-5": float(np.mean(dg <= 1e-5))}
    print(json.dumps(res))
    return res


def test_precision_1024_molecules_vs_oracle(gpu, oracle_lib):
    mols = []
    for t in range(1024):
        Z, xyz = molgen.random_chno(60, 900000 + t)
        mols.append({"Z": Z, "xyz": xyz, "charge": 1})
    res = _mixed_vs_oracle(oracle_lib, mols, "precision 1024 x 60 atoms")
    assert res["both_converged"] >= 0.95 * 1024
    assert res["frac_dE_le_1e-6"] >= 0.99 and res["frac_dg_le_1e-5"] >= 0.99


def test_cid_64_large_ions_vs_oracle(gpu, oracle_lib):
    mols = molgen.cid_workload(64, 60, 80, seed0=5000)
    res = _mixed_vs_oracle(oracle_lib, mols, "CID 64 x (60-80 atoms + Ar)")
    assert res["both_converged"] >= 54  # hot 60-80-atom cations: a few SCCs reach the iteration limit
    assert res["frac_dE_le_1e-6"] >= 0.95 and res["frac_dg_le_1e-5"] >= 0.95

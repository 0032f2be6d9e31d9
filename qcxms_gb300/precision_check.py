"""Mixed-precision versus FP64 energies and gradients on a batch of molecules.

Usage: python -m qcxms_gb300.precision_check [--ntraj 64] [--natoms 60]

Runs the same seeded molecules through the FP64 SCC path and the mixed path
(FP32 iterations finished in FP64) and prints one JSON line with the largest
energy and gradient differences and the fraction of molecules within 1e-6 Eh
and 1e-5 Eh/Bohr. The FP64 path itself is checked against the CPU oracle by
the test suite.
"""
import argparse
import json

import numpy as np

from . import Batch, molgen


def run(ntraj=64, natoms=60, seed0=0, scc=None):
    """scc: (max_iter, econv, pconv, mixing) for both paths; default thresholds if None.
    At the default thresholds (1e-7 Eh, 1e-6) the two paths may stop at iterates
    whose gradients differ by several 1e-6 Eh/Bohr; tight thresholds isolate the
    arithmetic."""
    mols = []
    for t in range(ntraj):
        Z, xyz = molgen.random_chno(natoms, 900000 + seed0 + t)
        mols.append({"Z": Z, "xyz": xyz, "charge": 1})
    out = {}
    for prec in ("fp64", "mixed"):
        b = Batch(mols)
        b.set_precision(prec)
        if scc:
            b.set_scc(*scc)
        b.egrad()
        out[prec] = b.get()
        out[prec]["split_grad"] = b.split(out[prec]["grad"])
    ok = (out["fp64"]["status"] == 0) & (out["mixed"]["status"] == 0)
    de = np.abs(out["fp64"]["energy"] - out["mixed"]["energy"])[ok]
    dg = np.array([np.abs(a - b).max() for a, b, k in zip(out["fp64"]["split_grad"], out["mixed"]["split_grad"], ok)
                   if k])
    return {"ntraj": ntraj, "natoms": natoms, "both_converged": int(ok.sum()),
            "max_abs_dE": float(de.max()) if len(de) else None, "median_abs_dE": float(np.median(de)) if len(de) else None,
            "max_abs_dg": float(dg.max()) if len(dg) else None,
            "frac_dE_le_1e-6": float(np.mean(de <= 1e-6)) if len(de) else None,
            "frac_dg_le_1e-5": float(np.mean(dg <= 1e-5)) if len(dg) else None}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ntraj", type=int, default=64)
    ap.add_argument("--natoms", type=int, default=60)
    a = ap.parse_args()
    res = run(a.ntraj, a.natoms)
    tight = run(a.ntraj, a.natoms, scc=(100, 1e-10, 1e-8, 0.25))
    res["tight_scc"] = {k: tight[k] for k in ("both_converged", "max_abs_dE", "max_abs_dg")}
    print(json.dumps(res))


if __name__ == "__main__":
    main()

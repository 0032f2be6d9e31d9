"""Writes the small ensemble fixture tests/golden/TMPQCXMS/ in the layout of
QCxMS's wrstart (src/utility.f90:321-373): TMP.n/qcxms.start with the
trajectory number as (i4), eimp and tadd as (D22.14) and per atom
vx vy vz velof as (7D22.14), and TMP.n/start.xyz (xyz, Angstrom).

Fortran's Dw.d edit descriptor prints 0.<d digits>D<sign><2-digit exponent>,
right-justified in w columns; fortran_d() restates that. Run from the repo
root: python tests/golden/make_start_files.py"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from qcxms_gb300 import molgen  # noqa: E402
from qcxms_gb300.constants import AUTOAA, SYMBOLS  # noqa: E402


def fortran_d(x, w=22, d=14):
    if x == 0.0:
        s = "0." + "0" * d + "D+00"
    else:
        m, e = ("%.*E" % (d - 1, abs(x))).split("E")
        digits = m.replace(".", "")
        s = "0." + digits + "D%+03d" % (int(e) + 1)
        if x < 0:
            s = "-" + s
    return s.rjust(w)


def main():
    root = os.path.join(HERE, "TMPQCXMS")
    rng = np.random.default_rng(2024)
    for n, nat in [(1, 5), (2, 9), (10, 7)]:
        Z, xyz = molgen.random_chno(nat, 40 + n)
        xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
        vel = molgen.maxwell_boltzmann(Z, 800.0, 40 + n)
        velof = rng.uniform(0.5, 2.0, nat)
        d = os.path.join(root, "TMP.%d" % n)
        os.makedirs(d, exist_ok=True)
        with open(os.path.join(d, "qcxms.start"), "w") as f:
            f.write("%4d\n" % n)
            f.write(fortran_d(rng.uniform(0.05, 0.4)) + "\n")
            f.write(fortran_d(rng.uniform(1000.0, 3000.0)) + "\n")
            for a in range(nat):
                f.write("".join(fortran_d(v) for v in (*vel[a], velof[a])) + "\n")
        with open(os.path.join(d, "start.xyz"), "w") as f:
            f.write("%d\n\n" % nat)
            for a in range(nat):
                f.write("%-2s %20.14f %20.14f %20.14f\n" % (SYMBOLS[int(Z[a])], *(xyz[a] * AUTOAA)))


if __name__ == "__main__":
    main()

"""Batched production driver: every trajectory of a QCxMS ensemble on one GPU.

``bin/pqcxms`` starts one ``qcxms --prod`` process per ``TMPQCXMS/TMP.n``
directory; each runs the MD loop of ``src/md.f90`` (heating, bookkeeping, exit
rules) and, when the ion has fragmented, the fragment IPs of ``analyse``
(``src/analyse.f90``). Here all trajectories of the ensemble advance together:

1. ``read_ensemble`` loads ``start.xyz`` and ``qcxms.start`` of every trajectory;
2. one batch runs the MD with the heating (``impactscale``) and the exit rules
   on the device, in blocks of steps, until every trajectory has ended;
3. the averaged structures of the trajectories that ended in 2-10 fragments go
   through ``fragment_ips`` in one batch (neutral and cation of every fragment).

As in the reference, the IPs use the structure averaged over the last steps
(``axyz``, ``src/md.f90:352-362, 695``) with the fragment numbers of the final
structure. Differences from the reference: the electronic
temperature is the one given (the reference's default, ``ieetemp = 0``, gives
the constant 5000 + 20000 ax); the charge assignment of ``write_fragments``
and the output files are not written.

Usage: ``python -m qcxms_gb300.driver TMPQCXMS --etemp 17000 --max-steps 10000``
"""
import argparse
import json

import numpy as np

from . import Batch, constants, fragment_formula, fragment_ips, read_ensemble


def run_ensemble(root, etemp, charge=1, nfragexit=2, more=250, max_steps=10000, tstep_fs=0.5, block=100,
                 precision="mixed", ip_precision=0, ip_etemp=300.0):
    """Run every trajectory of ``root`` to its end; returns one dict per trajectory."""
    mols = read_ensemble(root, charge=charge)
    dt = tstep_fs * constants.FSTOAU
    b = Batch(mols, etemp=etemp)
    b.set_precision(precision)
    b.egrad()
    b.set_md_heating([m["eimp"] for m in mols], [m["tadd"] for m in mols], dt,
                     np.concatenate([m["velof"] for m in mols]))
    b.set_md_rules(nfragexit, more, max_steps)
    while True:
        active, _ = b.progress()
        if not active.any():
            break
        b.step(block, dt)
    st = b.md_state()
    r = b.get()
    axyz = b.md_avg_xyz()
    frag, nfrag = b.fragments(3.0, 1, 0)
    off = np.concatenate([[0], np.cumsum([len(m["Z"]) for m in mols])])
    out = []
    ends = []
    for i, m in enumerate(mols):
        sl = slice(off[i], off[i + 1])
        res = {"itrj": m["itrj"], "mdok": bool(st["mdok"][i]), "fragstate": int(st["fragstate"][i]),
               "nstep": int(st["nstep"][i]), "nfrag": int(nfrag[i]), "frag": frag[sl].tolist(),
               "fragT": st["fragT"][i, :max(1, min(int(nfrag[i]), 10))].tolist(), "energy": float(r["energy"][i]),
               "status": int(r["status"][i])}
        if nfrag[i] <= 10:
            # fragment masses and formulas (fragmass, src/fragments.f90:10-84)
            fm, formula = fragment_formula(m["Z"], frag[sl], m["mass"])
            res["fragm_amu"], res["formula"] = fm.tolist(), formula
        out.append(res)
        if 2 <= nfrag[i] <= 10:
            # analyse gets the averaged structure (src/md.f90:695, write_fragments.f90:102-106)
            ends.append((i, {"Z": m["Z"], "xyz": axyz[sl], "frag": frag[sl]}))
    b.close()
    if ends:
        ip, ef, ok = fragment_ips([s for _, s in ends], 1, etemp=ip_etemp, precision=ip_precision)
        for k, (i, _) in enumerate(ends):
            out[i]["fragip_eV"] = ip[k][:, 0].tolist()
            out[i]["ipok"] = bool(ok[k])
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("root", help="ensemble directory holding TMP.n/start.xyz and TMP.n/qcxms.start")
    ap.add_argument("--etemp", type=float, required=True, help="electronic temperature (K)")
    ap.add_argument("--charge", type=int, default=1)
    ap.add_argument("--nfragexit", type=int, default=2)
    ap.add_argument("--max-steps", type=int, default=10000)
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--out", default=None, help="write the results as JSON here")
    a = ap.parse_args()
    res = run_ensemble(a.root, a.etemp, a.charge, a.nfragexit, max_steps=a.max_steps, precision=a.precision)
    for t in res:
        print("traj %5d  mdok %d  fragstate %d  steps %6d  fragments %d  %s  IPs %s" %
              (t["itrj"], t["mdok"], t["fragstate"], t["nstep"], t["nfrag"], " ".join(t.get("formula", [])),
               " ".join("%.2f" % x for x in t.get("fragip_eV", []))))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(res, f, indent=1)


if __name__ == "__main__":
    main()

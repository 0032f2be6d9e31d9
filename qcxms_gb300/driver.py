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
structure, and the electronic temperature follows ``setetemp`` after every step
(``src/md.f90:443-446``): 5000 + 20000 ax (+ eimp ieetemp while heating). With
``--etemp`` given, the start's evaluation runs at that temperature
(``src/md.f90:167-171``); without it at ``setetemp(1, eimp)``.

Results: one JSON record per trajectory, and ``qcxms.res`` lines
(``qcx_format_res``) for the fragments of trajectories that ended in 2-10
fragments. Their charges come from the Boltzmann weights of the fragment IPs
(``boltz``, ``src/utility.f90:469-498``) at the trajectory's mean temperature:
the reference's own assignment (``src/write_fragments.f90:116-121``) reads
``fragip(i,0)``, outside its array, so its numbers are not reproducible.

Several GPUs of one node (``torchrun --nproc-per-node N -m qcxms_gb300.driver
...``): the trajectories are independent, as ``bin/pqcxms``'s processes are, so
each rank runs its own shard of the ensemble (``shard_ensemble``) on its own GPU
with no exchange on the data path; the ranks' result records are merged at the
end (``gather_results``), the one collective.

Usage: ``python -m qcxms_gb300.driver TMPQCXMS --max-steps 10000 --res qcxms.res``
"""
import argparse
import json
import os

import numpy as np

from . import Batch, basis, boltz, constants, format_res, fragment_formula, fragment_ips, read_ensemble


def shard_ensemble(mols, world):
    """Split the trajectories of an ensemble over ``world`` ranks with balanced
    work. An evaluation's cost is dominated by the SCC's eigen work, O(nao^3)
    per iteration with one CTA per molecule, so each trajectory is weighted by
    nao^3 and the trajectories are dealt largest first to the rank with the least
    weight so far (greedy longest-processing-time partition: the heaviest rank
    carries at most 4/3 of the best possible split's maximum, and at most the
    mean plus one trajectory's weight). Ties go to the lower rank and the lower
    index, so every rank computes the same split. Returns one ascending index
    list per rank; every index appears in exactly one."""
    if world < 1:
        raise ValueError("world must be at least 1")
    cost = [float(basis.nao_of(m["Z"])) ** 3 for m in mols]
    load = [0.0] * world
    out = [[] for _ in range(world)]
    for i in sorted(range(len(mols)), key=lambda i: (-cost[i], i)):
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += cost[i]
    return [sorted(s) for s in out]


def gather_results(res, world):
    """The result records of every rank merged in trajectory order (``itrj``):
    the only exchange between the ranks of a sharded run (gloo, host objects)."""
    if world == 1:
        return res
    import torch.distributed as dist
    parts = [None] * world
    dist.all_gather_object(parts, res)
    return sorted((t for p in parts for t in p), key=lambda t: t["itrj"])


def run_ensemble(root, etemp=-1.0, charge=1, nfragexit=2, more=250, max_steps=10000, tstep_fs=0.5, block=100,
                 precision="mixed", ip_precision=0, ip_etemp=300.0, ax=0.0, ieetemp=0.0, rank=0, world=1):
    """Run every trajectory of ``root`` to its end (with world > 1: this rank's
    shard of them); returns one dict per trajectory.
    etemp > 0: the start's electronic temperature; otherwise setetemp's."""
    mols = read_ensemble(root, charge=charge)
    if world > 1:
        mols = [mols[i] for i in shard_ensemble(mols, world)[rank]]
        if not mols:
            return []
    dt = tstep_fs * constants.FSTOAU
    b = Batch(mols, etemp=etemp if etemp > 0 else 5000.0)
    b.set_precision(precision)
    b.set_md_heating([m["eimp"] for m in mols], [m["tadd"] for m in mols], dt,
                     np.concatenate([m["velof"] for m in mols]))
    if etemp > 0:
        b.egrad()
        b.set_md_etemp(ax, ieetemp)  # later evaluations follow setetemp
    else:
        b.set_md_etemp(ax, ieetemp)  # the start too
        b.egrad()
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
            tmean = float(st["tav"][i]) / max(1, int(st["nstep"][i]))
            q = boltz(2, tmean, ip[k][:, :1])[:, 0] if ok[k] else np.zeros(len(out[i]["formula"]))
            out[i]["fragchrg"] = q.tolist()
            res = []
            for j in range(out[i]["nfrag"]):
                zs = [z for z in range(1, 19) if np.any((np.asarray(mols[i]["Z"]) == z) &
                                                        (np.asarray(out[i]["frag"]) == j + 1))]
                cnt = [int(np.sum((np.asarray(mols[i]["Z"]) == z) & (np.asarray(out[i]["frag"]) == j + 1)))
                       for z in zs]
                res.append(format_res(q[j], charge, out[i]["itrj"], 1, j + 1, zs, cnt))
            out[i]["res_lines"] = res
    return out


def gs_sampling(mols, nmax, path_fmt, etemp=298.15, tstep_fs=0.5, precision="fp64"):
    """Ground-state sampling run of every molecule (md with it = 0: NVE, the
    etemp of the ground-state runs, src/input.f90:142), writing path_fmt % i as
    qcxms.gs: nmax, then the coordinates and velocities at each of the nmax
    loop tops (the state before each step, src/md.f90:379-385). Returns the
    number of records written per molecule (fewer when a run stops)."""
    from . import write_gs
    dt = tstep_fs * constants.FSTOAU
    b = Batch(mols, etemp=etemp)
    b.set_precision(precision)
    b.egrad()
    xs, vs = [], []
    nrec = np.zeros(b.nmol, dtype=int)
    for k in range(nmax):
        r = b.get()
        active, _ = b.progress()
        xs.append(b.split(r["xyz"]))
        vs.append(b.split(r["vel"]))
        nrec += active > 0
        if not active.any():
            break
        b.step(1, dt)
    b.close()
    for i in range(len(mols)):
        n = int(nrec[i])
        write_gs(path_fmt % i, nmax, np.array([xs[k][i] for k in range(n)]), np.array([vs[k][i] for k in range(n)]))
    return nrec.tolist()


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("root", help="ensemble directory holding TMP.n/start.xyz and TMP.n/qcxms.start")
    ap.add_argument("--etemp", type=float, default=-1.0,
                    help="electronic temperature of the start (K); default: setetemp's, 5000 + 20000 ax")
    ap.add_argument("--ax", type=float, default=0.0)
    ap.add_argument("--ieetemp", type=float, default=0.0)
    ap.add_argument("--res", default=None, help="write the qcxms.res lines here")
    ap.add_argument("--charge", type=int, default=1)
    ap.add_argument("--nfragexit", type=int, default=2)
    ap.add_argument("--max-steps", type=int, default=10000)
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--out", default=None, help="write the results as JSON here")
    a = ap.parse_args()
    rank, world = int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))
    if world > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():  # without one, the first Batch fails with the library's error
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group("gloo")  # host records only; nothing on the data path
    res = run_ensemble(a.root, a.etemp, a.charge, a.nfragexit, max_steps=a.max_steps, precision=a.precision,
                       ax=a.ax, ieetemp=a.ieetemp, rank=rank, world=world)
    res = gather_results(res, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
        if rank != 0:
            return
    if a.res:
        with open(a.res, "w") as f:
            for t in res:
                for line in t.get("res_lines", []):
                    f.write(line + "\n")
    for t in res:
        print("traj %5d  mdok %d  fragstate %d  steps %6d  fragments %d  %s  IPs %s" %
              (t["itrj"], t["mdok"], t["fragstate"], t["nstep"], t["nfrag"], " ".join(t.get("formula", [])),
               " ".join("%.2f" % x for x in t.get("fragip_eV", []))))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(res, f, indent=1)


if __name__ == "__main__":
    main()

"""Trajectory-step throughput of the GFN2-xTB MD hot path on one GB300.

Workload (default): 256 seeded C/H/N/O radical cations with 5-40 atoms
(element fractions C 0.35, H 0.5, N 0.05, O 0.1), charge +1, initial
temperatures uniform in 1000-4000 K, 0.5 fs leapfrog steps, FP64, one captured
CUDA graph per MD step. A step is leapfrog + energy + analytic gradient for
every trajectory; the metric counts completed trajectory-steps per second.

Lines printed (one JSON line):
  default           the CUDA path (libqcxgpu.so), device-resident state
  --impl reference  the CPU restatement of the same step (the QCxMS reference
                    path itself needs a Fortran toolchain and tblite, neither of
                    which exists here), all host threads, bounded sample

Multi-GPU: trajectories are independent; with torchrun each rank runs its own
shard (disjoint seeds) with no collective on the data path.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GFN2-xTB trajectory-steps/s"
# DRAM bytes (read + write) of one k_scc launch per molecule, from an ncu capture of a
# launch over 2 molecules of the 16-trajectory batch (1.845 MB read, 0.050 MB written);
# a launch touches each molecule's own data only.
SCC_DRAM_BYTES_PER_MOLECULE = (1.844736e6 + 4.992e4) / 2


def bf16_tensor_peak():
    """Dense bf16 tensor peak (TFLOP/s): the measured figure of MEASURED_PEAKS.json when
    the file is there, else the fallback of one earlier GB300 measurement."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        for k in ("bf16_tflops", "bf16_tflops_sustained"):
            if k in d:
                return float(d[k]), "MEASURED_PEAKS.json " + k
    except (OSError, ValueError):
        pass
    return 1900.0, "fallback (1.9 PFLOP/s bf16 burst, one earlier GB300 measurement)"
NTRAJ, NMIN, NMAX = 256, 5, 40
# SCC iterations one step grants the largest molecule of a molecule group (a
# molecule of n AOs gets 20 (nmax / n)^2, nmax the group's largest); an SCC
# that needs more continues in the next step while its trajectory waits.
SCC_BUDGET = 20
# candidates of the budget autotuner of paced runs (0, no budget, measured
# 40-50 % slower on the 256-trajectory workload, is left out; 10 suits the
# collision workload of large ions)
AUTOTUNE_BUDGETS = (10, 20, 40, 60)
# MD steps of the largest molecules' group per timed paced call (the other
# groups take as many as fit into the same time)
PACED_STEPS = 1
DT_FS = 0.5
ETEMP = 300.0


def workload(rank, ntraj=None, kind="batch"):
    from qcxms_gb300 import molgen
    if kind == "cid":
        n = ntraj or 4096
        return molgen.cid_workload(n, 10, 80, seed0=rank * n)
    n = ntraj or NTRAJ
    return molgen.batch_workload(n, NMIN, NMAX, seed0=rank * NTRAJ)


WORKLOAD_NAMES = {
    "batch": "256 C/H/N/O cations, 5-40 atoms, T0 1000-4000 K, 0.5 fs",
    "cid": "4096 C/H/N/O/S cations, 10-80 atoms, + Ar at 40 eV lab frame, b ~ U(0, 2 A), 0.5 fs",
}


def reduce_over_ranks(t, done, world, device):
    """Whole-job figures of weakly scaled ranks: the slowest rank's time (max) and
    the units all ranks processed (sum). No other collective touches the data path."""
    import torch
    v = torch.tensor([t, done], dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist
        tmax, dsum = v[0:1].clone(), v[1:2].clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        dist.all_reduce(dsum, op=dist.ReduceOp.SUM)
        return float(tmax[0]), float(dsum[0])
    return float(v[0]), float(v[1])


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def scc_flops(nao, iters):
    """Algorithmic FLOPs of the SCC kernel: per molecule k*(9n^3 eigensolve + 2n^3
    density) + 2n^3 energy-weighted density (fixed counting convention)."""
    n3 = nao.astype(np.float64) ** 3
    return float(np.sum(iters * 11.0 * n3 + 2.0 * n3))


def measured_peak(torch, dtype):
    """Dense throughput of this GPU on CUDA cores (cuBLAS GEMM 4096^3 in dtype,
    TF32 tensor cores off for FP32; best of 5), TFLOP/s."""
    n = 4096
    torch.backends.cuda.matmul.allow_tf32 = False
    a = torch.randn(n, n, dtype=dtype, device="cuda")
    b = torch.randn(n, n, dtype=dtype, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        torch.cuda.synchronize()
        best = max(best, 2.0 * n ** 3 / (s.elapsed_time(e) * 1e-3) / 1e12)
    del a, b
    return best


def stratified(mols, k):
    """k molecules spread evenly over the size order of mols (largest first)."""
    order = sorted(range(len(mols)), key=lambda i: -len(mols[i]["Z"]))
    if k >= len(mols):
        return [mols[i] for i in order]
    pick = np.linspace(0, len(mols) - 1, k).round().astype(int)
    return [mols[order[i]] for i in pick]


def cpu_sample(mols, seconds, nthreads, chunk=10):
    """Time the oracle restatement on a bounded sample of the workload: calls of
    `chunk` MD steps each (trajectories largest first under a dynamic schedule,
    all threads busy at once), until `seconds` have passed. A trajectory whose
    calculation fails stops, as on the GPU. The rate is the accepted steps over
    the threads' busy time divided by the thread count: the idle tail of a
    call, when fewer trajectories than threads are left, is not counted,
    because a full ensemble run (bin/pqcxms: one process per trajectory, as many
    at once as cores) keeps every core busy with the next trajectory. Returns
    (trajectory-steps/s, calls, seconds, accepted steps, wall-clock rate)."""
    import oracle
    from qcxms_gb300 import constants
    kT = ETEMP * constants.KB_AU
    dt = DT_FS * constants.FSTOAU
    mols = [dict(m) for m in mols]
    # initial gradients (setup, untimed)
    rc, _, grads, _ = oracle.egrad_batch(mols, kT, nthreads=nthreads)
    active = (rc == 0).astype(np.int32)
    steps_done = np.zeros(len(mols), dtype=np.int32)
    busy = np.zeros(len(mols))
    done, calls, busy_sum, t0 = 0, 0, 0.0, time.perf_counter()
    while time.perf_counter() - t0 < seconds and active.any():
        fails, xyz, vel, g, ep, it = oracle.md_batch(mols, chunk, dt, grads, kT, nthreads=nthreads, active=active,
                                                     steps_done=steps_done, busy_s=busy)
        busy_sum += float(busy.sum())
        off = 0
        for i, m in enumerate(mols):
            n = len(m["Z"])
            m["xyz"], m["vel"], grads[i] = xyz[off:off + n], vel[off:off + n], g[off:off + n]
            off += n
        done += int(steps_done.sum())
        calls += 1
    el = time.perf_counter() - t0
    return done / (busy_sum / nthreads), calls, el, done, done / el


def cpu_sample_desc(sample, ntraj, calls, chunk, el, done, wall_rate):
    nat = [len(m["Z"]) for m in sample]
    return ("%d of the %d trajectories, stratified by size (%d-%d atoms, mean %.1f), %d calls of %d MD steps "
            "(%d accepted trajectory-steps, %.1f s); CPU FP64 restatement of leapfrog + energy/gradient + checkqc, "
            "OpenMP over trajectories, largest first, failed trajectories stop; rate over the threads' busy time "
            "(wall-clock rate with the idle tails of the calls: %.1f)"
            % (len(sample), ntraj, min(nat), max(nat), float(np.mean(nat)), calls, chunk, done, el, wall_rate))


def plain_fp64_single(qg, constants, nsteps=6):
    """Plain FP64 single-trajectory path: one C6H12O2 radical cation (20 atoms,
    charge +1, etemp 300 K), 500 K Maxwell-Boltzmann velocities, 0.5 fs steps."""
    import torch
    from qcxms_gb300 import molgen
    Z, xyz = molgen.c6h12o2()
    m = {"Z": Z, "xyz": xyz, "vel": molgen.maxwell_boltzmann(Z, 500.0, 1234), "mass": molgen.masses(Z), "charge": 1}
    b = qg.Batch([m], etemp=ETEMP)
    b.set_precision("fp64")
    b.egrad()
    dt = DT_FS * constants.FSTOAU
    b.step(2, dt)
    b.sync()
    stream = torch.cuda.ExternalStream(b.stream())
    _, s0 = b.progress()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record(stream)
    b.step(nsteps, dt)
    e.record(stream)
    e.synchronize()
    _, s1 = b.progress()
    done = float(np.sum(s1 - s0))
    b.close()
    return done / (s.elapsed_time(e) * 1e-3)


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    mols = workload(0)
    ncpu = os.cpu_count() or 1
    sample = stratified(mols, 2 * ncpu)
    vals = []
    desc = ""
    for _ in range(max(1, args.steps)):
        v, calls, el, done, wall = cpu_sample(sample, max(4.0, 20.0 / max(1, args.steps)), ncpu)
        vals.append(v)
        desc = cpu_sample_desc(sample, NTRAJ, calls, 10, el, done, wall)
    v = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "trajectory-steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * NTRAJ / v, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD_NAMES["batch"], "ntraj_per_gpu": NTRAJ, "atoms": [NMIN, NMAX],
                   "etemp_K": ETEMP, "precision": "fp64 (CPU restatement)"},
        "cpu_baseline": {"value": v, "unit": "trajectory-steps/s", "cores": ncpu, "kind": "port", "sample": desc},
        "e2e": {"value": v, "unit": "trajectory-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def accuracy_check(b, mols, k=32):
    """Energies and gradients of the batch's last evaluation against FP64 on a
    stratified sample of k running trajectories at their current geometries:
    the CPU FP64 oracle and the GPU FP64 path."""
    import oracle
    import qcxms_gb300 as qg
    from qcxms_gb300 import constants
    r = b.get()
    act, _ = b.progress()
    xyz = b.split(r["xyz"])
    grad = b.split(r["grad"])
    cand = [i for i in range(b.nmol) if act[i] and r["status"][i] == 0]
    cand.sort(key=lambda i: -len(mols[i]["Z"]))
    pick = [cand[j] for j in np.linspace(0, len(cand) - 1, min(k, len(cand))).round().astype(int)]
    sub = [{"Z": mols[i]["Z"], "xyz": xyz[i], "charge": mols[i]["charge"]} for i in pick]
    rc, e_o, g_o, _ = oracle.egrad_batch(sub, ETEMP * constants.KB_AU, nthreads=os.cpu_count() or 1)
    b64 = qg.Batch(sub, etemp=ETEMP)
    b64.set_precision("fp64")
    b64.egrad()
    r64 = b64.get()
    g64 = b64.split(r64["grad"])
    b64.close()
    ok = [j for j in range(len(pick)) if rc[j] == 0 and r64["status"][j] == 0]
    dE = np.array([abs(r["energy"][pick[j]] - e_o[j]) for j in ok])
    dg = np.array([np.abs(grad[pick[j]] - g_o[j]).max() for j in ok])
    dE64 = np.array([abs(r["energy"][pick[j]] - r64["energy"][j]) for j in ok])
    dg64 = np.array([np.abs(grad[pick[j]] - g64[j]).max() for j in ok])
    nat = [len(s["Z"]) for s in sub]
    return {"sample": "%d running trajectories at their current geometries, stratified by size (%d-%d atoms)"
                      % (len(ok), min(nat), max(nat)),
            "vs_fp64_oracle": {"max_abs_dE_Eh": float(dE.max()), "max_abs_dg_Eh_per_bohr": float(dg.max()),
                               "frac_dE_within_1e-6": float(np.mean(dE <= 1e-6)),
                               "frac_dg_within_1e-5": float(np.mean(dg <= 1e-5))},
            "vs_gpu_fp64": {"max_abs_dE_Eh": float(dE64.max()), "max_abs_dg_Eh_per_bohr": float(dg64.max())},
            "note": "both sides at the default SCC thresholds (1e-7 Eh, 1e-6); differences include where "
                    "two converged SCC runs stop"}


def run_gpu(args):
    import torch
    import qcxms_gb300 as qg
    from qcxms_gb300 import constants

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dt = DT_FS * constants.FSTOAU
    mols = workload(rank, args.ntraj, args.workload)
    b = qg.Batch(mols, etemp=ETEMP)
    b.set_precision(args.precision)
    b.set_guess(args.guess)
    if args.scc_budget:
        b.set_scc_budget(args.scc_budget)
    b.egrad()
    if args.md_rules:
        # the electron-impact MD loop's heating, bookkeeping and exit rules on the
        # device (impactscale over the first 100 steps, nfragexit 2, more 250)
        rng = np.random.default_rng(11 + rank)
        b.set_md_heating(rng.uniform(0.1, 0.3, b.nmol), np.full(b.nmol, 100 * dt), dt)
        b.set_md_rules(2, 250, 100000)
    b.sync()
    stream = torch.cuda.ExternalStream(b.stream())
    nao, nat = b.sizes()
    l2_flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    paced = args.stepping == "paced"

    kstep = args.md_steps if args.md_steps else (PACED_STEPS if paced else 1)

    def one_step():
        if paced:
            b.step_paced(kstep, dt)
        else:
            b.step(kstep, dt)

    # ---- device-resident timing: graph replay, L2 flushed between steps ----
    # Whole-batch steps: timing marks inside the step graph give the SCC phase of
    # every timed step (first group's SCC start to last group's SCC end). Paced
    # steps: the groups' SCC launches overlap one another and the other kernels,
    # so the SCC rate is taken over the whole timed region.
    b.set_timing(not paced)
    tune = None
    if paced and not args.no_autotune:
        # untimed: pick the per-step SCC budget and its scale on a second batch of
        # the same trajectories (real MD steps), so that the timed batch starts from
        # the workload's initial state: the batch ages over a run (trajectories
        # fragment and stop, small molecules run ahead) and 24 tuning calls on the
        # timed batch itself lowered the timed rate by ~15 %
        tb = qg.Batch(mols, etemp=ETEMP)
        tb.set_precision(args.precision)
        tb.set_guess(args.guess)
        tb.egrad()
        (best, per_group), rates = tb.autotune_budget(AUTOTUNE_BUDGETS, calls=2, tstep=dt, steps_per_call=kstep)
        tb.close()
        b.set_scc_budget(best)
        b.set_scc_budget_scale(bool(per_group))
        tune = {"candidates": {"%d/%s" % (k, "group" if g else "batch"): round(v, 1) for (k, g), v in rates.items()},
                "chosen": best, "scale": "largest molecule of each group" if per_group else "largest molecule of the batch",
                "tuned_on": "a second batch of the same trajectories"}
    for _ in range(args.warmup):
        one_step()
    barrier()
    total_ms = 0.0
    launches = 0
    scc_flops_sum = scc_ms_sum = 0.0
    scc_iters_all = []
    scc_launches = []
    phase = {"step": [], "scc_span": [], "scc_sum": [], "integrals_sum": [], "gradient_sum": []}
    # End to end through the public API with pinned host buffers, on the same
    # calls as the device-resident timing: every timed step loads coordinates and
    # velocities from pinned host buffers (qcx_batch_load_state: running
    # trajectories continue, stopped ones stay stopped), runs the step between
    # two events on the batch stream (the device-resident time: the copies
    # precede the first event in stream order) and reads coordinates, velocities
    # and energies back; the host clock around all three is the end-to-end time.
    # Both rates count the same completed steps.
    r = b.get()
    hx = torch.from_numpy(r["xyz"]).pin_memory()
    hv = torch.from_numpy(r["vel"]).pin_memory()
    he = torch.zeros(b.nmol, dtype=torch.float64).pin_memory()
    e2e_s = dev_done = 0.0

    with ClockSampler(local) as clk:
        barrier()
        for _ in range(args.steps):
            _, st_before_steps = b.progress()
            isum0 = b.iterations()
            l2_flush.zero_()
            torch.cuda.synchronize()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0 = time.perf_counter()
            b.load_state_ptr(hx.data_ptr(), hv.data_ptr())
            s.record(stream)
            one_step()
            e.record(stream)
            b.get_ptr(hx.data_ptr(), hv.data_ptr(), he.data_ptr())
            e2e_s += time.perf_counter() - t0
            e.synchronize()
            step_ms = s.elapsed_time(e)
            total_ms += step_ms
            launches += b.kernel_launches()
            st, it = b.status_iters()
            _, st_after_steps = b.progress()
            # SCC work of this step from the device's iteration counters: 11 n^3 per
            # iteration, 2 n^3 per completed evaluation (all launches of the step)
            dit = (b.iterations() - isum0).astype(np.float64)
            nev = (st_after_steps - st_before_steps).astype(np.float64)
            dev_done += float(nev.sum())
            n3 = nao.astype(np.float64) ** 3
            scc_flops_sum += float(np.sum(dit * 11.0 * n3 + nev * 2.0 * n3))
            scc_iters_all.append(it[(nev > 0) & ((st & qg.STATUS_SCC_PENDING) == 0)])
            scc_launches.append(float(nev.sum() + np.sum((st & qg.STATUS_SCC_PENDING) != 0)))
            if paced:
                scc_ms_sum += step_ms
                phase["step"].append(step_ms)
            else:
                tm = b.timing()
                scc_ms_sum += tm["scc_span"]
                mk = tm["marks"]
                phase["step"].append(tm["step"])
                phase["scc_span"].append(tm["scc_span"])
                phase["scc_sum"].append(tm["scc_sum"])
                phase["integrals_sum"].append(float(np.sum(mk[:, 1] - mk[:, 0])))
                phase["gradient_sum"].append(float(np.sum(mk[:, 3] - mk[:, 2])))
        barrier()
    act_end, steps1 = b.progress()
    total_ms, done_all = reduce_over_ranks(total_ms, dev_done, world, "cuda")
    value = done_all / (total_ms * 1e-3)
    iters_cat = np.concatenate(scc_iters_all) if scc_iters_all else np.zeros(1)
    e2e_s, e2e_done = reduce_over_ranks(e2e_s, dev_done, world, "cuda")
    e2e = e2e_done / e2e_s
    h2d = 2 * 3 * 8 * b.natom
    d2h = 2 * 3 * 8 * b.natom + 8 * b.nmol

    # ---- roofline of the dominant kernel (SCC) over the timed steps ----
    achieved = scc_flops_sum / (scc_ms_sum * 1e-3) / 1e12
    # The mixed kernel runs its O(n^3) work on the FP32 pipes (FP32 iterations and
    # the double-float finishing iterations); the FP64 kernel on the FP64 pipe.
    mixed = args.precision == "mixed"
    peak = measured_peak(torch, torch.float32 if mixed else torch.float64)
    tpk, tsrc = bf16_tensor_peak()
    plain = plain_fp64_single(qg, constants) if rank == 0 and not args.no_plain else None
    accuracy = accuracy_check(b, mols) if rank == 0 and mixed and not args.no_accuracy else None

    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            ncpu = os.cpu_count() or 1
            sample = stratified(workload(0), 2 * ncpu)
            v, calls, el, cdone, wall = cpu_sample(sample, 12.0, ncpu)
            cpu = {"value": v, "unit": "trajectory-steps/s", "cores": ncpu, "kind": "port",
                   "sample": cpu_sample_desc(sample, NTRAJ, calls, 10, el, cdone, wall)}
        med = {k: round(statistics.median(v), 3) for k, v in phase.items() if v}
        if paced:
            _, gsteps, gms = b.group_info()
            execution = ("size-bucketed: 8 molecule groups by size, each stepping from its own CUDA graph on its own "
                         "stream; one timed step = one paced call in which the largest molecules' group takes %d MD "
                         "steps and the groups took %s steps" % (kstep, gsteps.tolist()))
            unit = ("all k_scc launches of the timed region (the groups' launches overlap one another and the "
                    "integral and gradient kernels); time = the timed region; FLOPs from the device's per-molecule "
                    "iteration counters")
        else:
            execution = ("one CUDA graph per MD step, 8 molecule groups on separate streams; one timed step = %d MD "
                         "steps of the whole batch" % kstep)
            unit = ("the SCC phase of one timed step: one k_scc launch per molecule group (8, concurrent); time = "
                    "first group's SCC start to last group's SCC end, from event marks inside the step graph; "
                    "FLOPs from the device's per-molecule iteration counters")
        line = {
            "metric": METRIC, "value": value, "unit": "trajectory-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32+df64" if mixed else "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD_NAMES[args.workload], "ntraj_per_gpu": b.nmol,
                       "atoms": [NMIN, NMAX] if args.workload == "batch" else [10, 81],
                       "etemp_K": ETEMP, "precision": args.precision, "scc_guess": args.guess,
                       "scc_iteration_limit": 250,
                       "scc_budget_per_step": tune["chosen"] if tune else args.scc_budget,
                       "scc_budget_autotune": tune,
                       "arithmetic": ("FP32 SCC iterations, then double-float (hi+lo FP32) finishing iterations; "
                                      "FP64 integrals, potentials of the finishing iterations, Fermi level, Broyden, "
                                      "energies and gradient") if mixed else "FP64 throughout",
                       "md_rules_on_device": bool(args.md_rules),
                       "execution": execution,
                       "md_steps_per_timed_step": kstep,
                       "l2": "flushed between timed steps (256 MiB write)",
                       "mean_nao": float(np.mean(nao)),
                       "mean_scc_iters": float(np.mean(iters_cat)) if len(iters_cat) else 0.0,
                       "active_trajectories_end": int(np.sum(act_end)),
                       "stopped_trajectories": int(b.nmol - np.sum(act_end))},
            "e2e": {"value": e2e, "unit": "trajectory-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "roofline": {"bound": "fp32" if mixed else "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak,
                         "traffic": SCC_DRAM_BYTES_PER_MOLECULE * float(np.mean(scc_launches)),
                         "kernel": "k_scc",
                         "launch_unit": unit,
                         "peak_source": "measured in this run: cuBLAS %s GEMM 4096^3 on CUDA cores "
                                        "(MEASURED_PEAKS.json holds only HBM and bf16 tensor peaks)"
                                        % ("FP32" if mixed else "FP64"),
                         "flops_convention": "algorithmic, per molecule: 11 n^3 per SCC iteration (9 n^3 eigensolve, "
                                             "2 n^3 density) + 2 n^3 per completed evaluation (W)",
                         "tensor": {"peak": tpk, "unit": "TFLOP/s", "frac": achieved / tpk, "peak_source": tsrc,
                                    "note": "the same achieved FLOPs against the dense bf16 tensor peak: the "
                                            "kernel's FP32 products run on the tensor cores (split-TF32), its "
                                            "eigensolver sweeps and FP64 work on the CUDA cores"}},
            "kernel_ms": med,
            "clocks": clk.summary(),
        }
        if accuracy:
            line["accuracy"] = accuracy
        if cpu:
            line["cpu_baseline"] = cpu
        if plain:
            line["config"]["plain_fp64_single_trajectory_steps_per_s"] = plain
            line["config"]["speedup_vs_plain_fp64_single_trajectory"] = value / plain
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_fragip(args):
    """Fragment IPs at trajectory ends (src/analyse.f90:13-467, GFN2): 256
    structures that fell into 2-5 fragments (molgen.fragmented), the neutral
    and cation of every fragment in one batch per call of qcx_fragment_ips.
    Every call goes through the C ABI with host buffers (batch set-up, copies,
    kernels, results), so the value is end to end. One GPU (replicas only)."""
    import qcxms_gb300 as qg
    from qcxms_gb300 import molgen
    n = args.ntraj or NTRAJ
    structs = [molgen.fragmented(s, 2 + s % 4) for s in range(n)]
    prec = 1 if args.precision == "mixed" else 0
    nfrag = sum(int(np.max(s["frag"])) for s in structs)
    # single points on the GPU: neutral and cation of every fragment, less the
    # bare protons (no electrons: self energy on the host); their coordinates
    # go in and their energies and status words come out every call
    nsp = h2d = 0
    for s in structs:
        for f in range(1, int(np.max(s["frag"])) + 1):
            na = int(np.sum(s["frag"] == f))
            lone_h = na == 1 and int(s["Z"][s["frag"] == f][0]) == 1
            nsp += 1 if lone_h else 2
            h2d += (1 if lone_h else 2) * (24 * na + 4 * na)
    d2h = 12 * nsp
    for _ in range(args.warmup):
        qg.fragment_ips(structs, 1, precision=prec)
    ts = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            ip, ef, ok = qg.fragment_ips(structs, 1, precision=prec)
            ts.append(time.perf_counter() - t0)
    el = sum(ts)
    value = n * args.steps / el
    cpu = None
    if not args.no_cpu_baseline:
        import oracle
        done, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < 10.0 and done < n:
            s = structs[done]
            oracle.fragment_ips(s["Z"], s["xyz"], s["frag"], 1)
            done += 1
        cel = time.perf_counter() - t0
        cpu = {"value": done / cel, "unit": "structures/s", "cores": 1, "kind": "port",
               "sample": "first %d of the %d structures (%.1f s), CPU FP64 restatement, one thread" % (done, n, cel)}
    line = {"metric": "fragment-IP structures/s", "value": value, "unit": "structures/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec == 0 else "f64/f32", "data": "synthetic",
            "config": {"workload": "%d fragmented C/H/N/O structures, 2-5 fragments, neutral + cation per "
                                   "fragment, 300 K" % n, "fragments": nfrag, "gpu_single_points": nsp,
                       "precision": args.precision, "ipok_fraction": float(np.mean(ok)),
                       "l2": "inputs copied from host every call (batch built per call)"},
            "e2e": {"value": value, "unit": "structures/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "clocks": clk.summary(), "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ntraj", type=int, default=None, help="smaller batch for profiling runs (default 256)")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--workload", default="batch", choices=["batch", "cid", "fragip"])
    ap.add_argument("--no-plain", action="store_true", help="skip the single-trajectory FP64 reference leg")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP64 accuracy check after the timed steps")
    ap.add_argument("--md-rules", action="store_true",
                    help="run the MD heating, bookkeeping and exit rules on the device in the timed steps "
                         "(the end-to-end leg sets new coordinates, which switches them off)")
    ap.add_argument("--stepping", default="paced", choices=["paced", "graph"],
                    help="paced: every molecule group steps from its own graph, small molecules several times per "
                         "step of the largest (default); graph: one graph per step for the whole batch")
    ap.add_argument("--no-autotune", action="store_true",
                    help="paced runs: keep --scc-budget instead of picking the budget by measurement")
    ap.add_argument("--scc-budget", type=int, default=SCC_BUDGET,
                    help="SCC iterations per step for the largest molecule (0: none); slower SCCs continue in the "
                         "next step while their trajectory waits, as independent trajectory processes would")
    ap.add_argument("--md-steps", type=int, default=0,
                    help="MD steps per timed step (paced: of the largest molecules' group); default %d paced, "
                         "1 graph" % PACED_STEPS)
    ap.add_argument("--guess", default="zero", choices=["zero", "previous"],
                    help="SCC start: zero moments every step (the reference's behaviour, default) or the "
                         "trajectory's converged moments of the previous step (opt-in)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "fragip":
        run_fragip(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

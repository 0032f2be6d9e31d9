"""GPU parity: the CUDA path (through the C ABI) against the CPU FP64 oracle.

Tolerances (FP64 path): energies 1e-8 Eh, gradients 1e-7 Eh/Bohr, integrals
1e-12; both sides run the same SCC algorithm and thresholds, so differences
come only from floating-point summation order and the eigensolver."""
import numpy as np
import pytest

import qcxms_gb300 as qg
from qcxms_gb300 import constants, molgen
from tests import molecules

pytestmark = pytest.mark.gpu
KT = 300.0 * constants.KB_AU
# Tight SCC thresholds: both sides converge to the same fixed point far below
# the default thresholds, so differences measure the arithmetic, not where the
# iteration happened to stop. With the default thresholds (1e-7 Eh, 1e-6)
# gradients of two correct implementations may differ by a few 1e-6 Eh/Bohr.
TIGHT_GPU = (100, 1e-11, 1e-9, 0.25)
DEFAULT_GRAD_TOL = 5e-6


def tight_opts(oracle_lib):
    return oracle_lib.default_opts(econv=1e-11, pconv=1e-9)


def _batch(mols, etemp=300.0):
    return qg.Batch([{"Z": Z, "xyz": xyz, "charge": c} for Z, xyz, c in mols], etemp=etemp)


@pytest.mark.parametrize("name", sorted(molecules.ALL_SMALL))
def test_energy_gradient_small(gpu, oracle_lib, name):
    Z, xyz, c = molecules.ALL_SMALL[name]()
    b = _batch([(Z, xyz, c)])
    b.set_scc(*TIGHT_GPU)
    b.egrad()
    r = b.get()
    rc, e, g, q, info = oracle_lib.egrad(Z, xyz, c, kT=KT, opts=tight_opts(oracle_lib))
    # egrad's checkqc (src/iniqm.f90:650) applies to both: H2+ along z has no x/y
    # gradient and a single atom none at all, so gnorm = 0 rejects them (E = 0)
    ok, e_chk = oracle_lib.checkqc(e, g, q, c)
    assert r["status"][0] == (0 if ok else qg.STATUS_CHECKQC)
    assert r["energy"][0] == e_chk if not ok else abs(r["energy"][0] - e) < 1e-8
    t = b.energy_terms(0)
    e_dev = (t["band"] + t["ies"] + t["e3"] + t["aes"] + t["axc"] + t["disp"] + t["ts"]) + (t["atm"] + t["rep"])
    assert abs(e_dev - e) < 1e-8
    assert np.abs(r["grad"] - g).max() < 1e-7
    assert np.abs(r["qat"] - q).max() < 1e-7


def test_integrals_match_oracle(gpu, oracle_lib):
    Z, xyz, c = molecules.h2s_ch_cation()
    b = _batch([(Z, xyz, c)])
    b.egrad()
    S, H0, Dm, Qm, cn, cnd = oracle_lib.integrals(Z, xyz)
    assert np.abs(b.matrix(0, 0) - S).max() < 1e-12
    assert np.abs(b.matrix(0, 1) - H0).max() < 1e-12
    P = oracle_lib.scc(Z, xyz, c, kT=KT)[0]
    assert np.abs(b.matrix(0, 8) - P).max() < 1e-7


def test_c6h12o2_and_random_batch(gpu, oracle_lib):
    # Converging to 1e-11 Eh / 1e-9 takes 40-60 iterations on these cations; the
    # GPU's SCC path differs from the oracle's (summation order of the pair sums)
    # and may need more, so a molecule near the limit of 100 can stop there on
    # one side. Every molecule both sides converged is compared.
    mols = [molecules.c6h12o2()] + [molecules.random_chno(n, s) for s, n in enumerate([5, 12, 23, 31, 40])]
    b = _batch(mols)
    b.set_scc(*TIGHT_GPU)
    b.egrad()
    r = b.get()
    g = b.split(r["grad"])
    both = 0
    for i, (Z, xyz, c) in enumerate(mols):
        rc, e, gref, q, info = oracle_lib.egrad(Z, xyz, c, kT=KT, opts=tight_opts(oracle_lib))
        if rc != 0 or r["status"][i] != 0:
            continue
        both += 1
        assert abs(r["energy"][i] - e) < 1e-8, (i, r["energy"][i], e)
        assert np.abs(g[i] - gref).max() < 1e-7
    assert both >= 5


def test_default_thresholds_within_scc_tolerance(gpu, oracle_lib):
    mols = [molecules.c6h12o2()] + [molecules.random_chno(n, s) for s, n in enumerate([12, 31])]
    b = _batch(mols)
    b.egrad()
    r = b.get()
    g = b.split(r["grad"])
    for i, (Z, xyz, c) in enumerate(mols):
        rc, e, gref, q, info = oracle_lib.egrad(Z, xyz, c, kT=KT)
        assert r["status"][i] == 0
        assert abs(r["energy"][i] - e) < 1e-7
        assert np.abs(g[i] - gref).max() < DEFAULT_GRAD_TOL


def test_batch_equals_single_runs(gpu):
    mols = [molecules.random_chno(n, 50 + n) for n in (7, 19, 33)]
    b = _batch(mols)
    b.egrad()
    r = b.get()
    for i, m in enumerate(mols):
        s = _batch([m])
        s.egrad()
        rs = s.get()
        assert abs(rs["energy"][0] - r["energy"][i]) < 1e-12
        assert np.abs(rs["grad"] - b.split(r["grad"])[i]).max() < 1e-12


def test_dropin_get_xtb_egrad(gpu, oracle_lib, tmp_path):
    Z, xyz, c = molecules.c6h12o2()
    out = tmp_path / "xtb.last"
    q, e, g, stat = qg.get_xtb_egrad(Z, xyz, c, 2, qg.gfn2_xtb, 300.0, str(out))
    assert stat == 0 and out.exists()
    rc, e0, g0, q0, _ = oracle_lib.egrad(Z, xyz, c, kT=KT)
    assert abs(e - e0) < 1e-8 and np.abs(g - g0).max() < DEFAULT_GRAD_TOL
    # second call with moved atoms reuses the cached device state
    xyz2 = xyz + 0.01
    q, e2, g2, stat = qg.get_xtb_egrad(Z, xyz2, c, 2, qg.gfn2_xtb, 300.0)
    rc, e1, g1, _, _ = oracle_lib.egrad(Z, xyz2, c, kT=KT)
    assert stat == 0 and abs(e2 - e1) < 1e-8
    assert qg.get_xtb_egrad(Z, xyz, c, 2, qg.gfn1_xtb, 300.0)[3] == 5


def test_gpu_gradient_central_differences(gpu):
    Z, xyz, c = molecules.ch2o_cation()
    b = _batch([(Z, xyz, c)])
    b.set_scc(100, 1e-12, 1e-10, 0.25)
    b.egrad()
    g = b.get()["grad"]
    h = 1e-4
    for a in range(len(Z)):
        for k in range(3):
            e = []
            for sgn in (1, -1):
                x = xyz.copy(); x[a, k] += sgn * h
                b.set_state(xyz=x)
                b.egrad()
                e.append(b.get()["energy"][0])
            assert abs((e[0] - e[1]) / (2 * h) - g[a, k]) < 1e-6


def test_md_steps_match_oracle(gpu, oracle_lib):
    mols = []
    for s, n in enumerate([6, 14, 20]):
        Z, xyz = molgen.random_chno(n, 200 + s)
        mols.append({"Z": Z, "xyz": xyz, "vel": molgen.maxwell_boltzmann(Z, 1500.0, s), "mass": molgen.masses(Z),
                     "charge": 1})
    b = qg.Batch(mols)
    b.set_scc(*TIGHT_GPU)
    b.egrad()
    g0 = b.split(b.get()["grad"])
    nsteps, dt = 10, 0.5 * constants.FSTOAU
    b.step(nsteps, dt)
    r = b.get()
    fails, xyz, vel, grad, epot, iters = oracle_lib.md_batch(mols, nsteps, dt, g0, KT, opts=tight_opts(oracle_lib))
    assert fails == 0
    assert np.abs(r["xyz"] - xyz).max() < 1e-8
    assert np.abs(r["vel"] - vel).max() < 1e-10
    assert np.abs(r["energy"] - epot).max() < 1e-7
    # leapfrog + CN + one kernel per shell-pair class (integrals, gradient) + SCC + reset + assembly
    assert b.kernel_launches() % nsteps == 0 and b.kernel_launches() >= nsteps * 7


def test_nve_energy_conservation(gpu):
    # leapfrog kinetic energy of step k belongs to the geometry of step k-1
    Z, xyz = molgen.c6h12o2()
    vel = molgen.maxwell_boltzmann(Z, 500.0, 1234)
    b = qg.Batch([{"Z": Z, "xyz": xyz, "vel": vel, "mass": molgen.masses(Z), "charge": 1}])
    b.egrad()
    epot = [b.get()["energy"][0]]
    etot = []
    for _ in range(40):
        b.step(1, 0.2 * constants.FSTOAU)
        r = b.get()
        assert r["status"][0] == 0
        etot.append(epot[-1] + r["ekin"][0])
        epot.append(r["energy"][0])
    assert max(etot) - min(etot) < 5e-3


def test_failed_trajectory_is_masked(gpu):
    # an SCC capped at 2 iterations cannot converge: the trajectory stops,
    # the others keep going, and new coordinates restart it
    mols = [molecules.c6h12o2(), molecules.h2o_cation()]
    b = _batch(mols)
    b.egrad()
    b.set_scc(2, 1e-7, 1e-6, 0.25)
    b.egrad()
    active, steps = b.progress()
    assert list(active) == [0, 0] and list(steps) == [1, 1]
    b.set_scc(100, 1e-7, 1e-6, 0.25)
    b.step(3, 0.5 * constants.FSTOAU)
    active, steps = b.progress()
    assert list(steps) == [1, 1]
    b.set_state(xyz=np.concatenate([m[1] for m in mols]))
    b.egrad()
    active, steps = b.progress()
    assert list(active) == [1, 1] and list(steps) == [2, 2]


@pytest.mark.parametrize("name", ["h2o+", "ch2o+", "h2s-ch+", "h2o+ar"])
def test_mixed_precision_small(gpu, oracle_lib, name):
    # mixed path tolerance: 1e-6 Eh energy, 1e-5 Eh/Bohr gradient against the FP64 oracle
    Z, xyz, c = molecules.ALL_SMALL[name]()
    b = _batch([(Z, xyz, c)])
    b.set_precision("mixed")
    b.egrad()
    r = b.get()
    rc, e, g, q, info = oracle_lib.egrad(Z, xyz, c, kT=KT)
    assert r["status"][0] == 0
    assert abs(r["energy"][0] - e) < 1e-6
    assert np.abs(r["grad"] - g).max() < 1e-5


def test_mixed_precision_batch(gpu, oracle_lib):
    mols = [molecules.c6h12o2()] + [molecules.random_chno(n, 300 + n) for n in (8, 17, 26, 35, 40)]
    b = _batch(mols)
    b.set_precision("mixed")
    b.egrad()
    r = b.get()
    g = b.split(r["grad"])
    both = 0
    for i, (Z, xyz, c) in enumerate(mols):
        rc, e, gref, q, info = oracle_lib.egrad(Z, xyz, c, kT=KT)
        if rc != 0:
            continue  # no converged reference (the 40-atom cation does not converge in 100 iterations)
        assert r["status"][i] == 0, i
        both += 1
        assert abs(r["energy"][i] - e) < 1e-6, (i, r["energy"][i] - e)
        assert np.abs(g[i] - gref).max() < 1e-5
    assert both >= 5


def test_mixed_md_matches_fp64(gpu):
    # 8 trajectories: an SCC that does not converge within the iteration limit
    # stops a trajectory in one of the two runs now and then (hot random cations),
    # so the test compares the ones that ran through in both
    mols = []
    for s, n in enumerate([9, 14, 21, 26, 33, 12, 17, 28]):
        Z, xyz = molgen.random_chno(n, 400 + s)
        mols.append({"Z": Z, "xyz": xyz, "vel": molgen.maxwell_boltzmann(Z, 1000.0, s), "mass": molgen.masses(Z),
                     "charge": 1})
    out = {}
    for prec in ("fp64", "mixed"):
        b = qg.Batch(mols)
        b.set_precision(prec)
        b.egrad()
        b.step(20, 0.5 * constants.FSTOAU)
        out[prec] = b.get()
    ok = (out["fp64"]["status"] == 0) & (out["mixed"]["status"] == 0)
    assert ok.sum() >= 2
    # After 20 steps the two runs sit at slightly different geometries: at the
    # default SCC thresholds their gradients differ by up to ~2e-6 Eh/Bohr, which
    # moves an H atom by ~0.5 (2e-6 / 1836) (20 * 20.7)^2 ~ 1e-4 Bohr, worth a
    # few 1e-6 Eh at gradients of 0.05 Eh/Bohr. The single-point contract (1e-6 Eh)
    # is tested at identical geometries elsewhere; here the trajectories stay
    # within that propagated bound.
    assert np.abs(out["fp64"]["energy"] - out["mixed"]["energy"])[ok].max() < 5e-6
    xa = qg_split(out["fp64"]["xyz"], mols)
    xb = qg_split(out["mixed"]["xyz"], mols)
    for i in np.nonzero(ok)[0]:
        assert np.abs(xa[i] - xb[i]).max() < 1e-4


def qg_split(arr, mols):
    out, o = [], 0
    for m in mols:
        out.append(arr[o:o + len(m["Z"])])
        o += len(m["Z"])
    return out

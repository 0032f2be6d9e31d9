"""Stop rules of the collision MD (src/cid.f90:739-1052) on the device.

CPU: the oracle restatement on a constructed approach-and-recoil sequence of
the gas atom with a known collision step, the fragmentation rule and a failed
call. GPU: the device rules inside the step graph against the oracle fed with
the same per-step coordinates, velocities and ion fragment counts, bit for
bit, over 160 steps of 6 collision trajectories (at least one collides)."""
import numpy as np
import pytest

import qcxms_gb300 as qg
from qcxms_gb300 import constants, molgen

DT = 0.5 * constants.FSTOAU


def _approach(o, nfrag_after=1, fail_at=None, nsteps=200):
    """Three ion atoms at rest and a gas atom moving in along x, turning at
    step 50 and moving out; unit masses except the gas atom."""
    mass = [1.0, 1.0, 1.0, 40.0]
    vel = [[0.0] * 3] * 4

    def xyz(k):
        gx = 20.0 - 0.3 * k if k <= 50 else 5.0 + 0.3 * (k - 50)
        return [[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [gx, 0.0, 0.0]]

    s = o.cid_rules_begin(xyz(0), mass, 100000)
    for k in range(1, nsteps + 1):
        nf = nfrag_after if (s["collided"] and k > 0) else 1
        o.cid_rules_step(s, fail_at == k, xyz(k), vel, mass, nf, DT, 300.0)
        if s["done"]:
            return s, k
    return s, nsteps


def test_oracle_collision_known_answers(oracle_lib):
    o = oracle_lib
    s, k = _approach(o)
    # distance checks every 10 steps; the minimum is seen at step 50, the
    # distance grows at steps 60, 70, 80, 90, 100: collision marked at step 100,
    # the run then ends 800 * (2 * 0.5 fs) = 800 steps later
    assert s["collided"] and not s["done"] and s["total_steps"] == 100 + 800
    assert s["nstep"] == 200 and s["m"] == 100  # the temperature mean restarts at the collision
    # the ion falls apart after the collision: the end moves to add_steps (0 for 3 atoms) later
    s, k = _approach(o, nfrag_after=2)
    assert s["done"] and s["fragmented"] and k == 101 and not s["failed"]
    # a failed energy call ends the run
    s, k = _approach(o, fail_at=30)
    assert s["done"] and s["failed"] and k == 30
    # the first step's temperature is tinit; collision energy of an ion at rest is 0
    s = o.cid_rules_begin([[0, 0, 0], [1, 0, 0], [5, 0, 0]], [1.0, 1.0, 40.0], 10)
    o.cid_rules_step(s, False, [[0, 0, 0], [1, 0, 0], [5, 0, 0]], [[0.0] * 3] * 3, [1.0, 1.0, 40.0], 1, DT, 450.0)
    assert s["avgT"] == 450.0 and s["ecom"] == 0.0


def test_gas_atom_mass_is_the_reference_literal(oracle_lib):
    """gas%mIatom = 39.948 * amutoau (src/input.f90:531): a default-real literal
    (single precision, promoted for the product) times amutoau = amutokg *
    (1/metokg) (src/xtb_mctc_convert.f90:47-51). The workload places it at
    mass0(nuc0) (src/cid.f90:657) and the collision rules take beta =
    m_gas / (m_gas + summass) from it, summass summed in atom order
    (src/cid.f90:342-347). All bit for bit."""
    amutoau = 1.660539040e-27 * (1.0 / 9.10938356e-31)
    m_ar = float(np.float32(39.948)) * amutoau
    assert float(np.float32(39.948)) != 39.948  # the literal is not the double 39.948
    assert constants.gas_mass_au(18) == m_ar and m_ar != constants.MASS_AU[18]
    for m in molgen.cid_workload(5, 10, 14, seed0=31):
        assert m["Z"][-1] == 18 and m["mass"][-1] == m_ar
        summass = 0.0
        for x in m["mass"][:-1]:
            summass = summass + x
        s = oracle_lib.cid_rules_begin(m["xyz"], m["mass"], 100)
        assert s["summass"] == summass
        # two steps of an ion moving by 0.01 Bohr per step along x: the collision
        # energy is beta * E_velo in eV with beta = m_gas / (m_gas + summass)
        x0 = np.asarray(m["xyz"], dtype=np.float64)
        for k in (1, 2):
            xk = x0.copy()
            xk[:-1, 0] += 0.01 * k
            oracle_lib.cid_rules_step(s, False, xk, np.zeros_like(x0), m["mass"], 1, DT, 300.0)
        v = (0.01 / DT) / (1.0 / 2.18769126364e6) * (1.0 / 2.18769126364e6)
        e_velo = (0.5 * summass) * (v * v)
        assert abs(s["ecom"] - (m_ar / (m_ar + summass)) * e_velo * constants.AUTOEV) < 1e-12 * s["ecom"]


def test_oracle_averaged_structures_known_answers(oracle_lib):
    """src/cid.f90:743-746, 802-909, 1095-1101 on a constructed run: a 4-atom ion
    (gas atom approaching, so no collision) whose coordinates are known per step.
    Steps 1-60 one fragment: the window restarts after 50 loop tops, the result
    is the mean of steps 51-60. Steps 61-80 two fragments (2 + 2 atoms): the
    fragments' mean over 61-80. At step 81 a fragment changes its atom count
    (1 + 3): the count restarts, steps 82-131 fill it to cnt_steps = 50 and the
    average freezes; later steps (and the ion going back to one fragment)
    leave it."""
    o = oracle_lib
    mass = [1.0, 1.0, 1.0, 1.0, 40.0]
    vel = [[0.0] * 3] * 5
    rng = np.random.default_rng(3)
    base = rng.normal(size=(4, 3))

    def xyz(k):
        x = np.vstack([base + 0.01 * k * np.arange(1, 13).reshape(4, 3), [[60.0 - 0.01 * k, 0.0, 0.0]]])
        return x

    def labels(k):
        if k <= 60:
            return [1, 1, 1, 1], 1
        if k <= 80:
            return [1, 1, 2, 2], 2
        if k <= 140:
            return [1, 2, 2, 2], 2
        return [1, 1, 1, 1], 1

    s = o.cid_rules_begin(xyz(0), mass, 100000)
    for k in range(1, 61):
        lab, nf = labels(k)
        o.cid_rules_step(s, False, xyz(k), vel, mass, nf, DT, 300.0, frag=lab)
    want = sum(xyz(k)[:4] for k in range(51, 61)) / 10
    assert np.allclose(o.cid_avg_xyz(s), want, rtol=0, atol=1e-12)
    assert s["xyzavg_dump"] == 10 and s["check_fragmented"] == 1
    for k in range(61, 81):
        lab, nf = labels(k)
        o.cid_rules_step(s, False, xyz(k), vel, mass, nf, DT, 300.0, frag=lab)
    assert s["count_average"] == 1 and s["cnt"] == 20
    assert np.allclose(o.cid_avg_xyz(s), sum(xyz(k)[:4] for k in range(61, 81)) / 20, rtol=0, atol=1e-12)
    lab, nf = labels(81)
    o.cid_rules_step(s, False, xyz(81), vel, mass, nf, DT, 300.0, frag=lab)
    assert s["cnt"] == 0 and np.all(o.cid_avg_xyz(s) == 0.0)
    for k in range(82, 132):
        lab, nf = labels(k)
        o.cid_rules_step(s, False, xyz(k), vel, mass, nf, DT, 300.0, frag=lab)
    frozen = sum(xyz(k)[:4] for k in range(82, 132)) / 50
    assert s["count_average"] == 0 and s["cnt"] == 0
    assert np.allclose(o.cid_avg_xyz(s), frozen, rtol=0, atol=1e-12)
    for k in range(132, 160):
        lab, nf = labels(k)
        o.cid_rules_step(s, False, xyz(k), vel, mass, nf, DT, 300.0, frag=lab)
    assert s["check_fragmented"] == 2 and np.allclose(o.cid_avg_xyz(s), frozen, rtol=0, atol=1e-12)
    assert not s["done"] and not s["collided"]


@pytest.mark.gpu
def test_gpu_cid_rules_match_oracle(gpu, oracle_lib):
    o = oracle_lib
    mols = molgen.cid_workload(6, 10, 12, seed0=900, gap_aa=1.5)
    b = qg.Batch(mols)
    b.egrad()
    tinit, ntot, nsteps = 500.0, 100000, 160
    b.set_cid_rules(tinit, ntot)
    r = b.get()
    off = np.concatenate([[0], np.cumsum([len(m["Z"]) for m in mols])])
    ref = [o.cid_rules_begin(r["xyz"][off[i]:off[i + 1]], list(m["mass"]), ntot) for i, m in enumerate(mols)]
    # gradfail of egrad ends a collision run: a failed calculation or any checkqc rejection (src/cid.f90:763)
    fail = qg.STATUS_SCC_NOT_CONVERGED | qg.STATUS_NON_FINITE | qg.STATUS_CHOLESKY_FAILED | qg.STATUS_CHECKQC
    keys = ["nstep", "nfrag", "collided", "fragmented", "total_steps", "done", "failed"]
    for step in range(nsteps + 1):
        st = b.cid_state()
        for i in range(len(mols)):
            s = ref[i]
            for kk in keys:
                assert st[kk][i] == s[kk], (step, i, kk)
            assert st["avg_temp"][i] == s["avgT"] and st["ecom_ev"][i] == s["ecom"], (step, i)
        if step == nsteps or st["done"].all():
            break
        b.step(1, DT)
        r = b.get()
        for i, m in enumerate(mols):
            sl = slice(off[i], off[i + 1])
            lab, nf = o.fragments(m["Z"][:-1], r["xyz"][sl][:-1])
            o.cid_rules_step(ref[i], bool(r["status"][i] & fail), r["xyz"][sl], r["vel"][sl], list(m["mass"]), nf,
                             DT, tinit, frag=list(lab))
        if step % 20 == 19:
            ax = b.cid_avg_xyz()
            for i in range(len(mols)):
                sl = slice(off[i], off[i + 1] - 1)
                want = o.cid_avg_xyz(ref[i])
                assert np.array_equal(ax[sl], want), (step, i)
    # the set exercises the collision detection (how many collide within 160
    # steps depends on the trajectories' SCC paths; the CPU oracle's own runs
    # of the same set collide 5 times)
    assert sum(s["collided"] for s in ref) >= 1

"""MD bookkeeping and exit rules of an electron-impact fragmentation run
(src/md.f90:285-682, it > 0, isec = 1, no heating phase).

CPU: the oracle restatement on hand-built sequences with a known outcome for
every exit rule. GPU: the device rules inside the captured step graph against
the oracle fed with the same per-step energies, kinetic energies, velocities
and fragment numbers; integer state and every double bit for bit."""
import numpy as np
import pytest

import qcxms_gb300 as qg
from qcxms_gb300 import constants, molgen

DT = 0.5 * constants.FSTOAU


def _run(o, seq, nfragexit=2, more=3, max_steps=100000, epot0=-10.0):
    """Feed (epot, nfrag) pairs; eight atoms at rest, unit masses, the first
    nfrag - 1 atoms each a fragment of their own."""
    mass = [1.0] * 8
    vel = [[0.0, 0.0, 0.0]] * 8
    s = o.md_rules_begin(vel, mass, epot0)
    for k, (e, nf) in enumerate(seq):
        frag = list(range(1, nf)) + [nf] * (8 - nf + 1)
        o.md_rules_step(s, e, 0.0, vel, mass, frag, nf, DT, nfragexit, more, max_steps)
        if s["done"]:
            return s, k + 1
    return s, len(seq)


def test_oracle_exit_rules_known_answers(oracle_lib):
    o = oracle_lib
    # energy error above 0.1 Eh: exit, taken only with 2..4 fragments
    s, k = _run(o, [(-10.0, 1)] * 5 + [(-9.5, 1)])
    assert s["done"] and s["mdok"] == 0 and k == 6 and s["fragstate"] == 0
    s, k = _run(o, [(-10.0, 2)] * 2 + [(-9.5, 2)], nfragexit=3)
    assert s["done"] and s["mdok"] == 1 and k == 3
    # a failed energy call (Epot = 0) ends the run at the next loop top
    s, k = _run(o, [(-10.0, 1), (0.0, 1)])
    assert s["done"] and s["mdok"] == 0 and k == 2
    # nfragexit fragments: `more` further steps, then exit with fragstate 1
    s, k = _run(o, [(-10.0, 1)] * 3 + [(-10.0, 2)] * 10, nfragexit=2, more=3)
    assert s["done"] and s["mdok"] == 1 and s["fragstate"] == 1 and k == 3 + 4
    # back to one fragment resets the count one step later (src/md.f90:426)
    s, k = _run(o, [(-10.0, 2)] * 3 + [(-10.0, 1)] + [(-10.0, 2)] * 10, nfragexit=2, more=3)
    assert k == 4 + 4 and s["fragstate"] == 1
    # more than nfragexit fragments: immediate exit
    s, k = _run(o, [(-10.0, 1)] * 2 + [(-10.0, 3)], nfragexit=2)
    assert s["done"] and s["mdok"] == 1 and s["fragstate"] == 1 and k == 3
    # more than 6 fragments: an error, not taken
    s, k = _run(o, [(-10.0, 7)], nfragexit=10)
    assert s["done"] and s["mdok"] == 0 and k == 1
    # two fragments for more than 1000 steps: fragstate 2
    s, k = _run(o, [(-10.0, 2)] * 1100, nfragexit=3)
    assert s["done"] and s["fragstate"] == 2 and k == 1001
    # step limit
    s, k = _run(o, [(-10.0, 1)] * 50, max_steps=20)
    assert s["done"] and s["mdok"] == 1 and s["fragstate"] == 1 and s["nstep"] == 20 and k == 20
    # no start energy: no run at all
    s = o.md_rules_begin([[0.0] * 3], [1.0], 0.0)
    assert s["done"] and s["nstep"] == 0


def test_oracle_averaged_structure_window(oracle_lib):
    o = oracle_lib
    mass, vel = [1.0, 1.0], [[0.0] * 3] * 2
    pos = lambda k: [[float(k), 0.0, 0.0], [0.0, float(k), 0.0]]
    s = o.md_rules_begin(vel, mass, -1.0, xyz=pos(0))
    for k in range(1, 61):
        o.md_rules_step(s, -1.0, 0.0, vel, mass, [1, 1], 1, DT, 2, 250, 60, xyz=pos(k))
    # the run ends at the step limit (60 loop tops, positions 0..59); the window
    # restarted after 50 tops, so it holds positions 50..59
    assert s["done"] and s["kdump"] == 10 and o.md_avg_xyz(s)[0][0] == sum(range(50, 60)) / 10


def test_oracle_temperatures(oracle_lib):
    o = oracle_lib
    mass = [2.0, 3.0, 4.0]
    vel = [[0.1, 0.0, 0.0], [0.0, 0.2, 0.0], [0.0, 0.0, 0.3]]
    s = o.md_rules_begin(vel, mass, -5.0)
    ek = 0.5 * (2.0 * 0.01 + 3.0 * 0.04 + 4.0 * 0.09)
    assert s["nstep"] == 1 and abs(s["tav"] - ek / (1.5 * 3 * o.KB)) < 1e-9
    o.md_rules_step(s, -5.0, ek, vel, mass, [1, 2, 2], 2, DT, 3, 250, 100)
    # fragment 2 holds atoms 2 and 3: T = E_int / (1.5 * 2 * kB)
    e2 = 0.5 * 3.0 * 0.04 + 0.5 * 4.0 * 0.09
    assert abs(s["fragT"][1] - e2 / (1.5 * 2 * o.KB)) < 1e-9


def _kicked_batch():
    """Cations with their H atoms kicked outward (0.02 au, about 10 eV for H):
    some lose one H (2 fragments), some two (3), some none."""
    mols = []
    for k in range(12):
        Z, xyz = molgen.random_chno(6 + k % 5, 300 + k)
        Z = np.asarray(Z)
        xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
        vel = molgen.maxwell_boltzmann(Z, 300.0, 300 + k)
        hs = np.nonzero(Z == 1)[0]
        nkick = k % 3
        c = xyz.mean(0)
        for h in hs[:nkick]:
            d = xyz[h] - c
            vel[h] += 0.02 * d / np.linalg.norm(d)
        mols.append({"Z": Z, "xyz": xyz, "vel": vel, "mass": molgen.masses(Z), "charge": 1})
    return mols


@pytest.mark.gpu
def test_gpu_md_rules_match_oracle(gpu, oracle_lib):
    o = oracle_lib
    mols = _kicked_batch()
    b = qg.Batch(mols)
    b.egrad()
    r0 = b.get()
    nfragexit, more, max_steps = 2, 5, 40
    b.set_md_rules(nfragexit, more, max_steps)
    off = np.concatenate([[0], np.cumsum([len(m["Z"]) for m in mols])])
    fail = qg.STATUS_SCC_NOT_CONVERGED | qg.STATUS_NON_FINITE | qg.STATUS_CHOLESKY_FAILED
    ref = []
    for i, m in enumerate(mols):
        e = 0.0 if r0["status"][i] & fail else r0["energy"][i]
        ref.append(o.md_rules_begin(r0["vel"][off[i]:off[i + 1]], list(m["mass"]), e,
                                    xyz=r0["xyz"][off[i]:off[i + 1]]))
    for step in range(max_steps + 2):
        st = b.md_state()
        for i in range(len(mols)):
            s = ref[i]
            assert st["nstep"][i] == s["nstep"] and st["done"][i] == s["done"], (step, i)
            assert st["nfrag"][i] == s["nfrag"] and st["fragstate"][i] == s["fragstate"], (step, i)
            assert st["mdok"][i] == s["mdok"], (step, i)
            assert st["tav"][i] == s["tav"] and st["eerror"][i] == s["eerror"], (step, i)
            assert np.array_equal(st["fragT"][i], np.array(s["fragT"])), (step, i)
        if st["done"].all():
            break
        b.step(1, DT)
        r = b.get()
        frag, nf = b.fragments(3.0, 1, 0)
        for i, m in enumerate(mols):
            e = 0.0 if r["status"][i] & fail else r["energy"][i]
            o.md_rules_step(ref[i], e, r["ekin"][i], r["vel"][off[i]:off[i + 1]], list(m["mass"]),
                            list(frag[off[i]:off[i + 1]]), int(nf[i]), DT, nfragexit, more, max_steps,
                            xyz=r["xyz"][off[i]:off[i + 1]])
    st = b.md_state()
    assert st["done"].all()
    # the averaged structures (src/md.f90:352-362, 695), bit for bit
    axyz = b.md_avg_xyz()
    for i in range(len(mols)):
        if ref[i]["avxyz"] is not None:
            assert np.array_equal(axyz[off[i]:off[i + 1]], np.array(o.md_avg_xyz(ref[i]))), i
    # the set exercises the fragment exits and the step limit
    assert (st["nfrag"] >= 2).sum() >= 3 and (st["nstep"] == max_steps).sum() >= 1
    active, _ = b.progress()
    assert not active.any()


@pytest.mark.gpu
def test_new_md_rules_reach_the_captured_step_graphs(gpu):
    # the loop rules are kernel arguments of the step graphs: rules set again
    # after a step (a new step limit) apply from the next step, in whole-batch
    # and in grouped stepping
    mols = molgen.batch_workload(8, 6, 12, seed0=500)
    for grouped in (False, True):
        b = qg.Batch(mols)
        b.egrad()
        b.set_md_rules(2, 250, 100000)
        ngroup = len(b.group_info()[1])
        step = (lambda: b.step_groups(np.ones(ngroup, dtype=np.int32), DT)) if grouped else (lambda: b.step(1, DT))
        step()
        b.set_md_rules(2, 250, 3)
        for _ in range(5):
            step()
        st = b.md_state()
        active, _ = b.progress()
        # every run ended at the new limit at the latest (a failed evaluation
        # would have stopped its trajectory earlier)
        assert not active.any() and (st["nstep"] <= 3).all(), (grouped, st["nstep"], active)
        b.close()


def test_oracle_impactscale(oracle_lib):
    o = oracle_lib
    mass = [1837.0, 21874.0, 29166.0]
    vel = [[1e-3, 0.0, 0.0], [0.0, -2e-4, 1e-4], [1e-4, 1e-4, 0.0]]
    e0 = o._ekinet(vel, mass)
    v = [list(x) for x in vel]
    assert o.impactscale(v, mass, None, 0.1, 0.05, e0)
    e1 = o._ekinet(v, mass)
    # the target eimp * ff + e0 is reached to 0.001 Eh (plus at most one increment of 0.0002)
    assert e1 > e0 + 0.005 - 0.001 and e1 < e0 + 0.005 + 4.1e-4 * e1
    # heating weights: atoms with velof 0 keep their velocities
    v = [list(x) for x in vel]
    o.impactscale(v, mass, [1.0, 0.0, 1.0], 0.1, 0.05, e0)
    assert v[1] == vel[1] and v[0] != vel[0]
    assert o.md_heating(0.2, 10 * DT, DT)[2] == 10


@pytest.mark.gpu
def test_gpu_md_heating_match_oracle(gpu, oracle_lib):
    """Heating phase: velocities after every step (leapfrog restated by the
    oracle, then impactscale) and the rule state bit for bit."""
    o = oracle_lib
    mols = []
    for k in range(8):
        Z, xyz = molgen.random_chno(8 + k, 700 + k)
        Z = np.asarray(Z)
        mols.append({"Z": Z, "xyz": np.asarray(xyz, dtype=np.float64).reshape(-1, 3),
                     "vel": molgen.maxwell_boltzmann(Z, 500.0, 700 + k), "mass": molgen.masses(Z), "charge": 1})
    b = qg.Batch(mols)
    b.egrad()
    rng = np.random.default_rng(5)
    eimp = rng.uniform(0.05, 0.3, len(mols))
    tadd = np.array([(8 + k) * DT for k in range(len(mols))])
    velof = rng.uniform(0.5, 2.0, b.natom)
    b.set_md_heating(eimp, tadd, DT, velof)
    nfragexit, more, max_steps = 3, 20, 25
    b.set_md_rules(nfragexit, more, max_steps)
    off = np.concatenate([[0], np.cumsum([len(m["Z"]) for m in mols])])
    fail = qg.STATUS_SCC_NOT_CONVERGED | qg.STATUS_NON_FINITE | qg.STATUS_CHOLESKY_FAILED
    r = b.get()
    ref = []
    for i, m in enumerate(mols):
        e = 0.0 if r["status"][i] & fail else r["energy"][i]
        ref.append(o.md_rules_begin(r["vel"][off[i]:off[i + 1]], list(m["mass"]), e,
                                    o.md_heating(eimp[i], tadd[i], DT)))
    assert [s["nadd"] for s in ref] == list(range(8, 16))
    heated = 0
    for step in range(max_steps + 1):
        st = b.md_state()
        for i in range(len(mols)):
            s = ref[i]
            assert st["nstep"][i] == s["nstep"] and st["done"][i] == s["done"], (step, i)
            assert st["tav"][i] == s["tav"] and st["eerror"][i] == s["eerror"], (step, i)
            assert np.array_equal(st["fragT"][i], np.array(s["fragT"])), (step, i)
        if st["done"].all():
            break
        prev = r
        b.step(1, DT)
        r = b.get()
        frag, nf = b.fragments(3.0, 1, 0)
        for i, m in enumerate(mols):
            if ref[i]["done"]:
                continue
            sl = slice(off[i], off[i + 1])
            _, vpre, _ = o.leapfrog(prev["grad"][sl], m["mass"], DT, prev["xyz"][sl], prev["vel"][sl])
            vpre = [list(x) for x in vpre]
            scaled = ref[i]["nstep"] <= ref[i]["nadd"] and ref[i]["nfrag"] == 1
            e = 0.0 if r["status"][i] & fail else r["energy"][i]
            o.md_rules_step(ref[i], e, r["ekin"][i], vpre, list(m["mass"]), list(frag[sl]), int(nf[i]), DT,
                            nfragexit, more, max_steps, velof=list(velof[sl]))
            assert np.array_equal(np.array(vpre), r["vel"][sl]), (step, i)
            heated += scaled
    assert heated >= 8 * 8


def test_oracle_setetemp_known_answers(oracle_lib):
    o = oracle_lib
    assert o.setetemp(1, 0.2, 0.0, 0.0) == 5000.0
    assert o.setetemp(1, 0.2, 0.05, 20000.0) == 5000.0 + 1000.0 + 0.2 * 20000.0
    assert o.setetemp(2, 0.2, 0.05, 20000.0) == 6000.0  # fragmented: no IEE term
    assert o.setetemp(1, -0.1, 0.05, 20000.0) == 6000.0
    # along the heating: dum = eimp - eimp*nstep/nadd falls to 0 at nstep = nadd
    v = [[0.02, 0.0, 0.0]]
    s = o.md_rules_begin(v, [1837.0], -1.0, heat=(0.3, 0.05, 10), etemp=(0.0, 10000.0))
    assert s["etemp"] == 5000.0 + 0.3 * 10000.0
    temps = []
    for k in range(12):
        o.md_rules_step(s, -1.0, o._ekinet(v, [1837.0]), v, [1837.0], [1], 1, DT, 3, 250, 1000, etemp=(0.0, 10000.0))
        assert not s["done"]
        temps.append(s["etemp"])
    assert temps[0] == 5000.0 + (0.3 - 0.3 * 1.0 / 10.0) * 10000.0
    assert temps[9] == 5000.0 and temps[11] == 5000.0  # nstep >= nadd: dum <= 0


@pytest.mark.gpu
def test_gpu_md_etemp_match_oracle(gpu, oracle_lib):
    """Per-step electronic temperature (setetemp after every step): the device
    value equals the oracle's bit for bit after every step, and every
    evaluation runs at the temperature set after the previous step (energies
    against the oracle at that kT)."""
    o = oracle_lib
    mols = []
    for k in range(4):
        Z, xyz = molgen.random_chno(6 + 2 * k, 800 + k)
        Z = np.asarray(Z)
        mols.append({"Z": Z, "xyz": np.asarray(xyz, dtype=np.float64).reshape(-1, 3),
                     "vel": molgen.maxwell_boltzmann(Z, 500.0, 800 + k), "mass": molgen.masses(Z), "charge": 1})
    b = qg.Batch(mols)
    eimp = np.array([0.1, 0.2, 0.25, 0.3])
    tadd = np.array([6 * DT, 8 * DT, 10 * DT, 12 * DT])
    ax, ieet = 0.05, 20000.0
    b.set_md_heating(eimp, tadd, DT)
    b.set_md_etemp(ax, ieet)
    b.egrad()
    r = b.get()
    off = np.concatenate([[0], np.cumsum([len(m["Z"]) for m in mols])])
    # the start's evaluation ran at setetemp(1, eimp)
    for i, m in enumerate(mols):
        sl = slice(off[i], off[i + 1])
        et0 = o.setetemp(1, eimp[i], ax, ieet)
        rc, e, g, q, info = o.egrad(m["Z"], r["xyz"][sl], 1, kT=et0 * constants.KB_AU)
        assert rc == 0 and abs(r["energy"][i] - e) < 1e-7, i
    nfragexit, more, max_steps = 3, 20, 14
    b.set_md_rules(nfragexit, more, max_steps)
    fail = qg.STATUS_SCC_NOT_CONVERGED | qg.STATUS_NON_FINITE | qg.STATUS_CHOLESKY_FAILED
    ref = [o.md_rules_begin(r["vel"][off[i]:off[i + 1]], list(m["mass"]),
                            0.0 if r["status"][i] & fail else r["energy"][i], o.md_heating(eimp[i], tadd[i], DT),
                            etemp=(ax, ieet)) for i, m in enumerate(mols)]
    et = b.md_etemp()
    assert all(et[i] == ref[i]["etemp"] for i in range(len(mols)))
    for step in range(max_steps):
        if all(s["done"] for s in ref):
            break
        prev, et_prev = r, b.md_etemp()
        b.step(1, DT)
        r = b.get()
        frag, nf = b.fragments(3.0, 1, 0)
        for i, m in enumerate(mols):
            if ref[i]["done"]:
                continue
            sl = slice(off[i], off[i + 1])
            if step in (0, 5) and not r["status"][i] & fail:
                rc, e, g, q, info = o.egrad(m["Z"], r["xyz"][sl], 1, kT=et_prev[i] * constants.KB_AU)
                assert rc != 0 or abs(r["energy"][i] - e) < 1e-7, (step, i)
            _, vpre, _ = o.leapfrog(prev["grad"][sl], m["mass"], DT, prev["xyz"][sl], prev["vel"][sl])
            vpre = [list(x) for x in vpre]
            e = 0.0 if r["status"][i] & fail else r["energy"][i]
            o.md_rules_step(ref[i], e, r["ekin"][i], vpre, list(m["mass"]), list(frag[sl]), int(nf[i]), DT,
                            nfragexit, more, max_steps, etemp=(ax, ieet))
        et = b.md_etemp()
        for i in range(len(mols)):
            if not ref[i]["done"]:
                assert et[i] == ref[i]["etemp"], (step, i, et[i], ref[i]["etemp"])

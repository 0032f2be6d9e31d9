"""checkqc (src/iniqm.f90:684-732) on the product path.

egrad puts every GFN2 result through checkqc (src/iniqm.f90:650): |E| < 1e-8,
a gradient norm outside [1e-8, 20] (gnorm sums grad(1,i)**2 + grad(2,i)**2 +
grad(2,i)**2, no z term, src/iniqm.f90:727), or a cation whose largest atomic
charge is below 1e-5 in magnitude reject the result; the last two set E = 0,
which ends the MD run at its next loop top (src/md.f90:317).

CPU: the oracle's restatement against hand-made cases with known outcomes.
GPU: the device function (through qcx_checkqc) against the oracle bit for bit
on constructed arrays that trip every branch, and the batch path on a
close-contact cation (gradient norm 27 Eh/Bohr) next to a normal one.
"""
import numpy as np
import pytest

from qcxms_gb300 import constants

KT = 300.0 * constants.KB_AU


def _close_contact_ch4(d):
    """CH4+ with one H at distance d (Bohr) from C."""
    Z = np.array([6, 1, 1, 1, 1], dtype=np.int32)
    x = np.array([[0, 0, 0], [1.2, 1.2, 1.2], [-1.2, -1.2, 1.2], [-1.2, 1.2, -1.2], [1.2, -1.2, -1.2]], float)
    x[1] = x[1] / np.linalg.norm(x[1]) * d
    return Z, x


def _cases():
    """(energy, grad, qat, charge, expected code) covering every branch and its edges."""
    rng = np.random.default_rng(5)
    g = rng.normal(scale=0.05, size=(6, 3))
    q = np.array([0.3, 0.2, 0.1, 0.2, 0.1, 0.1])
    out = [(-10.0, g, q, 1, 0), (-10.0, g, q, 0, 0),
           (5e-9, g, q, 1, 1), (-9.99e-9, g, q, 1, 1), (1e-8, g, q, 1, 0)]
    # gradient norm: huge z only is accepted (the norm has no z term)
    gz = np.zeros((6, 3)); gz[:, 2] = 100.0
    out.append((-10.0, gz, q, 1, 2))  # x, y zero: norm 0 < 1e-8
    gzx = gz.copy(); gzx[0, 0] = 0.1
    out.append((-10.0, gzx, q, 1, 0))
    # norm around 20: sqrt(x^2 + 2 y^2) on one atom
    for x in (19.999999, 20.0, 20.000001):
        gg = np.zeros((2, 3)); gg[0, 0] = x
        out.append((-3.0, gg, np.array([0.5, 0.5]), 1, 2 if x > 20.0 else 0))
    gy = np.zeros((2, 3)); gy[1, 1] = 20.0 / np.sqrt(2.0)  # y counted twice: norm 20 up to rounding
    out.append((-3.0, gy, np.array([0.5, 0.5]), 1, None))
    # tiny but nonzero norm
    gt = np.zeros((3, 3)); gt[2, 0] = 5e-9
    out.append((-3.0, gt, np.array([0.4, 0.3, 0.3]), 1, 2))
    # charges of a cation: largest below 1e-5 in magnitude; neutral systems skip the test
    qz = np.array([-0.2, 9e-6, -0.1, -0.3, 0.0, -0.4])
    out += [(-10.0, g, qz, 1, 3), (-10.0, g, qz, 0, 0), (-10.0, g, qz, -1, 0),
            (-10.0, g, np.array([-0.2, 1.1e-5, -0.1, -0.3, 0.0, -0.4]), 1, 0),
            (-10.0, g, -np.abs(q), 2, 0)]
    return out


def test_oracle_checkqc_known_answers(oracle_lib):
    for e, g, q, c, want in _cases():
        ok, e2 = oracle_lib.checkqc(e, g, q, c)
        if want is None:
            continue
        assert ok == (want == 0), (e, c, want)
        assert e2 == (0.0 if want in (2, 3) else e)
    # gnorm: grad(2,i) twice, no z
    g = np.array([[1.0, 2.0, 3.0], [0.5, 0.25, 7.0]])
    assert oracle_lib.gnorm(g) == np.sqrt(((0 + 1.0 + 4.0) + 4.0 + 0.25 + 0.0625) + 0.0625)


def test_oracle_rejects_close_contact(oracle_lib):
    Z, x = _close_contact_ch4(0.5)
    rc, e, g, q, info = oracle_lib.egrad(Z, x, 1, kT=KT)
    assert rc == 0 and oracle_lib.gnorm(g) > 20.0
    assert oracle_lib.checkqc(e, g, q, 1) == (False, 0.0)
    Z, x = _close_contact_ch4(1.0)
    rc, e, g, q, info = oracle_lib.egrad(Z, x, 1, kT=KT)
    assert rc == 0 and oracle_lib.checkqc(e, g, q, 1) == (True, e)


@pytest.mark.gpu
def test_device_checkqc_matches_oracle_bit_for_bit(gpu, oracle_lib):
    import qcxms_gb300 as qg
    rng = np.random.default_rng(17)
    cases = _cases()
    # random results around the thresholds
    for k in range(40):
        nat = int(rng.integers(1, 30))
        g = rng.normal(size=(nat, 3)) * 10.0 ** rng.uniform(-9, 1.5)
        q = rng.normal(size=nat) * 10.0 ** rng.uniform(-6, 0)
        e = float(rng.choice([-1.0, 1.0]) * 10.0 ** rng.uniform(-9, 1))
        cases.append((e, g, q, int(rng.integers(-1, 3)), None))
    codes = set()
    for e, g, q, c, want in cases:
        code, e_dev = qg.checkqc(e, g, q, c)
        ok, e_ref = oracle_lib.checkqc(e, g, q, c)
        assert (code == 0) == ok, (e, c, code)
        assert np.float64(e_dev).tobytes() == np.float64(e_ref).tobytes()
        if want is not None:
            assert code == want, (e, c, code, want)
        codes.add(code)
    assert codes == {0, 1, 2, 3}


@pytest.mark.gpu
def test_batch_applies_checkqc(gpu, oracle_lib):
    """A close-contact cation (gnorm 27 Eh/Bohr) is rejected with E = 0 and
    stops; a normal cation next to it is accepted; the decision and the energy
    equal the oracle's checkqc applied to the device's own result."""
    import qcxms_gb300 as qg
    from qcxms_gb300 import molgen
    Zc, xc = _close_contact_ch4(0.5)
    Zn, xn = _close_contact_ch4(1.6)
    Z6, x6 = molgen.c6h12o2()
    mols = [{"Z": Zc, "xyz": xc, "charge": 1}, {"Z": Zn, "xyz": xn, "charge": 1}, {"Z": Z6, "xyz": x6, "charge": 1}]
    b = qg.Batch(mols)
    b.egrad()
    r = b.get()
    active, steps = b.progress()
    assert r["status"][0] == constants_status_checkqc()
    assert r["energy"][0] == 0.0 and active[0] == 0 and steps[0] == 0
    for i in (1, 2):
        assert r["status"][i] == 0 and active[i] == 1 and steps[i] == 1
    # the same decision from the oracle's restatement on the device's outputs
    for i, sl in enumerate(b.split(np.arange(b.natom))):
        g, q = r["grad"][sl], r["qat"][sl]
        terms = b.energy_terms(i)
        ok, e_ref = oracle_lib.checkqc(terms["total"] if i else _unrejected_energy(b, 0), g, q, 1)
        assert ok == (i != 0)
        assert e_ref == r["energy"][i]
    # the single-structure drop-in reports the rejection as a failure with E = 0
    q_, e_, g_, stat = qg.get_xtb_egrad(Zc, xc, 1, 2)
    assert stat == -1 and e_ == 0.0
    q_, e_, g_, stat = qg.get_xtb_egrad(Zn, xn, 1, 2)
    assert stat == 0 and abs(e_ - r["energy"][1]) < 1e-9
    b.close()


def _unrejected_energy(b, i):
    """Electronic energy plus the three-body and repulsion terms of molecule i:
    the total before checkqc zeroed it."""
    t = b.energy_terms(i)
    return (t["band"] + t["ies"] + t["e3"] + t["aes"] + t["axc"] + t["disp"] + t["ts"]) + (t["atm"] + t["rep"])


def constants_status_checkqc():
    return 16  # QCX_STATUS_CHECKQC in include/qcxgpu.h

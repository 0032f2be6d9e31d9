"""Ensemble start files (TMPQCXMS/TMP.n/start.xyz and qcxms.start, written by
wrstart, src/utility.f90:321-373, read by rdstart, src/utility.f90:379-422).

CPU: the library's readers against an independent parse of the fixture in
tests/golden/TMPQCXMS (made by tests/golden/make_start_files.py in wrstart's
layout): every value exact. GPU: the loaded ensemble drives a batch with the
device heating and exit rules."""
import os

import numpy as np
import pytest

import qcxms_gb300 as qg
from qcxms_gb300 import constants

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "TMPQCXMS")


def _fortran_reals(line, width=22):
    return [float(line[i:i + width].replace("D", "E")) for i in range(0, len(line.rstrip("\n")), width)]


def test_read_ensemble_matches_files():
    mols = qg.read_ensemble(GOLDEN)
    assert [m["itrj"] for m in mols] == [1, 2, 10]
    for m in mols:
        d = os.path.join(GOLDEN, "TMP.%d" % m["itrj"])
        lines = open(os.path.join(d, "qcxms.start")).read().splitlines()
        assert int(lines[0]) == m["itrj"]
        assert m["eimp"] == _fortran_reals(lines[1])[0] and m["tadd"] == _fortran_reals(lines[2])[0]
        for a in range(len(m["Z"])):
            v = _fortran_reals(lines[3 + a])
            assert list(m["vel"][a]) == v[:3] and m["velof"][a] == v[3]
        xl = open(os.path.join(d, "start.xyz")).read().splitlines()
        assert int(xl[0]) == len(m["Z"])
        for a in range(len(m["Z"])):
            t = xl[2 + a].split()
            assert constants.SYMBOLS[m["Z"][a]] == t[0]
            assert list(m["xyz"][a]) == [float(x) * (1.0 / 0.52917726) for x in t[1:4]]
        assert np.array_equal(m["mass"], [constants.MASS_AU[z] for z in m["Z"]])


def test_write_start_reproduces_the_fixture(tmp_path):
    """qcx_write_start (C) and the fixture generator (Python) restate wrstart's
    D22.14 output independently: byte-identical files."""
    lib = qg.load_library()
    for m in qg.read_ensemble(GOLDEN):
        out = tmp_path / ("start.%d" % m["itrj"])
        vel = np.ascontiguousarray(m["vel"])
        velof = np.ascontiguousarray(m["velof"])
        assert lib.qcx_write_start(str(out).encode(), m["itrj"], len(m["Z"]), m["eimp"], m["tadd"], qg._dp(vel),
                                   qg._dp(velof)) == 0
        ref = open(os.path.join(GOLDEN, "TMP.%d" % m["itrj"], "qcxms.start")).read()
        assert out.read_text() == ref
    # zero, negative and large exponents
    out = tmp_path / "edge"
    vel = np.array([[0.0, -1.5e-12, 123456.789]])
    assert lib.qcx_write_start(str(out).encode(), 7, 1, 1.0, 0.99999999999999999, qg._dp(vel),
                               qg._dp(np.array([2.5]))) == 0
    lines = out.read_text().splitlines()
    assert lines[0] == "   7" and lines[1] == "  0.10000000000000D+01" and lines[2] == "  0.10000000000000D+01"
    assert lines[3] == ("  0.00000000000000D+00 -0.15000000000000D-11  0.12345678900000D+06"
                        "  0.25000000000000D+01")


def test_readers_reject_bad_input(tmp_path):
    lib = qg.load_library()
    nat = np.zeros(1, dtype=np.int32)
    assert lib.qcx_read_xyz(str(tmp_path / "missing.xyz").encode(), 0, qg._ip(nat), None, None) == -1
    bad = tmp_path / "bad.xyz"
    bad.write_text("2\n\nC 0 0 0\nXx 1 0 0\n")
    Z, xyz = np.zeros(2, dtype=np.int32), np.zeros((2, 3))
    assert lib.qcx_read_xyz(str(bad).encode(), 2, qg._ip(nat), qg._ip(Z), qg._dp(xyz)) == -1
    assert b"bad atom line" in lib.qcx_last_error()
    # more atoms than the caller's arrays hold
    ok = tmp_path / "ok.xyz"
    ok.write_text("2\ncomment\nC 0 0 0\n6 1.5 0 0\n")
    assert lib.qcx_read_xyz(str(ok).encode(), 1, qg._ip(nat), qg._ip(Z), qg._dp(xyz)) == -1
    assert lib.qcx_read_xyz(str(ok).encode(), 2, qg._ip(nat), qg._ip(Z), qg._dp(xyz)) == 0
    assert list(Z) == [6, 6] and xyz[1, 0] == 1.5 / 0.52917726
    short = tmp_path / "qcxms.start"
    short.write_text("   1\n  0.10000000000000D+00\n")
    assert lib.qcx_read_start(str(short).encode(), 2, None, None, None, None, None) == -1


@pytest.mark.gpu
def test_gpu_ensemble_drives_batch(gpu):
    mols = qg.read_ensemble(GOLDEN)
    dt = 0.5 * constants.FSTOAU
    b = qg.Batch(mols)
    b.egrad()
    b.set_md_heating([m["eimp"] for m in mols], [m["tadd"] for m in mols], dt,
                     np.concatenate([m["velof"] for m in mols]))
    b.set_md_rules(2, 250, 1000)
    b.step(5, dt)
    st = b.md_state()
    active, _ = b.progress()
    # every trajectory still running has taken the 5 steps after the first loop top
    assert ((st["nstep"] == 6) | (st["done"] == 1)).all() and (st["nstep"][active > 0] == 6).all()
    assert active.sum() >= 2


@pytest.mark.gpu
def test_gpu_driver_runs_ensemble_to_the_end(gpu):
    from qcxms_gb300 import driver
    res = driver.run_ensemble(GOLDEN, etemp=300.0, max_steps=30, block=10)
    assert [t["itrj"] for t in res] == [1, 2, 10]
    for t in res:
        assert 1 <= t["nstep"] <= 30 and len(t["frag"]) > 0
        # trajectories that ended in fragments carry their IPs and qcxms.res lines
        assert ("fragip_eV" in t) == (2 <= t["nfrag"] <= 10)
        if "fragip_eV" in t:
            assert len(t["res_lines"]) == t["nfrag"]
            assert abs(sum(float(line[:10]) for line in t["res_lines"]) - 1.0) < 1e-6 or not t["ipok"]
    assert any(t["nstep"] == 30 and t["mdok"] for t in res)


# --- output files: qcxms.gs and qcxms.res lines ---------------------------------

def _fortran_d(x, w, d):
    """Fortran Dw.d restated with Python's decimal formatting (independent of the
    library's printf-based one): 0.<d digits>D<sign><2 digits>, right-justified."""
    if x == 0.0:
        s = "0." + "0" * d + "D+00"
    else:
        m = "%.*e" % (d - 1, abs(x))
        mant, ex = m.split("e")
        e = int(ex) + 1
        s = ("-" if x < 0 else "") + "0." + mant.replace(".", "") + ("D%+03d" % e if abs(e) <= 99 else "%+04d" % e)
    return s.rjust(w) if len(s) <= w else "*" * w


def test_gs_file_bytes(tmp_path):
    """qcxms.gs: list-directed nmax, then (6d16.8) lines per atom and record
    (src/md.f90:150-153, 379-385). Known answers written out by hand, then a
    random record against the Python restatement of D16.8."""
    p = tmp_path / "qcxms.gs"
    xyz = np.array([[[1.5, -0.000123456789, 0.0]]])
    vel = np.array([[[2.5e-4, -1.0, 123456.789]]])
    qg.write_gs(str(p), 4000, xyz, vel)
    lines = p.read_text().split("\n")
    assert lines[0] == "        4000"
    assert lines[1] == ("  0.15000000D+01 -0.12345679D-03  0.00000000D+00"
                        "  0.25000000D-03 -0.10000000D+01  0.12345679D+06")
    rng = np.random.default_rng(4)
    xyz = rng.normal(scale=5.0, size=(3, 7, 3))
    vel = rng.normal(scale=3e-4, size=(3, 7, 3))
    qg.write_gs(str(p), 2, xyz, vel)
    lines = p.read_text().split("\n")
    assert lines[0] == "           2" and len(lines) == 1 + 21 + 1 and lines[-1] == ""
    for r in range(3):
        for a in range(7):
            want = "".join(_fortran_d(v, 16, 8) for v in list(xyz[r, a]) + list(vel[r, a]))
            assert lines[1 + 7 * r + a] == want


def test_res_line_bytes():
    """qcxms.res lines, format (F10.7,i3,2i5,2i2,2x,i3,2x,20(i4,i3))
    (src/write_fragments.f90:392-447). Electron-impact records have no collision
    number, so their items take the edit descriptors one position earlier."""
    # EI: fragment 2 of trajectory 17 (isec 1), C2H4O1, assigned charge 0.75
    line = qg.format_res(0.75, 1, 17, 1, 2, [1, 6, 8], [4, 2, 1])
    assert line == " 0.7500000  1   17    1 2 3    1     4  6   2  8   1"
    # CID: collision 3 of trajectory 123, fragment 1, C6H5 with charge 1
    line = qg.format_res(1.0, 1, 123, 1, 1, [1, 6], [5, 6], icoll=3)
    assert line == " 1.0000000  1  123    3 1 1    2     1  5   6  6"
    # negative charges, a number too wide for its field
    line = qg.format_res(-0.4999999, -1, 123456, 2, 10, [7], [1])
    assert line == "-0.4999999 -1*****    210 1    7     1"


@pytest.mark.gpu
def test_gpu_gs_sampling_writes_qcxms_gs(gpu, tmp_path):
    """A ground-state sampling run writes qcxms.gs: nmax, then one record of
    (6d16.8) lines per loop top; the first record is the start geometry."""
    from qcxms_gb300 import driver, molgen
    Z, xyz = molgen.c6h12o2()
    vel = molgen.maxwell_boltzmann(Z, 300.0, 5)
    mols = [{"Z": Z, "xyz": xyz, "vel": vel, "mass": molgen.masses(Z), "charge": 0}]
    nrec = driver.gs_sampling(mols, 4, str(tmp_path / "gs.%d"))
    assert nrec == [4]
    lines = (tmp_path / "gs.0").read_text().split("\n")
    assert lines[0] == "           4" and len(lines) == 1 + 4 * len(Z) + 1
    first = lines[1].split()
    assert abs(float(first[0].replace("D", "E")) - xyz[0][0]) < 1e-7 * max(1.0, abs(xyz[0][0]))

"""MO spectrum path: get_xtb_egrad(spec_calc=.true.) -> write_qmo
(src/tblite.f90:153-166, src/mo_energ.f90:7-80).

write_qmo forms per orbital k and atom a the Mulliken population
sum_{j on a} sum_l C(j,k) C(l,k) S(j,l) + 1e-10 and normalises each orbital's
row over the atoms; getspec reads the list-directed file back
(readpopmo, src/mo_energ.f90:82-107).

CPU: the oracle's restatement against properties with known answers (a
symmetric dimer splits every orbital evenly; the occupation-weighted
populations give the SCC's Mulliken charges; ihomo), and the two files byte for
byte against expected text. GPU: the device populations against the oracle on
jittered molecules, the single-structure entry point, and its error cases.
"""
import os

import numpy as np
import pytest

import qcxms_gb300 as qg
from qcxms_gb300 import constants

KT = 300.0 * constants.KB_AU
TIGHT = dict(econv=1e-11, pconv=1e-9)
VALENCE = {1: 1, 6: 4, 7: 5, 8: 6, 16: 6}


def _jittered(seed, Z, xyz):
    rng = np.random.default_rng(seed)
    return np.array(Z), np.array(xyz, dtype=float) + rng.normal(scale=0.08, size=(len(Z), 3))


def _mols():
    from qcxms_gb300 import molgen
    out = []
    Z6, x6 = molgen.c6h12o2()
    out.append(_jittered(1, Z6, x6) + (1,))
    out.append(_jittered(2, [8, 1, 1], [[0, 0, 0], [0, 1.43, 1.11], [0, -1.43, 1.11]]) + (0,))
    out.append(_jittered(3, [7, 1, 1, 1], [[0, 0, 0], [1.9, 0, 0.6], [-0.95, 1.65, 0.6], [-0.95, -1.65, 0.6]]) + (1,))
    out.append(_jittered(4, [6, 6, 8, 1, 1, 1, 1, 1, 1],
                         [[0.0, 0.0, 0.0], [2.87, 0.0, 0.0], [3.77, 2.44, 0.0], [-0.69, 1.95, 0.0],
                          [-0.69, -0.98, 1.69], [-0.69, -0.98, -1.69], [3.56, -0.98, 1.69], [3.56, -0.98, -1.69],
                          [5.60, 2.44, 0.0]]) + (1,))
    return out


def test_oracle_symmetric_dimer_splits_evenly(oracle_lib):
    Z = np.array([1, 1])
    x = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 1.4]])
    rc, emo, focc, qmo, ihomo, info = oracle_lib.mo_spectrum(Z, x, 0, kT=KT)
    assert rc == 0 and ihomo == 1 and np.all(np.diff(emo) >= 0.0)
    assert np.abs(qmo - 0.5).max() < 1e-12
    assert abs(focc.sum() - 2.0) < 1e-12


def test_oracle_populations_give_the_mulliken_charges(oracle_lib):
    """sum_k focc_k qmo(k, a) = valence electrons - q_a: the orbital rows are
    normalised (C_k^T S C_k = 1 up to the 1e-10 shifts), so the
    occupation-weighted populations are the Mulliken populations."""
    for Z, x, c in _mols():
        o = oracle_lib.default_opts(**TIGHT)
        rc, emo, focc, qmo, ihomo, info = oracle_lib.mo_spectrum(Z, x, c, kT=KT, opts=o)
        assert rc == 0
        assert np.allclose(qmo.sum(axis=1), 1.0, atol=1e-14)
        rc2, e, g, q, _ = oracle_lib.egrad(Z, x, c, kT=KT, opts=o)
        pop = focc @ qmo
        val = np.array([VALENCE[z] for z in Z], dtype=float)
        assert np.abs(pop - (val - q)).max() < 1e-8
        nel = val.sum() - c
        assert ihomo == max(int(np.floor(nel / 2)), 1)
        assert info["nao"] == len(emo)


def test_write_qmo_files(tmp_path):
    emo = np.array([-0.5, -0.0018374, 0.25])  # Eh
    focc = np.array([2.0, 1.0, 0.0])
    qmo = np.array([[0.5, 0.25, 0.25] + [0.0] * 9,
                    [0.05] * 12,
                    [1.0 / 3.0] + [0.0] * 10 + [-1e-4]])
    t, m = tmp_path / "tmp.mspec", tmp_path / "qcxms.Mspec.tbxtb"
    qg.write_qmo(str(t), str(m), emo, focc, qmo, 2)
    ev = [x * 27.21138505 for x in emo]
    # qcxms.Mspec.tbxtb: list-directed integers, then (i3,1x,f10.3), (1x,f6.2), (10(1x,f6.2))
    want = ["           3           2", "",
            "  1 %10.3f" % ev[0], "   2.00",
            "  50.00  25.00  25.00   0.00   0.00   0.00   0.00   0.00   0.00   0.00", "   0.00   0.00", "",
            "  2 %10.3f" % ev[1], "   1.00",
            "   5.00" * 10, "   5.00   5.00", "",
            "  3 %10.3f" % ev[2], "   0.00",
            "  33.33" + "   0.00" * 9, "   0.00  -0.01"]
    assert m.read_text() == "\n".join(want) + "\n"
    assert "  1    -13.606" in want[2] and "  2     -0.050" in want[7]
    # tmp.mspec: one list-directed item per record, gfortran's layout
    lines = t.read_text().split("\n")
    assert lines[0] == "           3           2"
    assert lines[2] == "   2.0000000000000000     "
    assert lines[3] == "  0.50000000000000000     "
    assert lines[4] == "  0.25000000000000000     "
    assert lines[6] == "   0.0000000000000000     "
    assert lines[16] == "   1.0000000000000000     "
    assert lines[17] == "   5.0000000000000003E-002"
    assert lines[1] == "  -13.605692525000000     "
    assert lines[1 + 2 * 14 + 2] == "  0.33333333333333331     "
    assert lines[-2] == "  -1.0000000000000000E-004"
    # readpopmo reads the numbers back exactly
    vals = [float(v) for v in lines[1:-1]]
    k = 0
    for i in range(3):
        assert vals[k] == ev[i] and vals[k + 1] == focc[i]
        assert vals[k + 2:k + 14] == list(qmo[i])
        k += 14
    assert len(vals) == k


def test_write_qmo_rejects_bad_input(tmp_path):
    with pytest.raises(RuntimeError):
        qg.write_qmo(str(tmp_path / "t"), None, np.zeros(0), np.zeros(0), np.zeros((0, 2)), 1)


@pytest.mark.gpu
def test_gpu_mo_populations_match_oracle(gpu, oracle_lib):
    mols = _mols()
    b = qg.Batch([{"Z": Z, "xyz": x, "charge": c} for Z, x, c in mols])
    b.set_precision("fp64")
    b.set_scc(250, TIGHT["econv"], TIGHT["pconv"], 0.25)
    b.set_keep_mo(True)
    b.egrad()
    r = b.get()
    o = oracle_lib.default_opts(**TIGHT)
    for i, (Z, x, c) in enumerate(mols):
        assert r["status"][i] in (0, qg.STATUS_CHECKQC)
        emo, focc, qmo, ih = b.mo_populations(i)
        rc, emo_o, focc_o, qmo_o, ih_o, _ = oracle_lib.mo_spectrum(Z, x, c, kT=KT, opts=o)
        assert rc == 0 and ih == ih_o
        assert np.abs(emo - emo_o).max() < 1e-9
        assert np.abs(focc - focc_o).max() < 1e-8
        assert np.abs(qmo - qmo_o).max() < 1e-7, i
        assert np.allclose(qmo.sum(axis=1), 1.0, atol=1e-14)
    b.close()


@pytest.mark.gpu
def test_gpu_mo_spectrum_entry_point(gpu, oracle_lib, tmp_path):
    Z, x, c = _mols()[0]
    e, emo, focc, qmo, ih = qg.mo_spectrum(Z, x, c, 2, etemp=300.0)
    rc, emo_o, focc_o, qmo_o, ih_o, info = oracle_lib.mo_spectrum(Z, x, c, kT=KT)
    assert rc == 0 and ih == ih_o and len(emo) == info["nao"]
    # default SCC thresholds on both sides: agreement to where two SCC runs stop
    assert np.abs(emo - emo_o).max() < 1e-5 and np.abs(qmo - qmo_o).max() < 1e-4
    assert abs(e - oracle_lib.egrad(Z, x, c, kT=KT)[1]) < 1e-6
    # getspec's check on the levels (src/mo_spec.f90:110) holds
    assert (emo[ih - 1] - emo[0]) * 27.21138505 >= 1.0
    qg.write_qmo(str(tmp_path / "tmp.mspec"), str(tmp_path / "qcxms.Mspec.tbxtb"), emo, focc, qmo, ih)
    vals = [float(v) for v in (tmp_path / "tmp.mspec").read_text().split()]
    assert vals[0] == len(emo) and vals[1] == ih and vals[2] == emo[0] * 27.21138505
    # too small a buffer and an unknown method fail cleanly
    with pytest.raises(RuntimeError):
        qg.mo_spectrum(Z, x, c, 2, max_nao=10)
    with pytest.raises(RuntimeError):
        qg.mo_spectrum(Z, x, c, 2, method=qg.gfn1_xtb)
    # mixed precision keeps no orbitals
    b = qg.Batch([{"Z": Z, "xyz": x, "charge": c}])
    b.set_keep_mo(True)
    b.set_precision("mixed")
    b.egrad()
    with pytest.raises(RuntimeError):
        b.mo_populations(0)
    b.close()

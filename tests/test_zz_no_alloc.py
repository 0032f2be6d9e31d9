"""qcx_egrad_noalloc: the allocation-free energy + gradient entry point.

Callers that cannot allocate device memory (their process hands all GPU memory
to another runtime's capped pool, or must not pay the synchronisation an
allocation implies) use this variant; its scratch is a fixed static device
array. It must give the same results as qcx_egrad, the allocating entry point,
on consecutive calls (the static array keeps the previous call's contents, so
the second call checks that every piece of state that must start fresh does).

This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

import qcxms_gb300 as qg
from tests import molecules

pytestmark = pytest.mark.gpu


def _bind(lib):
    P = ctypes.POINTER
    f = lib.qcx_egrad_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_int, P(ctypes.c_int32), P(ctypes.c_double), ctypes.c_int, ctypes.c_int,
                  ctypes.c_double, P(ctypes.c_double), P(ctypes.c_double), P(ctypes.c_double)]
    return f


def _call(f, Z, xyz, charge, etemp=300.0):
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    e = np.zeros(1)
    g = np.zeros((len(Z), 3))
    q = np.zeros(len(Z))
    d = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    rc = f(2, len(Z), Z.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), d(xyz), int(charge), 2, float(etemp),
           d(e), d(g), d(q))
    return rc, e[0], g, q


def test_noalloc_matches_allocating_entry_point(gpu):
    f = _bind(gpu)
    Z, xyz, c = molecules.c6h12o2()
    cases = [(Z, xyz), (Z, xyz + 0.02), molecules.h2s_ch_cation()[:2]]
    for Zi, xi in cases:  # consecutive calls share the static scratch array
        rc, e, g, q = _call(f, Zi, xi, c)
        qr, er, gr, stat = qg.get_xtb_egrad(Zi, xi, c, 2, qg.gfn2_xtb, 300.0)
        assert rc == 0 and stat == 0
        assert abs(e - er) < 1e-8
        assert np.abs(g - gr).max() < 1e-7
        assert np.abs(q - qr).max() < 1e-7


def test_noalloc_near_its_size_limit_matches_oracle(gpu, oracle_lib):
    """A 60-atom cation with 159 atomic orbitals, next to the limit of 160: the
    largest static regions in use. Two calls in a row; both agree with the
    allocating entry point and with the CPU oracle (default SCC thresholds on
    every side: energies within 1e-7 Eh, gradients within 5e-6 Eh/Bohr, the
    spread of where two correct SCC runs stop; the atomic sums of the
    potentials make the GPU's own SCC path vary between calls)."""
    from qcxms_gb300 import constants, molgen
    f = _bind(gpu)
    Z, xyz = molgen.random_chno(60, 6)
    assert oracle_lib.nao(Z) == 159
    rc_o, e_o, g_o, q_o, info = oracle_lib.egrad(Z, xyz, 1, kT=300.0 * constants.KB_AU)
    assert rc_o == 0
    for k in range(2):
        rc, e, g, q = _call(f, Z, xyz, 1)
        qr, er, gr, stat = qg.get_xtb_egrad(Z, xyz, 1, 2, qg.gfn2_xtb, 300.0)
        assert rc == 0 and stat == 0, k
        assert abs(e - er) < 1e-8 and np.abs(g - gr).max() < 5e-6
        assert abs(e - e_o) < 1e-7 and np.abs(g - g_o).max() < 5e-6 and np.abs(q - q_o).max() < 1e-5


def test_noalloc_rejects_oversized_input(gpu, capfd):
    f = _bind(gpu)
    Z = np.array([6] * 70, dtype=np.int32)
    xyz = np.arange(210, dtype=np.float64).reshape(70, 3) * 3.0
    rc, e, g, q = _call(f, Z, xyz, 1)
    assert rc == -1
    assert "static scratch limit" in capfd.readouterr().err
    gpu.qcx_last_error.restype = ctypes.c_char_p
    assert b"static scratch limit" in gpu.qcx_last_error()

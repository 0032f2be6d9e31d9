"""CPU tests of the FP64 oracle: the checker the CUDA path is held against.

Parity with tblite is unpinned (no tblite, parameters or reference energies
ship with QCxMS); these tests pin the oracle against independent
restatements, known answers, symmetry and finite differences instead.
"""
import math

import numpy as np
import pytest

from qcxms_gb300 import basis, constants, molgen
from tests import molecules

TIGHT = dict(econv=1e-12, pconv=1e-10, max_iter=100)


# --------------------------------------------------------------------------
# independent numpy restatement of the one-electron integrals
# --------------------------------------------------------------------------
ALPHA = basis.read_param("qcx_prim_alpha")
COEFF = basis.read_param("qcx_prim_coeff")
NPRIM = basis.read_param("qcx_sh_nprim", int)
SHL = basis.read_param("qcx_sh_l", int)
NSH = basis.read_param("qcx_nsh", int)
CART = {0: [(0, 0, 0)], 1: [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
        2: [(2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)]}
s3 = 1.0 / math.sqrt(3.0)
SPH = {0: np.eye(1), 1: np.eye(3),
       2: np.array([[0, 0, 0, 1, 0, 0], [0, 0, 0, 0, 0, 1], [-s3 / 2, -s3 / 2, s3, 0, 0, 0],
                    [0, 0, 0, 0, 1, 0], [0.5, -0.5, 0, 0, 0, 0]])}


def _dfact(n):
    return 1.0 if n <= 0 else n * _dfact(n - 2)


def _ov1d(i, j, a, b, A, B):
    # binomial expansion about the Gaussian product centre
    p = a + b
    P = (a * A + b * B) / p
    pre = math.exp(-a * b / p * (A - B) ** 2)
    s = 0.0
    for k in range(i + 1):
        for l in range(j + 1):
            n = k + l
            if n % 2:
                continue
            mom = _dfact(n - 1) / (2 * p) ** (n // 2) * math.sqrt(math.pi / p)
            s += math.comb(i, k) * math.comb(j, l) * (P - A) ** (i - k) * (P - B) ** (j - l) * mom
    return pre * s


def _shell_block(za, ka, Ra, zb, kb, Rb, raise_bra=(0, 0, 0)):
    la, lb = SHL[za][ka], SHL[zb][kb]
    out = np.zeros((len(CART[la]), len(CART[lb])))
    for i in range(NPRIM[za][ka]):
        for j in range(NPRIM[zb][kb]):
            a, b = ALPHA[za][ka][i], ALPHA[zb][kb][j]
            na = (2 * a / math.pi) ** 0.75 * (4 * a) ** (la / 2)
            nb = (2 * b / math.pi) ** 0.75 * (4 * b) ** (lb / 2)
            c = COEFF[za][ka][i] * COEFF[zb][kb][j] * na * nb
            for ca, ea in enumerate(CART[la]):
                for cb, eb in enumerate(CART[lb]):
                    v = 1.0
                    for k in range(3):
                        v *= _ov1d(ea[k] + raise_bra[k], eb[k], a, b, Ra[k], Rb[k])
                    out[ca, cb] += c * v
    return SPH[la] @ out @ SPH[lb].T


def numpy_integrals(Z, xyz):
    shells = [(ia, k) for ia, z in enumerate(Z) for k in range(NSH[z])]
    offs, n = [], 0
    for ia, k in shells:
        offs.append(n)
        n += 2 * SHL[Z[ia]][k] + 1
    S = np.zeros((n, n)); D = np.zeros((3, n, n)); Q = np.zeros((6, n, n))
    qpow = [(2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)]
    for s, (ia, ka) in enumerate(shells):
        for t, (ib, kb) in enumerate(shells):
            za, zb = Z[ia], Z[ib]
            na, nb = 2 * SHL[za][ka] + 1, 2 * SHL[zb][kb] + 1
            sl = (slice(offs[s], offs[s] + na), slice(offs[t], offs[t] + nb))
            S[sl] = _shell_block(za, ka, xyz[ia], zb, kb, xyz[ib])
            for c in range(3):
                r = [0, 0, 0]; r[c] = 1
                D[(c,) + sl] = _shell_block(za, ka, xyz[ia], zb, kb, xyz[ib], tuple(r))
            M = [_shell_block(za, ka, xyz[ia], zb, kb, xyz[ib], qp) for qp in qpow]
            tr = M[0] + M[1] + M[2]
            for q in range(3):
                Q[(q,) + sl] = 1.5 * M[q] - 0.5 * tr
            for q in range(3, 6):
                Q[(q,) + sl] = 1.5 * M[q]
    return S, D, Q


@pytest.mark.parametrize("name", ["ch2o+", "h2s-ch+", "h2o+ar"])
def test_integrals_match_independent_restatement(oracle_lib, name):
    Z, xyz, _ = molecules.ALL_SMALL[name]()
    S, H0, Dm, Qm, cn, cnd = oracle_lib.integrals(Z, xyz)
    S2, D2, Q2 = numpy_integrals(list(Z), xyz)
    assert np.abs(S - S2).max() < 1e-12
    assert np.abs(Dm - D2).max() < 1e-12
    assert np.abs(Qm - Q2).max() < 1e-12


def test_onsite_blocks_orthonormal(oracle_lib):
    Z, xyz, _ = molecules.h2s_ch_cation()
    S = oracle_lib.integrals(Z, xyz)[0]
    o = 0
    for z in Z:
        n = basis.nao_of([z])
        assert np.allclose(S[o:o + n, o:o + n], np.eye(n), atol=1e-12)
        o += n


def test_syev_matches_numpy(oracle_lib):
    rng = np.random.default_rng(0)
    for n in (1, 2, 3, 7, 30, 61):
        A = rng.normal(size=(n, n)); A = A + A.T
        rc, w, V = oracle_lib.syev(A)
        assert rc == 0
        assert np.allclose(w, np.linalg.eigvalsh(A), atol=1e-11)
        assert np.allclose(V.T @ V, np.eye(n), atol=1e-11)
        assert np.allclose(A @ V, V * w, atol=1e-10)


@pytest.mark.parametrize("name", ["h2o+", "ch2o+", "h2s-ch+", "h2o+ar"])
def test_gradient_central_differences(oracle_lib, name):
    Z, xyz, charge = molecules.ALL_SMALL[name]()
    o = oracle_lib.default_opts(**TIGHT)
    rc, e, g, q, info = oracle_lib.egrad(Z, xyz, charge, opts=o)
    assert rc == 0
    h = 1e-4
    for a in range(len(Z)):
        for k in range(3):
            xp = xyz.copy(); xp[a, k] += h
            xm = xyz.copy(); xm[a, k] -= h
            fd = (oracle_lib.egrad(Z, xp, charge, opts=o)[1] - oracle_lib.egrad(Z, xm, charge, opts=o)[1]) / (2 * h)
            assert abs(fd - g[a, k]) < 1e-6, (a, k, fd, g[a, k])


def test_translation_rotation_invariance(oracle_lib):
    Z, xyz, charge = molecules.c6h12o2()
    o = oracle_lib.default_opts(**TIGHT)
    rc, e, g, q, _ = oracle_lib.egrad(Z, xyz, charge, opts=o)
    assert np.abs(g.sum(0)).max() < 1e-10
    th = 0.7
    R = np.array([[math.cos(th), -math.sin(th), 0], [math.sin(th), math.cos(th), 0], [0, 0, 1]])
    rc2, e2, g2, q2, _ = oracle_lib.egrad(Z, xyz @ R.T + np.array([1.0, -2.0, 0.5]), charge, opts=o)
    assert abs(e - e2) < 1e-8
    assert np.abs(g @ R.T - g2).max() < 1e-6
    assert abs(q.sum() - charge) < 1e-10


def test_scc_converges_on_random_cations(oracle_lib):
    for seed in range(8):
        Z, xyz = molgen.random_chno(5 + 4 * seed, seed)
        rc, e, g, q, info = oracle_lib.egrad(Z, xyz, 1)
        assert rc == 0 and info["converged"] == 1
        assert abs(q.sum() - 1.0) < 1e-8


def test_single_atom_and_one_electron(oracle_lib):
    Z, xyz, c = molecules.single_atom()
    rc, e, g, q, info = oracle_lib.egrad(Z, xyz, c)
    assert rc == 0 and np.all(g == 0) and abs(q[0] - 1.0) < 1e-10
    Z, xyz, c = molecules.h2_cation()
    rc, e, g, q, info = oracle_lib.egrad(Z, xyz, c)
    assert rc == 0 and info["nel"] == 1.0
    assert np.allclose(q, [0.5, 0.5], atol=1e-10)


def _leapfrog_reference(grad, mass, tstep, xyz, vel):
    # line-by-line restatement of src/md.f90:749-773
    xyz = xyz.copy(); vel = vel.copy(); ke = 0.0
    for k in range(len(mass)):
        m = mass[k]
        for j in range(3):
            vold = vel[k, j]
            vel[k, j] = vel[k, j] - (tstep * grad[k, j] / m)
            vavg = 0.5 * (vold + vel[k, j])
            xyz[k, j] = xyz[k, j] + (tstep * vel[k, j])
            ke = ke + 0.5 * (m * vavg * vavg)
    return xyz, vel, ke


def test_leapfrog_bit_exact(oracle_lib):
    rng = np.random.default_rng(3)
    Z, xyz = molgen.c6h12o2()
    vel = molgen.maxwell_boltzmann(Z, 500.0, 1)
    grad = rng.normal(scale=0.05, size=xyz.shape)
    m = molgen.masses(Z)
    t = 0.5 * constants.FSTOAU
    x1, v1, k1 = oracle_lib.leapfrog(grad, m, t, xyz, vel)
    x2, v2, k2 = _leapfrog_reference(grad, m, t, xyz, vel)
    assert np.array_equal(x1, x2) and np.array_equal(v1, v2) and k1 == k2


def test_getspin_gnorm_checkqc(oracle_lib):
    # src/utility.f90:449-464
    assert oracle_lib.getspin([6, 1, 1, 1, 1], 1) == 2
    assert oracle_lib.getspin([6, 1, 1, 1, 1], 0) == 1
    assert oracle_lib.getspin([1], 1) == -1
    # src/iniqm.f90:719-732 counts grad(2,i) twice and drops z
    g = np.array([[1.0, 2.0, 100.0]])
    assert abs(oracle_lib.gnorm(g) - math.sqrt(1 + 4 + 4)) < 1e-15
    ok, e = oracle_lib.checkqc(-10.0, np.array([[0.1, 0.0, 0.0]]), np.array([0.5]), 1)
    assert ok and e == -10.0
    ok, e = oracle_lib.checkqc(1e-9, np.array([[0.1, 0.0, 0.0]]), np.array([0.5]), 1)
    assert not ok
    ok, e = oracle_lib.checkqc(-10.0, np.array([[30.0, 0.0, 0.0]]), np.array([0.5]), 1)
    assert not ok and e == 0.0
    ok, e = oracle_lib.checkqc(-10.0, np.array([[0.1, 0.0, 0.0]]), np.array([1e-6]), 1)
    assert not ok and e == 0.0


def test_scc_mixer_restart_gets_sloshing_molecules_out(oracle_lib):
    # MD snapshots of hot cations of the 256-trajectory workload whose SCC slosh
    # between near-degenerate states. Without the restart of the Broyden history
    # after 12 stagnating iterations, molecule 215 after 20 steps stops at the
    # limit of 250 (checked with a build without the restart); with it both
    # converge.
    kT = 300.0 * constants.KB_AU
    dt = 0.5 * constants.FSTOAU
    mols = molgen.batch_workload(256, 5, 40)
    for i, ns in ((215, 20), (210, 27)):
        m = mols[i]
        rc, e, g, q = oracle_lib.egrad_batch([m], kT, nthreads=1)
        fails, xyz, vel, grad, ep, its = oracle_lib.md_batch([m], ns, dt, g, kT, nthreads=1)
        assert fails == 0
        r, e, g, q, info = oracle_lib.egrad(m["Z"], xyz, 1, kT=kT)
        assert r == 0 and info["converged"] == 1 and info["iterations"] < 200, (i, info["iterations"])

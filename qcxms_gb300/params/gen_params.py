"""Generate the synthetic GFN2-form parameter set ``synth-gfn2-v1``.

The GFN2-xTB parameter tables live in tblite v0.2.1 (a meson subproject that
QCxMS pulls in, ``subprojects/tblite.wrap``) and are not shipped with QCxMS.
This script therefore builds a *synthetic* parameter set with the same
functional form, from simple published physical rules:

* valence shells and reference occupations from the aufbau order;
* Slater exponents from Slater's screening rules (H set to 1.2);
* Slater functions expanded in Gaussians by a least-squares fit written here
  (STO-nG, ``NPRIM`` primitives per shell, fitted at zeta = 1, scaled by zeta^2);
* Pauling electronegativities and static atomic polarizabilities;
* the D3-style covalent radii (4/3 x Pyykkoe-Atsumi 2009) that QCxMS itself
  carries in ``src/covalent_radii.f90:27-50,84-86``;
* smooth period-wise formulas for self-energies, hardnesses, third-order,
  multipole and repulsion constants;
* the published GFN2-xTB D4 damping and scaling constants (s8 = 2.7,
  a1 = 0.52, a2 = 5.0, s9 = 5.0, charge scaling 3.0 / 2.0, weighting 6.0) --
  literature numbers, not fitted here. The D4 reference data itself comes from
  QCxMS (gen_d4_reference.py).

Any other parameter file with the same layout (for example one converted from
tblite's GFN2 tables) can be written in the same format and dropped in.

Output: ``qcxms_gb300/csrc/qcx_params.h`` (plain C arrays indexed by atomic
number, shared by the CUDA library and by the CPU oracle).
Run: ``python qcxms_gb300/params/gen_params.py``.
"""
import math
import os

import numpy as np
from scipy import integrate, optimize

MAXZ = 18
NPRIM = 6
AATOAU = 1.0 / 0.52917726  # src/xtb_mctc_convert.f90:24-25

SYM = ["", "H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne",
       "Na", "Mg", "Al", "Si", "P", "S", "Cl", "Ar"]
# Pyykkoe-Atsumi 2009 single-bond covalent radii (Angstrom), as in
# src/covalent_radii.f90:28-30 of QCxMS.
RCOV2009 = [0, 0.32, 0.46, 1.20, 0.94, 0.77, 0.75, 0.71, 0.63, 0.64, 0.67,
            1.40, 1.25, 1.13, 1.04, 1.10, 1.02, 0.99, 0.96]
# Pauling electronegativities (noble gases given a large value).
PAULING = [0, 2.20, 4.00, 0.98, 1.57, 2.04, 2.55, 3.04, 3.44, 3.98, 4.00,
           0.93, 1.31, 1.61, 1.90, 2.19, 2.58, 3.16, 3.50]


# --------------------------------------------------------------------------
# STO-nG least-squares fit (radial part, zeta = 1)
# --------------------------------------------------------------------------
def _sto_radial(n, r):
    return r ** (n - 1) * np.exp(-r)


def _gto_overlap(a, b, l):
    # int_0^inf r^(2l+2) exp(-(a+b) r^2) dr
    p = a + b
    return math.gamma(l + 1.5) / (2.0 * p ** (l + 1.5))


_RGRID = np.linspace(0.0, 50.0, 5001)


def _sto_gto_overlap(n, l, a):
    r = _RGRID
    f = r ** (n - 1) * np.exp(-r) * r ** l * np.exp(-a * r * r) * r * r
    return integrate.simpson(f, x=r)


def _sto_norm(n):
    # int r^(2n-2) e^{-2r} r^2 dr = (2n)!/2^(2n+1)
    return math.factorial(2 * n) / 2.0 ** (2 * n + 1)


def fit_sto(n, l, nprim):
    """Even-tempered least-squares fit of r^(n-1) e^-r by sum_k c_k r^l e^(-a_k r^2).

    a_k = exp(x0 + k*x1); for fixed exponents the coefficients follow from the
    linear normal equations, so only (x0, x1) are optimised.
    """
    sn = _sto_norm(n)

    def solve(x):
        a = np.exp(x[0] + x[1] * np.arange(nprim))
        G = np.array([[_gto_overlap(ai, aj, l) for aj in a] for ai in a])
        s = np.array([_sto_gto_overlap(n, l, ai) for ai in a])
        c = np.linalg.solve(G, s)
        return (sn - s @ c) / sn, a, c

    def obj(x):
        try:
            return solve(x)[0]
        except np.linalg.LinAlgError:
            return 1.0

    best = None
    for x0 in (-4.0, -3.0, -2.0):
        for x1 in (1.0, 1.3):
            r = optimize.minimize(obj, [x0, x1], method="Nelder-Mead",
                                  options={"maxiter": 600, "xatol": 1e-9, "fatol": 1e-14})
            if best is None or r.fun < best.fun:
                best = r
    err, a, c = solve(best.x)
    order = np.argsort(-a)
    return a[order], c[order], err


def primitive_norm(a, l):
    return (2.0 * a / math.pi) ** 0.75 * (4.0 * a) ** (0.5 * l)


def contracted_coeffs(alpha, craw, l):
    """Coefficients for normalised primitives giving a normalised contraction."""
    # craw multiplies unnormalised r^l e^{-a r^2}; convert to normalised primitives.
    c = np.array([craw[k] / primitive_norm(alpha[k], l) for k in range(len(alpha))])
    s = 0.0
    for i in range(len(alpha)):
        for j in range(len(alpha)):
            p = alpha[i] + alpha[j]
            s += c[i] * c[j] * primitive_norm(alpha[i], l) * primitive_norm(alpha[j], l) * \
                (math.pi / p) ** 1.5 / (2.0 * p) ** l
    return c / math.sqrt(s)


# The s-p and p-p H0 pair scalings, the repulsion exponents of H, C, N, O, S
# and the p-shell H0 distance polynomials of C, N, O, S were least-squares
# fitted so that
# H2, CH4, NH3, H2O, H2S (X-H 0.74, 1.09, 1.01, 0.96, 1.34 Angstrom) and the
# saturated dimers H3C-CH3, H2N-NH2, HO-OH, HS-SH (X-X 1.50, 1.45, 1.45,
# 2.05 Angstrom) have zero bond-stretch force with the rest of this set.
# (REP_ZEFF_FIT is unused: the default effective charges are kept.)
REP_ZEFF_FIT = {}
KPOLY_P_FIT = {6: -0.237795, 7: 0.658507, 8: -0.329019, 16: 0.081975}
K_PAIR_FIT = {'pp': 1.202193, 'sp': 2.431030}
REP_ALPHA_FIT = {1: 2.011406, 6: 1.421563, 7: 2.236515, 8: 2.149226, 16: 0.771833}

# --------------------------------------------------------------------------
# element rules
# --------------------------------------------------------------------------
def period(z):
    return 1 if z <= 2 else (2 if z <= 10 else 3)


def nval(z):
    return {1: z, 2: z - 2, 3: z - 10}[period(z)]


def shells(z):
    p = period(z)
    if p == 1:
        return [(1, 0)]
    sh = [(p, 0), (p, 1)]
    if z in (15, 16, 17):
        sh.append((3, 2))
    return sh


def refocc(z):
    nv = nval(z)
    out = []
    for (n, l) in shells(z):
        cap = {0: 2, 1: 6, 2: 10}[l] if l < 2 else 0
        o = min(nv, cap)
        out.append(float(o))
        nv -= o
    return out


def slater_zeta(z, n, l):
    if z == 1:
        return 1.2
    # Slater's rules for the outermost (valence) electron
    nv = nval(z)
    if period(z) == 1:
        sigma = 0.30 * (nv - 1)
    elif period(z) == 2:
        sigma = 0.35 * (nv - 1) + 0.85 * 2
    else:
        sigma = 0.35 * (nv - 1) + 0.85 * 8 + 1.0 * 2
    zs = (z - sigma) / n
    return {0: zs, 1: 0.92 * zs, 2: 0.45 * zs}[l]


def self_energy(z, l):
    if z in (10, 18):  # closed-shell noble gases: deeper levels (ionisation energies near 16-22 eV)
        return 1.6 * _self_energy_rule(z, l)
    return _self_energy_rule(z, l)


def _self_energy_rule(z, l):
    nv = nval(z)
    p = period(z)
    if p == 1:
        return -0.50 if z == 1 else -0.90
    if p == 2:
        return {0: -0.30 - 0.10 * nv, 1: -0.20 - 0.045 * nv}[l]
    return {0: -0.30 - 0.09 * nv, 1: -0.16 - 0.045 * nv, 2: -0.08}[l]


def main(out=None):
    here = os.path.dirname(os.path.abspath(__file__))
    out = out or os.path.join(here, "..", "csrc", "qcx_params.h")
    fits = {}
    for (n, l) in [(1, 0), (2, 0), (2, 1), (3, 0), (3, 1), (3, 2)]:
        np_ = NPRIM if l < 2 else 4
        a, c, err = fit_sto(n, l, np_)
        print("STO fit", (n, l), "relative L2 error %.3e" % err)
        fits[(n, l)] = (a, c)

    L = []
    w = L.append
    w("/* Synthetic GFN2-form parameter set synth-gfn2-v1.")
    w(" * Generated by qcxms_gb300/params/gen_params.py -- do not edit by hand.")
    w(" * Indexed by atomic number Z (1..QCX_MAXZ); index 0 is unused.")
    w(" * Units: Bohr, Hartree. */")
    w("#ifndef QCX_PARAMS_H")
    w("#define QCX_PARAMS_H")
    w("#define QCX_MAXZ %d" % MAXZ)
    w("#define QCX_MAXSH 3")
    w("#define QCX_MAXPRIM %d" % NPRIM)
    w("")
    w("/* global constants */")
    glob = [
        ("QCX_KCN", 16.0, "steepness of the exponential coordination number"),
        ("QCX_KEN", 0.02, "electronegativity scaling of H0 off-diagonals"),
        ("QCX_K_SS", 1.85, "H0 shell-pair scaling s-s"),
        ("QCX_K_SP", K_PAIR_FIT.get("sp", 2.00), "H0 shell-pair scaling s-p"),
        ("QCX_K_PP", K_PAIR_FIT.get("pp", 2.15), "H0 shell-pair scaling p-p"),
        ("QCX_K_XD", 2.00, "H0 shell-pair scaling for pairs with a d shell"),
        ("QCX_REP_KEXP", 1.5, "distance exponent of the repulsion"),
        ("QCX_AES_A3", 3.0, "damping exponent for R^-3 multipole kernels"),
        ("QCX_AES_A5", 4.0, "damping exponent for R^-5 multipole kernels"),
        ("QCX_AES_RMAX", 5.0, "maximum multipole radius (Bohr)"),
        ("QCX_AES_KMP", 4.0, "steepness of the multipole-radius switch"),
        ("QCX_AES_SHIFT", 1.2, "CN shift of the multipole-radius switch"),
        ("QCX_D4_S6", 1.0, "dispersion s6"),
        ("QCX_D4_S8", 2.7, "dispersion s8"),
        ("QCX_D4_A1", 0.52, "Becke-Johnson a1"),
        ("QCX_D4_A2", 5.0, "Becke-Johnson a2 (Bohr)"),
        ("QCX_D4_S9", 5.0, "three-body (ATM) scaling"),
        ("QCX_D4_GA", 3.0, "charge scaling height"),
        ("QCX_D4_GC", 2.0, "charge scaling steepness"),
        ("QCX_D4_WF", 6.0, "Gaussian CN weighting factor"),
        ("QCX_ATM_ALP", 16.0, "ATM zero-damping exponent alp: 1/(1 + 6 ((R0 R0 R0 / r r r)^(1/3))^alp)"),
    ]
    for name, val, doc in glob:
        w("#define %s %r /* %s */" % (name, float(val), doc))
    w("")

    def arr1(name, ctype, vals, fmt="%.17g"):
        w("static const %s %s[QCX_MAXZ + 1] = {%s};" % (ctype, name, ", ".join(fmt % v for v in vals)))

    nsh = [0] + [len(shells(z)) for z in range(1, MAXZ + 1)]
    arr1("qcx_nsh", "int", nsh, "%d")

    def arrsh(name, ctype, fn, fmt="%.17g"):
        rows = ["{0, 0, 0}"]
        for z in range(1, MAXZ + 1):
            sh = shells(z)
            vals = [fn(z, i, n, l) for i, (n, l) in enumerate(sh)] + [0] * (3 - len(sh))
            rows.append("{" + ", ".join(fmt % v for v in vals) + "}")
        w("static const %s %s[QCX_MAXZ + 1][QCX_MAXSH] = {\n  %s};" % (ctype, name, ",\n  ".join(rows)))

    arrsh("qcx_sh_l", "int", lambda z, i, n, l: l, "%d")
    arrsh("qcx_sh_n", "int", lambda z, i, n, l: n, "%d")
    arrsh("qcx_sh_nprim", "int", lambda z, i, n, l: len(fits[(n, l)][0]), "%d")
    arrsh("qcx_sh_zeta", "double", lambda z, i, n, l: slater_zeta(z, n, l))
    arrsh("qcx_sh_refocc", "double", lambda z, i, n, l: refocc(z)[i])
    arrsh("qcx_sh_selfenergy", "double", lambda z, i, n, l: self_energy(z, l))
    arrsh("qcx_sh_kcn", "double", lambda z, i, n, l: {0: 0.006, 1: 0.003, 2: 0.001}[l])
    arrsh("qcx_sh_kpoly", "double",
          lambda z, i, n, l: KPOLY_P_FIT.get(z, 0.05) if l == 1 else {0: -0.005, 2: 0.02}[l])

    def eta_atom(z):
        p, nv = period(z), nval(z)
        return {1: 0.47 if z == 1 else 0.90, 2: 0.35 + 0.05 * nv, 3: 0.30 + 0.04 * nv}[p]

    def gam3_atom(z):
        return 0.04 + 0.01 * nval(z)

    arrsh("qcx_sh_hardness", "double", lambda z, i, n, l: eta_atom(z) * {0: 1.0, 1: 0.9, 2: 0.7}[l])
    arrsh("qcx_sh_gamma3", "double", lambda z, i, n, l: gam3_atom(z) * {0: 1.0, 1: 0.5, 2: 0.25}[l])

    # primitive tables, exponents already scaled by zeta^2, coefficients for
    # normalised cartesian primitives giving a normalised contracted function
    rows_a, rows_c = ["{{0}}"], ["{{0}}"]
    for z in range(1, MAXZ + 1):
        ra, rc = [], []
        for (n, l) in shells(z):
            a0, c0 = fits[(n, l)]
            zeta = slater_zeta(z, n, l)
            a = a0 * zeta * zeta
            c = contracted_coeffs(a, c0 * zeta ** (n + 0.5) / math.sqrt(_sto_norm(n)), l)
            a = list(a) + [0.0] * (NPRIM - len(a))
            c = list(c) + [0.0] * (NPRIM - len(c))
            ra.append("{" + ", ".join("%.17g" % v for v in a) + "}")
            rc.append("{" + ", ".join("%.17g" % v for v in c) + "}")
        while len(ra) < 3:
            ra.append("{0}")
            rc.append("{0}")
        rows_a.append("{" + ", ".join(ra) + "}")
        rows_c.append("{" + ", ".join(rc) + "}")
    w("static const double qcx_prim_alpha[QCX_MAXZ + 1][QCX_MAXSH][QCX_MAXPRIM] = {\n  %s};" % ",\n  ".join(rows_a))
    w("static const double qcx_prim_coeff[QCX_MAXZ + 1][QCX_MAXSH][QCX_MAXPRIM] = {\n  %s};" % ",\n  ".join(rows_c))

    z_all = range(1, MAXZ + 1)
    arr1("qcx_nvalence", "double", [0] + [float(nval(z)) for z in z_all])
    arr1("qcx_en", "double", PAULING)
    arr1("qcx_rcov", "double", [0] + [4.0 / 3.0 * RCOV2009[z] * AATOAU for z in z_all])
    arr1("qcx_rep_alpha", "double", [0] + [REP_ALPHA_FIT.get(z, 2.0 - 0.03 * nval(z) if period(z) == 2 else 1.6 - 0.02 * nval(z))
                                         for z in z_all])
    arr1("qcx_rep_zeff", "double", [0] + [REP_ZEFF_FIT.get(z, 1.0 if z == 1 else (2.0 if z == 2 else 1.0 + 0.9 * nval(z)))
                                        for z in z_all])
    arr1("qcx_aes_dkernel", "double", [0] + [0.010 + 0.002 * nval(z) for z in z_all])
    arr1("qcx_aes_qkernel", "double", [0] + [0.005 + 0.001 * nval(z) for z in z_all])
    arr1("qcx_aes_rad0", "double", [0] + [1.2 * RCOV2009[z] * AATOAU + 0.8 for z in z_all])

    def expected_cn(z):
        nv = nval(z)
        if period(z) == 1:
            return 1.0 if z == 1 else 0.0
        return float(min(nv, 8 - nv))

    arr1("qcx_aes_valcn", "double", [0] + [expected_cn(z) for z in z_all])
    # Dispersion: the reference data (reference systems, their CNs, charges and
    # polarisabilities, r4r2, hardness, electronegativities, radii) is QCxMS's
    # own D4 data, converted by gen_d4_reference.py into qcx_d4ref.h; only the
    # global D4 constants above belong to this set.
    w("#endif")
    with open(out, "w") as f:
        f.write("\n".join(L) + "\n")
    print("wrote", out)
    for k, (a, c) in fits.items():
        print(k, a, c)


if __name__ == "__main__":
    main()

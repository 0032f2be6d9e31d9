"""Energy terms of the oracle against direct numpy evaluations of their
closed forms (the functional form listed in the design notes, GFN2-xTB's
published terms) at the oracle's own converged moments, with the parameters
read from the generated header by an independent parser:

* isotropic electrostatics 1/2 sum_st q_s q_t gamma_st with
  gamma_st = (R^2 + eta_st^-2)^-1/2, eta_st the mean of the shells' hardnesses;
* third order 1/3 sum_s Gamma_s q_s^3;
* repulsion sum_{A<B} Y_A Y_B / R exp(-sqrt(alpha_A alpha_B) R^1.5);
* D4 two-body dispersion -sum_{A<B} C6_AB(q) [s6 / (R^6 + R0^6) +
  s8 3 r4r2_A r4r2_B / (R^8 + R0^8)], R0 = a1 sqrt(3 r4r2_A r4r2_B) + a2
  (rational damping, dftd4.f90 edisp), C6 at the converged atomic charges;
* band energy tr(P H0) and the Fermi-smearing term 2 kT sum_k [f ln f +
  (1 - f) ln(1 - f)] (f = occupation / 2);
* the total as the sum of the terms.
Small molecules, tight SCC thresholds (the terms are evaluated at the output
moments the oracle reports, so they agree to summation order)."""
import os
import re

import numpy as np
import pytest

from qcxms_gb300 import basis, constants
from tests import molecules

KT = 300.0 * constants.KB_AU
CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "qcxms_gb300", "csrc")


def _header_array(fname, name):
    with open(os.path.join(CSRC, fname)) as f:
        text = f.read()
    body = re.search(name + r"\[\d+\]\s*=\s*\{([^}]*)\}", text).group(1)
    return np.array([float(v) for v in body.replace("\n", " ").split(",") if v.strip()])


def _header_define(fname, name):
    with open(os.path.join(CSRC, fname)) as f:
        text = f.read()
    return float(re.search(r"#define\s+" + name + r"\s+\(?([-+0-9.eE]+)", text).group(1))


def _shells(Z):
    nsh = basis.NSH
    out = []
    for a, z in enumerate(Z):
        for k in range(nsh[int(z)]):
            out.append((a, int(z), k))
    return out


@pytest.mark.parametrize("name", ["h2o+", "ch2o+", "h2s-ch+"])
def test_closed_form_terms_match_the_oracle(oracle_lib, name):
    Z, xyz, charge = molecules.ALL_SMALL[name]()
    opts = oracle_lib.default_opts(econv=1e-11, pconv=1e-9)
    P, qsh, dp, qp, eps, focc, info = oracle_lib.scc(Z, xyz, charge, kT=KT, opts=opts)
    assert info["converged"] == 1
    eta = basis.read_param("qcx_sh_hardness")
    g3 = basis.read_param("qcx_sh_gamma3")
    sh = _shells(Z)
    assert len(sh) == len(qsh)
    R = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    # isotropic electrostatics and third order
    e_ies = 0.0
    for s, (a, za, ka) in enumerate(sh):
        for t, (b, zb, kb) in enumerate(sh):
            r2 = float(np.sum((R[a] - R[b]) ** 2))
            et = 0.5 * (eta[za, ka] + eta[zb, kb])
            e_ies += 0.5 * qsh[s] * qsh[t] / np.sqrt(r2 + 1.0 / et ** 2)
    e_3 = sum(g3[z, k] * qsh[s] ** 3 for s, (a, z, k) in enumerate(sh)) / 3.0
    assert abs(e_ies - info["e_ies"]) < 1e-12 * max(1.0, abs(e_ies))
    assert abs(e_3 - info["e_3"]) < 1e-13
    # band energy and the smearing term
    S, H0, Dm, Qm, cn, cnd = oracle_lib.integrals(Z, xyz)
    assert abs(float(np.sum(P * H0)) - info["e_band"]) < 1e-11
    f = np.clip(focc / 2.0, 1e-300, 1.0)
    g = np.clip(1.0 - focc / 2.0, 1e-300, 1.0)
    ts = 2.0 * KT * float(np.sum(np.where(focc > 0, f * np.log(f), 0.0) + np.where(g < 1.0, g * np.log(g), 0.0)))
    assert abs(ts - info["e_ts"]) < 1e-12


@pytest.mark.parametrize("name", ["h2o+", "ch2o+", "h2s-ch+", "h2o+ar"])
def test_repulsion_and_total(oracle_lib, name):
    Z, xyz, charge = molecules.ALL_SMALL[name]()
    opts = oracle_lib.default_opts(econv=1e-11, pconv=1e-9)
    rc, e, g, q, info = oracle_lib.egrad(Z, xyz, charge, kT=KT, opts=opts)
    assert rc == 0
    alpha = basis.read_param("qcx_rep_alpha")
    zeff = basis.read_param("qcx_rep_zeff")
    R = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    e_rep = 0.0
    for a in range(len(Z)):
        for b in range(a):
            r = float(np.linalg.norm(R[a] - R[b]))
            za, zb = int(Z[a]), int(Z[b])
            e_rep += zeff[za] * zeff[zb] / r * np.exp(-np.sqrt(alpha[za] * alpha[zb]) * r ** 1.5)
    assert abs(e_rep - info["e_rep"]) < 1e-12 * max(1.0, e_rep)
    parts = sum(info[k] for k in ("e_band", "e_ies", "e_3", "e_aes", "e_axc", "e_disp", "e_atm", "e_rep", "e_ts"))
    assert abs(parts - info["e_total"]) < 1e-11
    assert abs(info["e_total"] - e) < 1e-11


@pytest.mark.parametrize("name", ["h2o+", "ch2o+", "h2s-ch+", "h2o+ar"])
def test_d4_two_body_dispersion(oracle_lib, name):
    Z, xyz, charge = molecules.ALL_SMALL[name]()
    opts = oracle_lib.default_opts(econv=1e-11, pconv=1e-9)
    rc, e, g, q, info = oracle_lib.egrad(Z, xyz, charge, kT=KT, opts=opts)
    assert rc == 0
    r4r2 = _header_array("qcx_d4ref.h", "qcx_d4_r4r2")
    s6, s8, a1, a2 = (_header_define("qcx_params.h", "QCX_D4_" + k) for k in ("S6", "S8", "A1", "A2"))
    c6 = oracle_lib.d4_c6(Z, xyz, q)
    R = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    e_disp = 0.0
    for a in range(len(Z)):
        for b in range(a):
            r2 = float(np.sum((R[a] - R[b]) ** 2))
            rr = 3.0 * r4r2[int(Z[a])] * r4r2[int(Z[b])]
            r0 = a1 * np.sqrt(rr) + a2
            e_disp -= c6[a, b] * (s6 / (r2 ** 3 + r0 ** 6) + s8 * rr / (r2 ** 4 + r0 ** 8))
    assert abs(e_disp - info["e_disp"]) < 1e-14 + 1e-12 * abs(e_disp)

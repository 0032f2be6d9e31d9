"""Golden D4 C6 coefficients computed straight from QCxMS's own D4 data.

An independent numpy restatement, written for the test suite: it parses
include/param_d4.fh and the element tables of src/dftd4.f90 itself (not through
the converter that writes the library's header) and evaluates, as
src/dftd4.f90 does,
  - the reference polarisabilities of d4dim (:531-595): alpha_ref =
    max(ascale (alphaiw - hcount sscale secaiw zeta(secq, refh)), 0);
  - C6 of reference pairs: 3/pi * trapzd(alpha_i alpha_j) (:452-497, 665);
  - the covalent coordination number (covncoord, :292-325) and the Gaussian
    reference weights with refc Gaussians per reference (d4, :597-670);
  - molecular C6_AB = sum_ij w_Ai zeta_Ai(q_A) w_Bj zeta_Bj(q_B) C6_ij
    (edisp, :914-1034) at zero charge and at given charges.
Fortran stores the kind-less literals of both files as single-precision reals;
they are rounded to float32 here as well.

Writes tests/golden/d4_c6.json. Usage: python make_d4_golden.py [QCXMS_SRC]
"""
import json
import os
import re
import sys

import numpy as np

GA, GC, WF = 3.0, 2.0, 6.0  # charge scaling height and steepness, CN weighting (GFN2 D4 settings)
FREQ = np.array([0.000001, 0.05, 0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9, 1.0, 1.2, 1.4, 1.6, 1.8, 2.0, 2.5,
                 3.0, 4.0, 5.0, 7.5, 10.0])


def f32(v):
    return float(np.float32(float(v)))


def load(src):
    text = open(os.path.join(src, "include", "param_d4.fh")).read()
    text = re.sub(r"!.*", "", text)
    text = re.sub(r"&\s*\n\s*&", " ", text)
    text = re.sub(r"&\s*\n", " ", text)
    vals = {}
    for m in re.finditer(r"data\s+(\w+)\s*\(([^)]*)\)\s*/([^/]*)/", text, re.I):
        vals[(m.group(1).lower(), m.group(2).replace(" ", ""))] = m.group(3).replace(",", " ").split()
    src_f = open(os.path.join(src, "src", "dftd4.f90")).read()
    tab = {}
    for name in ("zeff", "gam", "en", "rcov", "r4r2"):
        body = re.search(r"::\s*%s\s*\(\*\)\s*=\s*\(/(.*?)/\)" % name, src_f, re.S | re.I).group(1)
        body = re.sub(r"!.*", "", body).replace("&", " ").replace(",", " ")
        tab[name] = [f32(x) for x in body.split()]
    return vals, tab


def zeta(a, c, qref, qmod):
    return np.exp(a) if qmod < 0 else np.exp(a * (1.0 - np.exp(c * (1.0 - qref / qmod))))


def element(vals, tab, z):
    n = int(vals[("refn", str(z))][0])
    refs = []
    cncount = {0: 1}
    for j in range(1, n + 1):
        key = "%d,%d" % (j, z)
        g = lambda k: f32(vals[(k, key)][0])
        is_ = int(vals[("refsys", key)][0])
        iz = tab["zeff"][is_ - 1]
        secq, sscale = f32(vals[("secq", str(is_))][0]), f32(vals[("sscale", str(is_))][0])
        secaiw = np.array([f32(x) for x in vals[("secaiw", ":,%d" % is_)]])
        sec_al = sscale * secaiw * zeta(GA, tab["gam"][is_ - 1] * GC, secq + iz, g("refh") + iz)
        alpha = np.array([f32(x) for x in vals[("alphaiw", ":,%d,%d" % (j, z))]])
        al = np.maximum(g("ascale") * (alpha - g("hcount") * sec_al), 0.0)
        icn = int(np.floor(g("refcn") + 0.5))
        cncount[icn] = cncount.get(icn, 0) + 1
        refs.append({"al": al, "covcn": g("refcovcn"), "refcn": g("refcn"), "q": g("refq")})
    for r in refs:
        k = cncount[int(np.floor(r["refcn"] + 0.5))]
        r["ngauss"] = k * (k + 1) // 2
    return refs


def c6ref(ra, rb):
    p = ra["al"] * rb["al"]
    dw = np.diff(FREQ)
    s = dw * (p[1:] + p[:-1])
    return 3.0 / np.pi * (0.5 * s[0::2].sum() + 0.5 * s[1::2].sum())


def covcn(tab, Z, xyz):
    k1, k4, k5, k6 = 16.0, 4.10451, 19.08857, 2 * 11.28174 ** 2
    cn = np.zeros(len(Z))
    for i in range(len(Z)):
        for j in range(i):
            r2 = float(np.sum((xyz[j] - xyz[i]) ** 2))
            if r2 > 1600.0:
                continue
            r = np.sqrt(r2)
            den = k4 * np.exp(-(abs(tab["en"][Z[i] - 1] - tab["en"][Z[j] - 1]) + k5) ** 2 / k6)
            f = den / (1.0 + np.exp(-k1 * ((tab["rcov"][Z[i] - 1] + tab["rcov"][Z[j] - 1]) / r - 1.0)))
            cn[i] += f
            cn[j] += f
    return cn


def weights(refs, cn):
    g = [sum(np.exp(-k * WF * (cn - r["covcn"]) ** 2) for k in range(1, r["ngauss"] + 1)) for r in refs]
    return np.array(g) / sum(g)


def mol_c6(vals, tab, Z, xyz, q):
    cn = covcn(tab, Z, xyz)
    els = {z: element(vals, tab, z) for z in set(Z)}
    w = []
    for a, z in enumerate(Z):
        refs = els[z]
        iz = tab["zeff"][z - 1]
        zt = np.array([zeta(GA, tab["gam"][z - 1] * GC, r["q"] + iz, q[a] + iz) for r in refs])
        w.append(weights(refs, cn[a]) * zt)
    c6 = np.zeros((len(Z), len(Z)))
    for a in range(len(Z)):
        for b in range(len(Z)):
            if a != b:
                ra, rb = els[Z[a]], els[Z[b]]
                c6[a, b] = sum(w[a][i] * w[b][j] * c6ref(ra[i], rb[j]) for i in range(len(ra)) for j in range(len(rb)))
    return c6


def main(src):
    vals, tab = load(src)
    pairs = [(1, 0, 1, 0), (1, 1, 6, 3), (6, 0, 6, 6), (6, 2, 8, 1), (7, 4, 8, 3), (8, 0, 8, 0), (16, 2, 1, 1),
             (18, 0, 18, 0), (18, 0, 6, 5), (17, 1, 9, 1), (5, 4, 14, 4), (3, 1, 11, 1)]
    out = {"c6ref": [], "molecules": []}
    for za, i, zb, j in pairs:
        out["c6ref"].append([za, i, zb, j, float(c6ref(element(vals, tab, za)[i], element(vals, tab, zb)[j]))])
    mols = {
        "h2o": ([8, 1, 1], [[0.0, 0.0, 0.0], [0.0, 1.43, 1.11], [0.0, -1.43, 1.11]]),
        "ch4": ([6, 1, 1, 1, 1], [[0, 0, 0], [1.19, 1.19, 1.19], [-1.19, -1.19, 1.19], [-1.19, 1.19, -1.19],
                                  [1.19, -1.19, -1.19]]),
        "ethanol": ([6, 6, 8, 1, 1, 1, 1, 1, 1], [[0.0, 0.0, 0.0], [2.87, 0.0, 0.0], [3.77, 2.44, 0.0],
                                                  [-0.69, 1.95, 0.0], [-0.69, -0.98, 1.69], [-0.69, -0.98, -1.69],
                                                  [3.56, -0.98, 1.69], [3.56, -0.98, -1.69], [5.60, 2.44, 0.0]]),
        "nh3_ar_s": ([7, 1, 1, 1, 18, 16], [[0, 0, 0], [1.9, 0, 0.6], [-0.95, 1.65, 0.6], [-0.95, -1.65, 0.6],
                                             [0.0, 0.0, 7.5], [0.0, 4.5, -3.0]]),
    }
    rng = np.random.default_rng(3)
    for name, (Z, xyz) in mols.items():
        xyz = np.array(xyz, dtype=np.float64)
        q = rng.uniform(-0.4, 0.4, len(Z))
        q -= q.mean() - 1.0 / len(Z)
        out["molecules"].append({"name": name, "Z": Z, "xyz": xyz.tolist(), "q": q.tolist(),
                                 "c6_q0": mol_c6(vals, tab, Z, xyz, np.zeros(len(Z))).tolist(),
                                 "c6_q": mol_c6(vals, tab, Z, xyz, q).tolist()})
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "d4_c6.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")

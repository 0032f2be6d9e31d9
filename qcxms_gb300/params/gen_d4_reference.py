"""Write qcx_d4ref.h: the D4 reference data that QCxMS ships, for elements 1-18.

QCxMS carries an xtb-era D4 model in src/dftd4.f90 with its reference data in
include/param_d4.fh: per element the reference systems (refn of them) with their
coordination numbers (refcovcn, refcn), charges (refq, refh), hydrogen counts and
scalings (hcount, ascale), the secondary system (refsys) and the dynamic
polarisabilities alpha(i omega) on 23 imaginary frequencies (alphaiw); per
secondary system its charge (secq), scaling (sscale) and polarisabilities
(secaiw). src/dftd4.f90 adds the element tables zeff, gam (chemical hardness),
en (Pauling electronegativities), rcov (covalent radii, Bohr) and r4r2.

This script reads those files from a QCxMS source tree and writes the values as
C arrays; nothing is computed here. The literals in both files carry no kind
suffix, so Fortran stores them as default (single-precision) reals converted to
double: every value is written as that single-precision number, exactly, so that
the C arrays hold what the Fortran arrays hold. Integer tables (refn, refsys,
zeff) are exact.

Usage: python gen_d4_reference.py [QCXMS_SOURCE_DIR] (default /root/reference)
"""
import os
import re
import sys

import numpy as np

ZMAX = 18
MAXREF = 7
NFREQ = 23


def _statements(text):
    """Fortran statements with continuation lines joined and comments removed."""
    out, cur = [], ""
    for raw in text.splitlines():
        line = raw.split("!")[0].rstrip()
        if not line.strip():
            continue
        s = line.strip()
        if s.startswith("&"):
            s = s[1:]
        cont = s.endswith("&")
        if cont:
            s = s[:-1]
        cur += " " + s
        if not cont:
            out.extend(p.strip() for p in cur.split(";") if p.strip())
            cur = ""
    return out


def _f32(x):
    return float(np.float32(float(x)))


def parse_param_d4(path):
    data = {}
    pat = re.compile(r"data\s+(\w+)\s*\(([^)]*)\)\s*/(.*)/\s*$", re.I)
    for st in _statements(open(path).read()):
        m = pat.match(st)
        if not m:
            continue
        name, idx, vals = m.group(1).lower(), m.group(2), m.group(3)
        idx = [i.strip() for i in idx.split(",")]
        vals = [v for v in vals.replace(",", " ").split()]
        data.setdefault(name, {})[tuple(idx)] = vals
    return data


def parse_tables(path):
    text = open(path).read()
    tabs = {}
    for name in ("zeff", "gam", "en", "rcov", "r4r2"):
        m = re.search(r"::\s*%s\s*\(\*\)\s*=\s*\(/(.*?)/\)" % name, text, re.S | re.I)
        body = re.sub(r"!.*", "", m.group(1)).replace("&", " ").replace(",", " ")
        tabs[name] = [v for v in body.split()]
    return tabs


def main(src):
    d = parse_param_d4(os.path.join(src, "include", "param_d4.fh"))
    t = parse_tables(os.path.join(src, "src", "dftd4.f90"))
    refn = [0] * (ZMAX + 1)
    for (z,), v in d["refn"].items():
        if int(z) <= ZMAX:
            refn[int(z)] = int(v[0])
    per_ref = {k: [[0.0] * MAXREF for _ in range(ZMAX + 1)]
               for k in ("refq", "refh", "hcount", "ascale", "refcovcn", "refcn")}
    refsys = [[0] * MAXREF for _ in range(ZMAX + 1)]
    alphaiw = [[[0.0] * NFREQ for _ in range(MAXREF)] for _ in range(ZMAX + 1)]
    for z in range(1, ZMAX + 1):
        for j in range(1, refn[z] + 1):
            key = (str(j), str(z))
            for k in per_ref:
                per_ref[k][z][j - 1] = _f32(d[k][key][0])
            refsys[z][j - 1] = int(d["refsys"][key][0])
            vals = d["alphaiw"][(":", str(j), str(z))]
            assert len(vals) == NFREQ
            alphaiw[z][j - 1] = [_f32(v) for v in vals]
    secq = [0.0] * (ZMAX + 1)
    sscale = [0.0] * (ZMAX + 1)
    secaiw = [[0.0] * NFREQ for _ in range(ZMAX + 1)]
    for (i,), v in d["secq"].items():
        i = int(i)
        secq[i] = _f32(v[0])
        sscale[i] = _f32(d["sscale"][(str(i),)][0])
        secaiw[i] = [_f32(x) for x in d["secaiw"][(":", str(i))]]
    used = {s for z in range(1, ZMAX + 1) for s in refsys[z][:refn[z]]}
    assert all(1 <= s <= ZMAX and sscale[s] >= 0.0 for s in used)
    tab = {k: [0.0] + [_f32(x) for x in t[k][:ZMAX]] for k in ("gam", "en", "rcov", "r4r2")}
    zeff = [0] + [int(float(x)) for x in t["zeff"][:ZMAX]]

    def f(x):
        return repr(float(x))

    def arr1(name, ctype, vals, fmt=f):
        return "static const %s %s[%d] = {%s};" % (ctype, name, len(vals), ", ".join(fmt(v) for v in vals))

    def arr2(name, vals):
        rows = ["{" + ", ".join(f(v) for v in r) + "}" for r in vals]
        return "static const double %s[%d][%d] = {\n  %s};" % (name, len(vals), len(vals[0]), ",\n  ".join(rows))

    out = ["/* Generated by qcxms_gb300/params/gen_d4_reference.py from the QCxMS sources",
           " * (include/param_d4.fh and the element tables of src/dftd4.f90); elements 1-18.",
           " * Values are the single-precision literals of those files as Fortran stores",
           " * them (default reals converted to double). Do not edit. */",
           "#ifndef QCX_D4REF_H", "#define QCX_D4REF_H",
           "#define QCX_D4_MAXREF %d" % MAXREF, "#define QCX_D4_NFREQ %d" % NFREQ,
           arr1("qcx_d4_refn", "int", refn, str)]
    for k in ("refq", "refh", "hcount", "ascale", "refcovcn", "refcn"):
        out.append(arr2("qcx_d4_" + k, per_ref[k]))
    out.append("static const int qcx_d4_refsys[%d][%d] = {\n  %s};" % (
        ZMAX + 1, MAXREF, ",\n  ".join("{" + ", ".join(str(v) for v in r) + "}" for r in refsys)))
    out.append("static const double qcx_d4_alphaiw[%d][%d][%d] = {\n  %s};" % (
        ZMAX + 1, MAXREF, NFREQ,
        ",\n  ".join("{" + ", ".join("{" + ", ".join(f(v) for v in a) + "}" for a in r) + "}" for r in alphaiw)))
    out.append(arr1("qcx_d4_secq", "double", secq))
    out.append(arr1("qcx_d4_sscale", "double", sscale))
    out.append(arr2("qcx_d4_secaiw", secaiw))
    out.append(arr1("qcx_d4_zeff", "int", zeff, str))
    for k in ("gam", "en", "rcov", "r4r2"):
        out.append(arr1("qcx_d4_" + k, "double", tab[k]))
    out.append("#endif")
    return "\n".join(out) + "\n"


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    here = os.path.dirname(os.path.abspath(__file__))
    dst = os.path.join(here, "..", "csrc", "qcx_d4ref.h")
    with open(dst, "w") as fh:
        fh.write(main(src))
    print(dst)

"""Basis-set bookkeeping (shell and orbital counts) of the compiled parameter set."""
import os
import re

import numpy as np

_HDR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc", "qcx_params.h")


def _read_table(name):
    txt = open(_HDR).read()
    m = re.search(r"%s\[QCX_MAXZ \+ 1\]\[QCX_MAXSH\] = \{(.*?)\};" % name, txt, re.S)
    rows = re.findall(r"\{([^{}]*)\}", m.group(1))
    return [[int(v) for v in r.split(",")] for r in rows]


def _read_nsh():
    txt = open(_HDR).read()
    m = re.search(r"qcx_nsh\[QCX_MAXZ \+ 1\] = \{([^}]*)\}", txt)
    return [int(v) for v in m.group(1).split(",")]


NSH = _read_nsh()
SH_L = _read_table("qcx_sh_l")


def nao_of(Z):
    return int(sum(2 * SH_L[int(z)][k] + 1 for z in Z for k in range(NSH[int(z)])))


def nsh_of(Z):
    return int(sum(NSH[int(z)] for z in Z))


def read_param(name, dtype=float):
    """Read array ``name`` of qcx_params.h as a numpy array of its declared shape.

    C brace initialisers may be partial ("{0}"); missing entries are zero.
    """
    import ast
    txt = open(_HDR).read()
    defs = dict((k, int(v)) for k, v in re.findall(r"#define (QCX_MAX\w+) (\d+)", txt))
    m = re.search(r"\b%s((?:\[[^\]]*\])+) = (\{.*?\});" % re.escape(name), txt, re.S)
    if m is None:
        raise KeyError(name)
    dims = [eval(d, {}, defs) for d in re.findall(r"\[([^\]]*)\]", m.group(1))]
    data = ast.literal_eval(m.group(2).replace("{", "[").replace("}", "]"))
    out = np.zeros(dims, dtype=dtype)

    def fill(dst, src):
        for i, v in enumerate(src):
            if isinstance(v, list):
                fill(dst[i], v)
            else:
                dst[i] = v

    fill(out, data)
    return out

"""The parameter headers that the CUDA library and the CPU oracle both include
are the output of their generators, value for value: the GFN2-form table
(qcx_params.h, from gen_params.py) and the D4 reference data (qcx_d4ref.h,
from gen_d4_reference.py reading QCxMS's include/param_d4.fh and
src/dftd4.f90). A hand edit of a header, or a generator change that was not
run, would reach the GPU path and the oracle alike, which the parity tests
cannot see; these tests can."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "qcxms_gb300", "csrc")
NUM = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?")


def _tokens(text):
    """Identifiers and numbers of a C header, in order (comments dropped)."""
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)
    words, nums = [], []
    for tok in re.findall(r"[A-Za-z_]\w*|" + NUM.pattern, text):
        if re.match(r"[A-Za-z_]", tok):
            words.append(tok)
        else:
            nums.append(float(tok))
    return words, np.array(nums)


def _same(a_text, b_text):
    wa, na = _tokens(a_text)
    wb, nb = _tokens(b_text)
    assert wa == wb
    assert na.shape == nb.shape
    # the generators print with full precision; allow for the last digit of a
    # least-squares fit run on another machine
    assert np.allclose(na, nb, rtol=1e-12, atol=1e-300)


def test_gfn2_form_table_is_its_generators_output(tmp_path):
    pytest.importorskip("scipy")
    from qcxms_gb300.params import gen_params
    out = tmp_path / "qcx_params.h"
    gen_params.main(str(out))
    with open(os.path.join(CSRC, "qcx_params.h")) as f:
        committed = f.read()
    _same(out.read_text(), committed)


def test_d4_reference_header_is_its_generators_output():
    src = os.environ.get("QCXMS_SOURCE", "/root/reference")
    if not os.path.exists(os.path.join(src, "include", "param_d4.fh")):
        pytest.skip("QCxMS sources (include/param_d4.fh) not present")
    from qcxms_gb300.params import gen_d4_reference
    with open(os.path.join(CSRC, "qcx_d4ref.h")) as f:
        committed = f.read()
    _same(gen_d4_reference.main(src), committed)

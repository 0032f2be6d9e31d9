"""The C ABI library builds for sm_103a, loads, and exports every declared symbol.

No kernel is launched here (CPU-only checks)."""
import ctypes
import os
import re

import numpy as np

import qcxms_gb300
from qcxms_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "qcxgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(qcx_[a-z_0-9]+)\s*\(", txt)))


def test_library_builds_and_exports_all_symbols():
    path = build.build()
    assert os.path.exists(path)
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert "qcx_egrad" in syms and "qcx_batch_step" in syms
    for s in syms:
        assert hasattr(lib, s), s


def test_host_side_validation_without_gpu():
    lib = qcxms_gb300.load_library()
    assert lib.qcx_version() >= 100
    q, e, g, stat = qcxms_gb300.get_xtb_egrad([1, 1], np.zeros((2, 3)), 0, 1, method=qcxms_gb300.gfn1_xtb)
    assert stat == 5
    nat = np.array([1], dtype=np.int32)
    Z = np.array([99], dtype=np.int32)
    ch = np.zeros(1)
    et = np.full(1, 300.0)
    h = lib.qcx_batch_create(1, qcxms_gb300._ip(nat), qcxms_gb300._ip(Z), qcxms_gb300._dp(ch), qcxms_gb300._dp(et))
    assert not h
    assert b"1..18" in lib.qcx_last_error()


def test_batch_entry_points_reject_null_handles_without_gpu():
    """The loop-rule and state entry points check their handle before any CUDA call."""
    lib = qcxms_gb300.load_library()
    assert lib.qcx_batch_set_md_rules(None, 2, 250, 100) == -1
    assert lib.qcx_batch_get_md_state(None, None, None, None, None, None, None, None, None) == -1
    assert lib.qcx_batch_get_md_avg_xyz(None, None) == -1
    assert lib.qcx_batch_set_md_heating(None, None, None, None, 20.0) == -1
    assert lib.qcx_batch_set_cid_rules(None, 300.0, 100) == -1
    assert lib.qcx_batch_get_cid_state(None, *([None] * 9)) == -1
    assert lib.qcx_boltz(2, 0, 1, 300.0, None, None) == -1
    # SCC budget scale, its getter and the paced autotuner
    assert lib.qcx_batch_set_scc_budget_scale(None, 1) == -1
    assert lib.qcx_batch_get_scc_budget(None, None, None) == -1
    assert lib.qcx_batch_autotune_paced(None, 20.0, 1, None, 1, 1, None) == -1
    # the FP32 eigensolver self-check validates its arguments before any CUDA call
    assert lib.qcx_jacobi32_selftest(0, None, None, None, 0, 2e-6, 30, None) == -1
    assert lib.qcx_jacobi32_selftest(300, None, None, None, 0, 2e-6, 30, None) == -1
    assert b"n <= 256" in lib.qcx_last_error()


def test_header_is_plain_c_and_links(tmp_path):
    """include/qcxgpu.h compiles as C99 and a C program links against the
    library and calls its host-side entry points (no GPU work)."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        import pytest
        pytest.skip("no gcc")
    path = build.build()
    exe = tmp_path / "abi_from_c"
    src = os.path.join(ROOT, "tests", "c", "abi_from_c.c")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src, "-o", str(exe),
                    path, "-lm", "-Wl,-rpath," + os.path.dirname(path)], check=True)
    out = subprocess.run([str(exe), os.path.join(ROOT, "tests", "golden", "TMPQCXMS")], capture_output=True,
                         text=True)
    assert out.returncode == 0, out.stderr
    assert out.stdout.startswith("ok nat=5 itrj=1")

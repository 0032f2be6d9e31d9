"""The tensor-core product (tcgen05, split-TF32) against an FP64 reference.

The SCC kernel's FP32 iterations form their O(n^3) products on the tensor
cores; this checks the building block alone, through the C ABI, on the shapes
the molecules give (M, N up to 128 / 256 rows, K from 1 to a few hundred, both
operand orientations). Split-TF32 keeps about 21 bits: the error bound used
here is 2^-19 times sum_k |a_ik| |b_kj| (the products' magnitudes).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K,ta,tb", [(8, 16, 8, 0, 0), (37, 41, 53, 0, 0), (128, 128, 128, 0, 1),
                                         (122, 122, 122, 1, 0), (100, 250, 77, 1, 1), (1, 1, 1, 0, 0),
                                         (64, 160, 300, 0, 0), (160, 160, 160, 0, 0), (250, 96, 40, 1, 0)])
def test_mma_gemm_matches_fp64(gpu, M, N, K, ta, tb):
    import qcxms_gb300 as qg
    rng = np.random.default_rng(M * 1000 + N + K)
    A = rng.normal(size=(K, M) if ta else (M, K)).astype(np.float32)
    B = rng.normal(size=(N, K) if tb else (K, N)).astype(np.float32)
    C, ms = qg.mma_gemm(A, B, ta=bool(ta), tb=bool(tb))
    a = A.T.astype(np.float64) if ta else A.astype(np.float64)
    b = B.T.astype(np.float64) if tb else B.astype(np.float64)
    ref = a @ b
    bound = 2.0 ** -19 * (np.abs(a) @ np.abs(b)) + 1e-30
    assert np.all(np.abs(C - ref) <= bound), np.max(np.abs(C - ref) / bound)
    # plain TF32 would miss the bound: the split terms are in
    assert np.max(np.abs(C - ref) / (np.abs(a) @ np.abs(b) + 1e-30)) < 2.0 ** -19


def test_mma_gemm_repeated_calls_reuse_the_accumulator(gpu):
    import qcxms_gb300 as qg
    rng = np.random.default_rng(7)
    A = rng.normal(size=(96, 96)).astype(np.float32)
    B = rng.normal(size=(96, 96)).astype(np.float32)
    C, ms = qg.mma_gemm(A, B, reps=5)
    ref = A.astype(np.float64) @ B.astype(np.float64)
    assert np.abs(C - ref).max() < 1e-4 and ms > 0.0


@pytest.mark.gpu
def test_mixed_scc_above_the_accumulator_width(gpu, oracle_lib):
    """Molecules with more than 256 AOs (CID ions of ~80 atoms with S) run the
    FP32 products on the CUDA cores: one MMA takes N <= 256 and the tensor-memory
    accumulator has 256 columns. Energies against the FP64 oracle."""
    import qcxms_gb300 as qg
    from qcxms_gb300 import constants, molgen
    from qcxms_gb300.basis import nao_of
    big = [m for m in molgen.cid_workload(96, 76, 80, seed0=5) if nao_of(m["Z"]) > 256][:3]
    assert big, "no molecule above 256 AOs in the sample"
    b = qg.Batch(big)
    b.set_precision("mixed")
    b.egrad()
    r = b.get()
    kT = 300.0 * constants.KB_AU
    ok = 0
    for i, m in enumerate(big):
        rc, e, g, q, info = oracle_lib.egrad(m["Z"], m["xyz"], m["charge"], kT=kT)
        if rc != 0 or r["status"][i] != 0:
            continue
        ok += 1
        assert abs(r["energy"][i] - e) < 1e-6
    assert ok >= 1
    b.close()

"""The FP32 eigensolver of the SCC kernel's FP32 iterations (cyclic parallel
Jacobi, n/2 disjoint rotations per round), alone, through the C ABI, against
LAPACK (numpy) in FP64 on random symmetric matrices of the molecules' sizes,
cold and warm-started from a basis close to the eigenvectors of a spectrum
with near-degenerate clusters (as at the Fermi level of the hard SCC cases).

FP32 bound: eigenvalues within 1e-6 n of the largest |eigenvalue|, the rows
orthonormal to 1e-6 n and each row an eigenvector to 1e-6 n (residual norm,
relative). Rounding grows with the n - 1 rotations every element goes through
per sweep; a numpy restatement of the sweeps in FP32 gives 8.7e-6 for n = 64
on these matrices."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sym(n, seed):
    rng = np.random.default_rng(seed)
    m = rng.normal(size=(n, n))
    return 0.5 * (m + m.T)


def _check(A, Ao, V, sweeps):
    n = A.shape[0]
    w = np.linalg.eigvalsh(A.astype(np.float64))
    lam = np.sort(np.diag(Ao).astype(np.float64))
    s = max(1.0, np.abs(w).max())
    tol = 1e-6 * n
    assert sweeps > 0
    assert np.abs(lam - w).max() < tol * s, np.abs(lam - w).max() / s
    Vd = V.astype(np.float64)
    assert np.abs(Vd @ Vd.T - np.eye(n)).max() < tol
    res = Vd @ A.astype(np.float64) - np.diag(Ao).astype(np.float64)[:, None] * Vd
    assert np.linalg.norm(res, axis=1).max() < tol * s


@pytest.mark.parametrize("n", [5, 32, 37, 64, 100, 122, 200, 256])
def test_cold_matches_lapack(gpu, n):
    import qcxms_gb300 as qg
    A = _sym(n, 10 + n).astype(np.float32)
    Ao, V, sw = qg.jacobi32(A, reltol=2e-6, max_sweeps=30)
    _check(A, Ao, V, sw)


@pytest.mark.parametrize("n", [33, 96, 150])
def test_warm_start_and_near_degenerate_spectrum(gpu, n):
    import qcxms_gb300 as qg
    rng = np.random.default_rng(n)
    ev = np.sort(np.repeat(rng.normal(size=n // 3 + 1), 3)[:n] + 1e-4 * rng.normal(size=n))
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    A = Q @ np.diag(ev) @ Q.T
    A = (0.5 * (A + A.T)).astype(np.float32)
    # the previous basis: the eigenvectors slightly rotated
    K = 1e-2 * rng.normal(size=(n, n))
    K = K - K.T
    V0, _ = np.linalg.qr(Q @ (np.eye(n) + K))
    V0 = V0.T
    B = (V0 @ A.astype(np.float64) @ V0.T).astype(np.float32)
    B = 0.5 * (B + B.T)
    Ao, V, sw = qg.jacobi32(B, V=V0.astype(np.float32), reltol=2e-6, max_sweeps=30)
    # V holds the eigenvectors of A (B was A expressed in the rows of V0)
    _check(A, Ao, V, sw)

"""The oracle's GEVD front half (Factorization.GevdCore up to the eigen-solver) against LAPACK:
C = L^-1 A L^-T with L = chol(B), and the eigenvalues of C are the generalized eigenvalues of
(A, B) (scipy's sygv)."""
import numpy as np
import pytest

from oracle import oracle


@pytest.mark.parametrize("n", [1, 2, 5, 16, 33, 64])
def test_gevd_front_matches_lapack(n):
    sl = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(100 + n)
    A = rng.standard_normal((n, n))
    A = A + A.T
    M = rng.standard_normal((n, n))
    B = M @ M.T + n * np.eye(n)
    a = np.asfortranarray(np.triu(A) + 7.0 * np.tril(np.ones((n, n)), -1)).flatten(order="F")
    b = B.flatten(order="F").copy()
    c = np.zeros(n * n)
    assert oracle.gevd_front(n, a, n, b, n, c) == 0
    L = np.linalg.cholesky(B)
    C_ref = np.linalg.solve(L, np.linalg.solve(L, A).T).T
    C = c.reshape(n, n, order="F")
    np.testing.assert_allclose(C, C_ref, rtol=0, atol=1e-12 * max(1.0, np.abs(C_ref).max()))
    np.testing.assert_allclose(b.reshape(n, n, order="F")[np.tril_indices(n)],
                               L[np.tril_indices(n)], rtol=0, atol=1e-12 * np.abs(L).max())
    w = sl.eigh(A, B, eigvals_only=True)
    np.testing.assert_allclose(np.linalg.eigvalsh(C), w, rtol=0, atol=1e-10 * max(1, np.abs(w).max()))


def test_gevd_front_not_positive_definite():
    n = 4
    a = np.eye(n).flatten(order="F")
    b = np.eye(n)
    b[2, 2] = -1.0
    b = b.flatten(order="F")
    c = np.zeros(n * n)
    assert oracle.gevd_front(n, a, n, b, n, c) == 3

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


def _upper_fill(A):
    """C as MatFlat's Complex GevdCore builds it from A's upper triangle: A above the diagonal,
    its conjugate transpose below, the diagonal as stored (Factorization.Gevd.cs:393-406)."""
    U = np.triu(A, 1)
    return U + U.conj().T + np.diag(np.diag(A))


@pytest.mark.parametrize("n", [1, 3, 17, 40])
def test_gevd_front_float_matches_lapack(n):
    sl = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(120 + n)
    A = rng.standard_normal((n, n))
    A = A + A.T
    M = rng.standard_normal((n, n))
    B = M @ M.T + n * np.eye(n)
    a = (np.triu(A) + 5.0 * np.tril(np.ones((n, n)), -1)).astype(np.float32).flatten(order="F")
    b = B.astype(np.float32).flatten(order="F")
    c = np.zeros(n * n, np.float32)
    assert oracle.gevd_front(n, a, n, b, n, c) == 0
    A32 = _upper_fill(a.reshape(n, n, order="F").astype(np.float64))
    L = np.linalg.cholesky(B.astype(np.float32).astype(np.float64))
    C_ref = np.linalg.solve(L, np.linalg.solve(L, A32).T).T
    C = c.reshape(n, n, order="F").astype(np.float64)
    np.testing.assert_allclose(C, C_ref, rtol=0, atol=2e-5 * max(1.0, np.abs(C_ref).max()))
    w = sl.eigh(A32, B.astype(np.float32).astype(np.float64), eigvals_only=True)
    np.testing.assert_allclose(np.linalg.eigvalsh(C), w, rtol=0, atol=1e-4 * max(1, np.abs(w).max()))


@pytest.mark.parametrize("n", [1, 2, 9, 33])
def test_gevd_front_complex_matches_lapack(n):
    sl = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(140 + n)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A = A + A.conj().T                          # Hermitian: a real diagonal
    M = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    B = M @ M.conj().T + n * np.eye(n)
    a = (np.triu(A) + (3.0 - 2.0j) * np.tril(np.ones((n, n)), -1)).flatten(order="F")
    b = B.flatten(order="F").copy()
    c = np.zeros(n * n, np.complex128)
    assert oracle.gevd_front(n, a, n, b, n, c) == 0
    L = np.linalg.cholesky(B)
    C_ref = np.linalg.solve(L, np.linalg.solve(L, A).conj().T).conj().T    # L^-1 A L^-H
    C = c.reshape(n, n, order="F")
    np.testing.assert_allclose(C, C_ref, rtol=0, atol=1e-12 * max(1.0, np.abs(C_ref).max()))
    np.testing.assert_allclose(b.reshape(n, n, order="F")[np.tril_indices(n)],
                               L[np.tril_indices(n)], rtol=0, atol=1e-12 * np.abs(L).max())
    w = sl.eigh(A, B, eigvals_only=True)
    np.testing.assert_allclose(np.linalg.eigvalsh(C), w, rtol=0, atol=1e-10 * max(1, np.abs(w).max()))


def test_gevd_front_complex_diagonal_as_stored():
    """A non-real diagonal of A is used as stored: MatFlat's row pass conjugates each row, solves
    and conjugates back, so the result is L^-1 C L^-H for C with that diagonal."""
    n = 6
    rng = np.random.default_rng(160)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    M = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    B = M @ M.conj().T + n * np.eye(n)
    a = A.flatten(order="F")
    b = B.flatten(order="F").copy()
    c = np.zeros(n * n, np.complex128)
    assert oracle.gevd_front(n, a, n, b, n, c) == 0
    L = np.linalg.cholesky(B)
    Cf = _upper_fill(A)
    C_ref = np.linalg.solve(L, Cf) @ np.linalg.inv(L).conj().T
    np.testing.assert_allclose(c.reshape(n, n, order="F"), C_ref, rtol=0, atol=1e-12 * np.abs(C_ref).max())


@pytest.mark.parametrize("dt", [np.float32, np.complex128])
def test_gevd_front_types_not_positive_definite(dt):
    n = 5
    a = np.eye(n).astype(dt).flatten(order="F")
    b = np.eye(n).astype(dt)
    b[3, 3] = -2.0
    b = b.flatten(order="F")
    c = np.zeros(n * n, dt)
    assert oracle.gevd_front(n, a, n, b, n, c) == 4


@pytest.mark.parametrize("dt", [np.float64, np.float32, np.complex128])
@pytest.mark.parametrize("n", [1, 2, 7, 33])
def test_gevd_row_form_is_matflats_order(dt, n):
    """The float / Complex GPU kernel runs MatFlat's two passes as row solves: D = conj(C), its
    rows solved, E = D^H, its rows solved, C = E^T.  Replayed here with the oracle's own
    SolveTriangular at stride n, the reformulation reproduces the oracle's GevdCore bit for bit
    (the stride and the order of the right-hand sides do not change any value)."""
    LOWER, NOTRANS = 122, 111
    rng = np.random.default_rng(180 + n)
    draw = (lambda *s: rng.standard_normal(s) + 1j * rng.standard_normal(s)) \
        if dt == np.complex128 else (lambda *s: rng.standard_normal(s))
    A = draw(n, n)
    M = draw(n, n)
    B = M @ M.conj().T + n * np.eye(n)
    a = A.astype(dt).flatten(order="F")
    b = B.astype(dt).flatten(order="F")
    ob, oc = b.copy(), np.zeros(n * n, dt)
    assert oracle.gevd_front(n, a, n, ob, n, oc) == 0
    lb = b.copy()
    assert oracle.cholesky(n, lb, n) == 0
    np.testing.assert_array_equal(lb.view(np.uint8), ob.view(np.uint8))
    Am = a.reshape(n, n, order="F")
    U = np.triu(Am, 1)
    C = U + U.conj().T + np.diag(np.diag(Am))           # MatFlat's C (diagonal as stored)
    D = np.asfortranarray(np.conj(C)).flatten(order="F")
    for r in range(n):                                   # rows of D, stride n
        seg = D[r:].copy()
        assert oracle.trsv(LOWER, NOTRANS, n, lb, n, seg, n) == 0
        D[r:] = seg
    E = np.asfortranarray(D.reshape(n, n, order="F").conj().T).flatten(order="F")
    for r in range(n):
        seg = E[r:].copy()
        assert oracle.trsv(LOWER, NOTRANS, n, lb, n, seg, n) == 0
        E[r:] = seg
    got = np.asfortranarray(E.reshape(n, n, order="F").T).flatten(order="F")
    np.testing.assert_array_equal(got.view(np.uint8), oc.view(np.uint8))

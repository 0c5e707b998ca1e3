"""CPU models of the evaluation orders the CUDA kernels use, against the oracle, bit for bit.

The kernels reorganise which lane computes what and when, never the operations that produce an
entry.  These models replay the kernels' schedules with scalar IEEE double arithmetic (numpy
scalars: every product and sum separately rounded, no FMA) and check that the reorganised
schedules give MatFlat's values, independently of the GPU:
  * Cholesky with split dots (potrf_group_split in csrc/chol.cu): each column's dots computed in
    two halves one step apart, at the pair boundary split_point(c);
  * LU in Crout order (csrc/lu.cu): step k finishes row k of U and column k+1 of L, with
    MatFlat's pivot rule (first index of the largest |v| among non-NaN entries; a NaN on the
    diagonal candidate is never displaced).
The FMA form's blocked LU for large orders (csrc/lu_big.cu) is a different arithmetic, so its
model is checked by what that form promises instead: MatFlat's pivots and sign where its screen
passes, a rejection where the choice could depend on rounding, a backward-stable factorization.
"""
import numpy as np
import pytest

from oracle import oracle

f64 = np.float64


def _dot(s, pairs):
    """Continues a MatFlat dot from partial sum s over the (x, y, x', y') pairs."""
    for xa, ya, xb, yb in pairs:
        s = f64(s + f64(f64(xa * ya) + f64(xb * yb)))
    return s


def _split_point(c):
    return ((c >> 1) | 1) if (c & 1) else ((c >> 1) & ~1)


def chol_split_model(a, n):
    """potrf_group_split's schedule on an n-by-n column-major array (lda = n); returns info."""
    A = [[f64(a[j * n + i]) for j in range(n)] for i in range(n)]   # A[i][j]
    Lm = [[f64(0.0)] * n for _ in range(n)]
    dsum = [f64(0.0)] * n
    full = [f64(0.0)] * n
    half = [[f64(0.0)] * n for _ in range(2)]
    for k in range(n):
        s = f64(A[k][k] - dsum[k])
        if not s > 0:
            return k + 1
        lkk = f64(np.sqrt(s))
        Lm[k][k] = lkk
        for j in range(k + 1, n):
            t = f64(f64(A[k][j] - full[j]) / lkk)
            Lm[j][k] = t
            dsum[j] = f64(dsum[j] + f64(t * t))
        c1, c2 = k + 1, k + 2
        h1, h2 = _split_point(c1), _split_point(c2)
        for j in range(c1 + 1, n):          # second halves of column c1
            if c1 == 1:
                s0, t0 = f64(Lm[j][0] * Lm[c1][0]), 1
            else:
                s0, t0 = half[c1 & 1][j], h1
            pairs = [(Lm[j][t], Lm[c1][t], Lm[j][t + 1], Lm[c1][t + 1]) for t in range(t0, c1, 2)]
            full[j] = _dot(s0, pairs)
        for j in range(c2 + 1, n):          # first halves of column c2
            t0 = c2 & 1
            s0 = f64(Lm[j][0] * Lm[c2][0]) if t0 else f64(0.0)
            pairs = [(Lm[j][t], Lm[c2][t], Lm[j][t + 1], Lm[c2][t + 1]) for t in range(t0, h2, 2)]
            half[c2 & 1][j] = _dot(s0, pairs)
    for j in range(n):
        for i in range(n):
            a[j * n + i] = Lm[i][j] if i >= j else 0.0
    return 0


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 8, 13, 24, 31])
def test_cholesky_split_schedule(n):
    rng = np.random.default_rng(500 + n)
    S = rng.standard_normal((n, n))
    A = S @ S.T + n * np.eye(n)
    a = A.flatten(order="F")
    got, exp = a.copy(), a.copy()
    assert chol_split_model(got, n) == 0
    assert oracle.cholesky(n, exp, n) == 0
    np.testing.assert_array_equal(got.view(np.uint64), exp.view(np.uint64))


def test_cholesky_split_schedule_failure():
    n = 6
    A = np.eye(n) * 4.0
    A[3, 3] = -1.0
    a = A.flatten(order="F")
    assert chol_split_model(a.copy(), n) == oracle.cholesky(n, a.copy(), n) == 4


def _pivot(v, j, m):
    """MatFlat's scan (Factorization.Lu.cs:323-330): p = j; p = i if |v_i| > |v_p|."""
    p = j
    for i in range(j + 1, m):
        if abs(v[i]) > abs(v[p]):
            p = i
    return p


def lu_crout_model(a, m, n):
    """Crout order on an m-by-n column-major array (lda = m); returns (piv, sign)."""
    A = [[f64(a[j * m + i]) for j in range(n)] for i in range(m)]
    piv = list(range(m))
    sign = 1
    mn = min(m, n)

    def dotk(i, j, k):                    # Dot(k, L(i, 0:k), U(0:k, j)) on the current rows
        s = f64(A[i][0] * A[0][j]) if (k & 1) else f64(0.0)
        t0 = k & 1
        return _dot(s, [(A[i][t], A[t][j], A[i][t + 1], A[t + 1][j]) for t in range(t0, k, 2)])

    for k in range(mn):
        # Column k of L (and U(k,k)): v(i,k) for i >= k, then the pivot, the swap and the scale.
        v = [None] * m
        for i in range(k, m):
            v[i] = f64(A[i][k] - dotk(i, k, k))
        p = _pivot(v, k, m)
        for i in range(k, m):
            A[i][k] = v[i]
        if p != k:
            A[p], A[k] = A[k], A[p]
            piv[p], piv[k] = piv[k], piv[p]
            sign = -sign
        d = A[k][k]
        if d != 0:
            for i in range(k + 1, m):
                A[i][k] = f64(A[i][k] / d)
        # Row k of U right of the diagonal: dots of length k against the final rows 0..k.
        for j in range(k + 1, n):
            A[k][j] = f64(A[k][j] - dotk(k, j, k))
    for j in range(n):
        for i in range(m):
            a[j * m + i] = A[i][j]
    return piv, sign


@pytest.mark.parametrize("m,n", [(1, 1), (2, 2), (3, 3), (5, 5), (9, 9), (16, 16), (23, 23),
                                 (7, 4), (4, 7)])
def test_lu_crout_schedule(m, n):
    rng = np.random.default_rng(600 + 31 * m + n)
    a = rng.standard_normal(m * n)
    if m * n > 8:
        a[5] = np.nan if m == 16 else a[5]          # a NaN in a candidate column
        a[m + 1] = 0.0
    got, exp = a.copy(), a.copy()
    piv_e = np.zeros(m, np.int32)
    sign_e = oracle.lu(m, n, exp, m, piv_e)
    piv_g, sign_g = lu_crout_model(got, m, n)
    np.testing.assert_array_equal(np.isnan(got), np.isnan(exp))
    np.testing.assert_array_equal(np.where(np.isnan(got), 0, got).view(np.uint64),
                                  np.where(np.isnan(exp), 0, exp).view(np.uint64))
    np.testing.assert_array_equal(piv_g, piv_e)
    assert sign_g == sign_e


def test_lu_crout_schedule_singular():
    """MatFlat's literal singular fixture (LuTests.cs:173): 1..9 row-major."""
    a = np.arange(1.0, 10.0).reshape(3, 3).flatten(order="F")
    got, exp = a.copy(), a.copy()
    piv_e = np.zeros(3, np.int32)
    sign_e = oracle.lu(3, 3, exp, 3, piv_e)
    piv_g, sign_g = lu_crout_model(got, 3, 3)
    np.testing.assert_array_equal(got.view(np.uint64), exp.view(np.uint64))
    np.testing.assert_array_equal(piv_g, piv_e)
    assert sign_g == sign_e


# The FMA form's pivot screen (LU_FMA_MARGIN_ULPS in csrc/mf_lu.cuh): the pivot's |v| bits must
# exceed every other candidate's by 2^26 units in the last place.
MARGIN_ULPS = 1 << 26


def lu_blocked_model(A, nb=32):
    """The blocked right-looking schedule of getrf_big_fma_kernel on an n-by-n array (numpy
    float64, separately rounded products and sums instead of fused ones): per panel of nb columns,
    each column's pivot search with the screen, the whole-row swap, reciprocal scaling and the
    rank-1 update of the panel's later columns; then U12 = L11^-1 A12 and A22 -= L21 U12.
    Returns (factors, piv, sign) or None when a column fails the screen."""
    from scipy.linalg import solve_triangular
    a = np.array(A, dtype=np.float64)
    n = a.shape[0]
    piv = np.arange(n)
    sign = 1
    for j0 in range(0, n, nb):
        j1 = min(n, j0 + nb)
        for j in range(j0, j1):
            col = a[j:, j]
            if not np.isfinite(col).all():
                return None
            keys = np.abs(col).view(np.uint64).astype(np.int64)
            p = int(np.argmax(keys))
            second = np.max(np.delete(keys, p)) if len(keys) > 1 else 0
            if keys[p] == 0 or keys[p] - second < MARGIN_ULPS:
                return None
            p += j
            if p != j:
                a[[j, p], :] = a[[p, j], :]
                piv[[j, p]] = piv[[p, j]]
                sign = -sign
            r = 1.0 / a[j, j]
            a[j + 1:, j] *= r
            a[j + 1:, j + 1:j1] -= np.outer(a[j + 1:, j], a[j, j + 1:j1])
        if j1 < n:
            a[j0:j1, j1:] = solve_triangular(a[j0:j1, j0:j1], a[j0:j1, j1:], lower=True,
                                             unit_diagonal=True, check_finite=False)
            a[j1:, j1:] -= a[j1:, j0:j1] @ a[j0:j1, j1:]
    return a, piv, sign


@pytest.mark.parametrize("n", [40, 129, 200, 333])
def test_lu_blocked_schedule_pivots(n):
    """Random N(0,1) matrices: the screen passes and the pivots and sign are MatFlat's; the
    factors reproduce PA to a normwise backward error within 1e-13 n."""
    rng = np.random.default_rng(700 + n)
    A = rng.standard_normal((n, n))
    out = lu_blocked_model(A)
    assert out is not None
    F, piv, sign = out
    exp = A.flatten(order="F")
    piv_e = np.zeros(n, np.int32)
    sign_e = oracle.lu(n, n, exp, n, piv_e)
    np.testing.assert_array_equal(piv, piv_e)
    assert sign == sign_e
    L = np.tril(F, -1) + np.eye(n)
    U = np.triu(F)
    assert np.linalg.norm(A[piv, :] - L @ U, 1) / np.linalg.norm(A, 1) <= 1e-13 * n


def test_lu_blocked_schedule_screen():
    """A near-tie (runner-up within 2^26 ulps), an exact tie in a later panel's column, a NaN and
    a zero column are rejected; a clear gap passes."""
    rng = np.random.default_rng(710)
    base = rng.standard_normal((100, 100))
    near = base.copy()
    near[5, 0], near[9, 0] = 50.0, -50.0 * (1.0 + 2.0 ** -45)
    assert lu_blocked_model(near) is None
    tie = base.copy()
    tie[60, 40] = tie[70, 40] = 1e6
    tie[60, :40] = tie[70, :40] = 0.0   # zero multipliers: no update reaches them, an exact tie
    assert lu_blocked_model(tie) is None
    nan = base.copy()
    nan[30, 70] = np.nan
    assert lu_blocked_model(nan) is None
    zero = base.copy()
    zero[:, 0] = 0.0
    assert lu_blocked_model(zero) is None
    clear = base.copy()
    clear[5, 0], clear[9, 0] = 50.0, -49.0
    assert lu_blocked_model(clear) is not None

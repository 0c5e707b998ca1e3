"""The study behind the decision not to build a certified-pivot FMA form of the LU (the north
star's plain form must reproduce MatFlat's pivots): a pivot certificate compares the chosen
candidate |v_p| - beta_p with every other |v_i| + beta_i, beta bounding the difference between
MatFlat's candidate and an FMA-order computation's.  From the exact identity for the Schur
complements of the two perturbed matrices B = PA + E, B' = PA + E_M,
    s(B) - s(B') = D22 - D21 X' - Y (D12 - D11 X'),   Y = L21 L11^-1,  X = U11^-1 U12,
|D| <= g (2|PA| + 2|L||U|).  This CPU test reruns the study on a small sample and checks what the
design relies on: the first-order elementwise bound (|Y| <= |l| |L11^-1|) is small enough to
certify random matrices of the batch's orders, the normwise bound is orders of magnitude looser,
and comparison-matrix (interval-style) inverse bounds explode."""
import numpy as np
from scipy.linalg import solve_triangular

U_ROUND = 2.0 ** -53


def _gepp(a):
    """Right-looking partial pivoting (first index of the largest |v|), the candidate columns."""
    n = a.shape[0]
    w = a.copy()
    perm = np.arange(n)
    cand = []
    for j in range(n):
        p = j + int(np.argmax(np.abs(w[j:, j])))
        if p != j:
            w[[j, p]] = w[[p, j]]
            perm[[j, p]] = perm[[p, j]]
        cand.append(w[j:, j].copy())
        w[j + 1:, j] = w[j + 1:, j] / w[j, j]
        w[j + 1:, j + 1:] -= np.outer(w[j + 1:, j], w[j, j + 1:])
    return w, perm, cand


def _bounds(a):
    n = a.shape[0]
    w, perm, cand = _gepp(a)
    L = np.tril(w, -1) + np.eye(n)
    U = np.triu(w)
    g = (n + 2) * U_ROUND / (1 - (n + 2) * U_ROUND)
    D = g * (2 * np.abs(a[perm]) + 2 * np.abs(L) @ np.abs(U))
    AL = np.abs(np.linalg.inv(L))
    AU = np.abs(np.linalg.inv(U))
    elem = norm = 0.0
    margin = np.inf
    for j in range(1, n):
        X = np.abs(np.linalg.inv(U)[:j, j] * U[j, j])
        wv = D[:j, j] + D[:j, :j] @ X
        be = D[j:, j] + D[j:, :j] @ X + np.abs(L[j:, :j]) @ (AL[:j, :j] @ wv)
        xn = AU[:j, :j].sum(1).max() * np.abs(U[:j, j]).max()
        wn = D[:j, j].max() + D[:j, :j].sum(1).max() * xn
        bn = D[j:, j] + D[j:, :j].sum(1) * xn + np.abs(L[j:, :j]).sum(1) * AL[:j, :j].sum(
            1).max() * wn
        v = np.abs(cand[j])
        vp = v[0]
        elem = max(elem, be.max() / vp)
        norm = max(norm, bn.max() / vp)
        if v.size > 1:
            margin = min(margin, (vp - be[0] - (v[1:] + be[1:]).max()) / vp)
    ML = -np.abs(L)
    np.fill_diagonal(ML, 1.0)
    interval = solve_triangular(ML, np.ones(n), lower=True).max()
    return elem, norm, margin, interval


def test_certificate_bounds_on_random_matrices():
    rng = np.random.default_rng(5)
    elems, norms, margins, intervals = [], [], [], []
    for n in (24, 64, 96, 128, 128):
        e, nb, m, iv = _bounds(rng.standard_normal((n, n)))
        elems.append(e)
        norms.append(nb)
        margins.append(m)
        intervals.append(iv)
    assert max(elems) < 1e-5                      # first-order elementwise: tight
    assert min(margins) > 0                       # every column certified
    assert min(n / e for n, e in zip(norms, elems)) > 10   # normwise: much looser
    assert intervals[-1] > 1e10                   # interval-style inverse bound at n = 128

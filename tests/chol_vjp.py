"""FP64 reference of the reverse mode of (L = Cholesky(A), log det A, x = A^-1 b), built from the
oracle's factor (MatFlat's Cholesky arithmetic) with numpy / scipy triangular solves.  Test
infrastructure: the GPU backward pass is compared with it, and it is itself checked against
central finite differences in tests/test_oracle_grad.py."""
import numpy as np
from scipy.linalg import solve_triangular

from oracle import oracle


def oracle_factor(A):
    n = A.shape[0]
    a = A.reshape(-1, order="F").copy()
    info = oracle.cholesky(n, a, n)
    return info, np.tril(a.reshape(n, n, order="F"))


def vjp(L, lbar, logdet_bar, x, xbar):
    """abar = sym(L^-T Phi(L^T lbar) L^-1) + logdet_bar A^-1 - sym(bbar x^T), bbar = A^-1 xbar."""
    n = L.shape[0]
    X = L.T @ np.tril(lbar)
    P = np.tril(X) - 0.5 * np.diag(np.diag(X)) + logdet_bar * np.eye(n)
    S = 0.5 * (P + P.T)
    Y = solve_triangular(L, S.T, lower=True, trans=1).T          # S L^-1  (L^T Y^T = S^T)
    G = solve_triangular(L, Y, lower=True, trans=1)               # L^-T Y
    bbar = np.zeros(n)
    if xbar is not None:
        z = solve_triangular(L, xbar, lower=True)
        bbar = solve_triangular(L, z, lower=True, trans=1)
        G = G - 0.5 * (np.outer(bbar, x) + np.outer(x, bbar))
    return 0.5 * (G + G.T), bbar


def objective(A, lbar, logdet_bar, b, xbar):
    """<lbar, L(A)> + logdet_bar log det A + <xbar, A^-1 b>, with numpy's Cholesky."""
    L = np.linalg.cholesky(A)
    f = np.sum(np.tril(lbar) * L) + logdet_bar * 2.0 * np.sum(np.log(np.diag(L)))
    if xbar is not None:
        f += xbar @ np.linalg.solve(A, b)
    return f

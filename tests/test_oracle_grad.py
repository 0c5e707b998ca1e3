"""The oracle's gradient of loss = y^T K^-1 y + log det K (composed from MatFlat's routines)
against the closed form K^-1 - alpha alpha^T and against central finite differences (h = 1e-6)."""
import numpy as np

from oracle import oracle
from workloads import synth


def _loss_grad(K, y):
    n = K.shape[0]
    k = K.reshape(-1, order="F").copy()
    yy = y.copy()
    g = np.zeros(n * n)
    info, loss = oracle.chol_grad(n, k, n, yy, g)
    return info, loss, g.reshape(n, n, order="F"), yy


def _fd(K, y, i, j, h=1e-6):
    E = np.zeros_like(K)
    E[i, j] = 1.0
    E[j, i] = 1.0
    lp = _loss_grad(K + h * E, y)[1]
    lm = _loss_grad(K - h * E, y)[1]
    return (lp - lm) / (2 * h)


def test_grad_matches_closed_form_and_fd_well_conditioned():
    rng = np.random.default_rng(4)
    for n in (1, 2, 5, 16, 33):
        b = rng.standard_normal((n, n))
        K = b @ b.T + n * np.eye(n)
        y = rng.standard_normal(n)
        info, loss, G, alpha = _loss_grad(K, y)
        assert info == 0
        Kinv = np.linalg.inv(K)
        a = Kinv @ y
        assert abs(loss - (y @ a + np.linalg.slogdet(K)[1])) <= 1e-12 * max(1.0, abs(loss))
        np.testing.assert_allclose(alpha, a, rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(G, Kinv - np.outer(a, a), rtol=1e-11, atol=1e-14)
        assert np.array_equal(G, G.T)
        for (i, j) in [(0, 0), (n - 1, 0), (n // 2, n // 3)]:
            an = G[i, j] * (1 if i == j else 2)      # symmetric perturbation of (i,j) and (j,i)
            assert abs(_fd(K, y, i, j) - an) <= 1e-6 * max(1.0, abs(an))


def test_grad_rbf_configuration():
    """The benchmark's RBF kernel matrices (n = 128, length 0.3, jitter 1e-6) are ill-conditioned
    (cond ~1e6-1e8): the gradient still matches the closed form, and central differences with
    h = 1e-6 agree to the accuracy such conditioning allows."""
    d = synth.rbf_batch(2, 128, seed=7)
    for m in range(2):
        K = d["a"][d["a_off"][m]:d["a_off"][m] + 128 * 128].reshape(128, 128, order="F")
        y = d["b"][d["b_off"][m]:d["b_off"][m] + 128]
        info, loss, G, _ = _loss_grad(K, y)
        assert info == 0
        Kinv = np.linalg.inv(K)
        a = Kinv @ y
        exact = Kinv - np.outer(a, a)
        assert np.max(np.abs(G - exact)) <= 1e-8 * np.max(np.abs(exact))
        for (i, j) in [(0, 0), (5, 3), (127, 64)]:
            an = G[i, j] * (1 if i == j else 2)
            assert abs(_fd(K, y, i, j) - an) <= 1e-2 * abs(an)


def test_non_pd_reports_info():
    K = np.array([[1.0, 2.0], [2.0, 1.0]])
    info, loss, _, _ = _loss_grad(K, np.ones(2))
    assert info == 2 and np.isnan(loss)


def test_reverse_mode_reference_matches_finite_differences():
    """The FP64 reference VJP of (Cholesky factor, log det, solve) used by the GPU backward tests
    agrees with central differences (h = 1e-6) along random symmetric directions."""
    from tests.chol_vjp import oracle_factor, objective, vjp
    rng = np.random.default_rng(21)
    for n in (1, 3, 8, 24):
        B = rng.standard_normal((n, n))
        A = B @ B.T + n * np.eye(n)
        b = rng.standard_normal(n)
        lbar = np.tril(rng.standard_normal((n, n)))
        ldb = rng.standard_normal()
        xbar = rng.standard_normal(n)
        info, L = oracle_factor(A)
        assert info == 0
        x = np.linalg.solve(A, b)
        G, bbar = vjp(L, lbar, ldb, x, xbar)
        np.testing.assert_allclose(bbar, np.linalg.solve(A, xbar), rtol=1e-10, atol=1e-12)
        for _ in range(3):
            E = rng.standard_normal((n, n))
            E = E + E.T
            h = 1e-6
            fd = (objective(A + h * E, lbar, ldb, b, xbar) -
                  objective(A - h * E, lbar, ldb, b, xbar)) / (2 * h)
            an = np.sum(G * E)
            assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (n, fd, an)


def test_reverse_mode_reference_reduces_to_the_loss_gradient():
    """With lbar = 0, logdet_bar = 1, xbar = y and x = alpha, the VJP is the loss gradient
    K^-1 - alpha alpha^T of the oracle's composition."""
    from tests.chol_vjp import oracle_factor, vjp
    rng = np.random.default_rng(22)
    n = 20
    B = rng.standard_normal((n, n))
    K = B @ B.T + n * np.eye(n)
    y = rng.standard_normal(n)
    info, loss, G, alpha = _loss_grad(K, y)
    _, L = oracle_factor(K)
    V, _ = vjp(L, np.zeros((n, n)), 1.0, alpha, y)
    np.testing.assert_allclose(V, G, rtol=1e-10, atol=1e-13)

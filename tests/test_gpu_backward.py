"""The reverse mode of Cholesky / log-determinant / solve on the GPU (mfg_dpotrf_backward_batched)
against the FP64 reference VJP built from the oracle's factor (tests/chol_vjp.py, itself pinned by
central differences), for random cotangents; the recomputed factor is bit-identical to the
forward kernel's; with the loss's cotangents it reproduces the fused loss gradient."""
import numpy as np
import pytest

from tests.chol_vjp import oracle_factor, vjp

pytestmark = pytest.mark.gpu


def _batch(rng, ns, cond_boost=True):
    mats, offs, boffs = [], [], []
    off = boff = 0
    for n in ns:
        B = rng.standard_normal((n, n))
        A = B @ B.T + (n if cond_boost else 1e-3) * np.eye(n)
        mats.append(A)
        offs.append(off)
        boffs.append(boff)
        off += n * n
        boff += n
    return mats, np.array(offs, np.int64), np.array(boffs, np.int64), off, boff


def _flat(mats):
    return np.concatenate([m.reshape(-1, order="F") for m in mats])


@pytest.mark.parametrize("recompute", [True, False])
def test_backward_matches_reference_vjp(mf, recompute):
    import torch
    rng = np.random.default_rng(31)
    ns = [1, 2, 5, 17, 31, 64, 100, 128]
    mats, a_off, b_off, total, btotal = _batch(rng, ns)
    lbars = [np.tril(rng.standard_normal((n, n))) for n in ns]
    ldbar = rng.standard_normal(len(ns))
    bs = [rng.standard_normal(n) for n in ns]
    xs = [np.linalg.solve(A, b) for A, b in zip(mats, bs)]
    xbars = [rng.standard_normal(n) for n in ns]
    plan = mf.CholeskyBatch(np.array(ns, np.int32), a_off, nrhs=1, b_off=b_off)
    a = torch.from_numpy(_flat(mats)).cuda()
    info = torch.zeros(len(ns), dtype=torch.int32, device="cuda")
    if not recompute:
        scratch_b = torch.zeros(btotal, dtype=torch.float64, device="cuda")
        plan.run(a, scratch_b, info)
    lbar = torch.from_numpy(_flat(lbars)).cuda()
    abar = torch.zeros(total, dtype=torch.float64, device="cuda")
    bbar = torch.zeros(btotal, dtype=torch.float64, device="cuda")
    plan.backward(a, abar, info, lbar=lbar, logdet_bar=torch.from_numpy(ldbar).cuda(),
                  x=torch.from_numpy(np.concatenate(xs)).cuda(),
                  xbar=torch.from_numpy(np.concatenate(xbars)).cuda(), bbar=bbar,
                  recompute=recompute)
    mf.context().synchronize()
    g = abar.cpu().numpy()
    gb = bbar.cpu().numpy()
    lf = a.cpu().numpy()
    assert (info.cpu().numpy() == 0).all()
    for m, n in enumerate(ns):
        _, L = oracle_factor(mats[m])
        # the factor the backward used is MatFlat's, bit for bit
        np.testing.assert_array_equal(np.tril(lf[a_off[m]:a_off[m] + n * n].reshape(n, n, order="F"))
                                      .view(np.uint64), L.view(np.uint64))
        G, bb = vjp(L, lbars[m], ldbar[m], xs[m], xbars[m])
        got = g[a_off[m]:a_off[m] + n * n].reshape(n, n, order="F")
        scale = np.max(np.abs(G))
        assert np.max(np.abs(got - G)) <= 1e-11 * n * scale, (n, np.max(np.abs(got - G)), scale)
        np.testing.assert_array_equal(got, got.T)
        np.testing.assert_allclose(gb[b_off[m]:b_off[m] + n], bb, rtol=1e-10,
                                   atol=1e-12 * np.max(np.abs(bb)))


def test_backward_fma_form(mf):
    """A Cholesky plan in the FMA form recomputes its factor in that form; the reverse pass then
    matches the FP64 reference VJP built from that factor, and the factor is a backward-stable
    Cholesky factor of A."""
    import torch
    rng = np.random.default_rng(33)
    ns = [1, 3, 17, 64, 100, 128]
    mats, a_off, b_off, total, btotal = _batch(rng, ns)
    lbars = [np.tril(rng.standard_normal((n, n))) for n in ns]
    ldbar = rng.standard_normal(len(ns))
    bs = [rng.standard_normal(n) for n in ns]
    xs = [np.linalg.solve(A, b) for A, b in zip(mats, bs)]
    xbars = [rng.standard_normal(n) for n in ns]
    plan = mf.CholeskyBatch(np.array(ns, np.int32), a_off, nrhs=1, b_off=b_off)
    plan.set_form("fma")
    a = torch.from_numpy(_flat(mats)).cuda()
    info = torch.zeros(len(ns), dtype=torch.int32, device="cuda")
    abar = torch.zeros(total, dtype=torch.float64, device="cuda")
    bbar = torch.zeros(btotal, dtype=torch.float64, device="cuda")
    plan.backward(a, abar, info, lbar=torch.from_numpy(_flat(lbars)).cuda(),
                  logdet_bar=torch.from_numpy(ldbar).cuda(),
                  x=torch.from_numpy(np.concatenate(xs)).cuda(),
                  xbar=torch.from_numpy(np.concatenate(xbars)).cuda(), bbar=bbar, recompute=True)
    mf.context().synchronize()
    g, gb, lf = abar.cpu().numpy(), bbar.cpu().numpy(), a.cpu().numpy()
    assert (info.cpu().numpy() == 0).all()
    for m, n in enumerate(ns):
        L = np.tril(lf[a_off[m]:a_off[m] + n * n].reshape(n, n, order="F"))
        A = mats[m]
        assert np.linalg.norm(A - L @ L.T, 1) / np.linalg.norm(A, 1) <= 1e-13 * n
        G, bb = vjp(L, lbars[m], ldbar[m], xs[m], xbars[m])
        got = g[a_off[m]:a_off[m] + n * n].reshape(n, n, order="F")
        scale = np.max(np.abs(G))
        assert np.max(np.abs(got - G)) <= 1e-11 * n * scale, (n, np.max(np.abs(got - G)), scale)
        np.testing.assert_allclose(gb[b_off[m]:b_off[m] + n], bb, rtol=1e-10,
                                   atol=1e-12 * np.max(np.abs(bb)))


def test_backward_reproduces_loss_gradient(mf):
    """lbar = 0, logdet_bar = 1, xbar = y, x = alpha: the gradient of y^T K^-1 y + log det K, as
    the fused loss-and-gradient entry point computes it."""
    import torch
    from workloads import synth
    d = synth.rbf_batch(6, 64, seed=12)
    n = d["n"]
    plan = mf.CholeskyBatch(n, d["a_off"], nrhs=1, b_off=d["b_off"])
    k = torch.from_numpy(d["a"].copy()).cuda()
    y = torch.from_numpy(d["b"].copy()).cuda()
    loss = torch.zeros(len(n), dtype=torch.float64, device="cuda")
    grad = torch.zeros_like(k)
    info = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    plan.loss_and_grad(k, y, loss, grad, info, keep_factor=False)     # y <- alpha
    a = torch.from_numpy(d["a"].copy()).cuda()
    abar = torch.zeros_like(a)
    ones = torch.ones(len(n), dtype=torch.float64, device="cuda")
    yb = torch.from_numpy(d["b"].copy()).cuda()
    plan.backward(a, abar, info, logdet_bar=ones, x=y, xbar=yb, recompute=True)
    mf.context().synchronize()
    g0 = grad.cpu().numpy()
    g1 = abar.cpu().numpy()
    scale = np.max(np.abs(g0))
    # RBF kernels at n = 64 are ill-conditioned: both are K^-1 - alpha alpha^T to ~cond * eps
    assert np.max(np.abs(g1 - g0)) <= 1e-6 * scale


def test_backward_reports_non_pd(mf):
    import torch
    n = 4
    A = np.eye(n)
    A[2, 2] = -1.0
    plan = mf.CholeskyBatch(np.array([n], np.int32), np.array([0], np.int64))
    a = torch.from_numpy(A.reshape(-1, order="F").copy()).cuda()
    abar = torch.zeros_like(a)
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    plan.backward(a, abar, info, logdet_bar=torch.ones(1, dtype=torch.float64, device="cuda"))
    mf.context().synchronize()
    assert info.cpu().numpy()[0] == 3

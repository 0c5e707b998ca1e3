"""Differentiable Cholesky / log-det / solve on the GPU against the oracle (bit for bit for the
factor, alpha and the gradient; the loss to 1e-14 because log() differs between libm's)."""
import numpy as np
import pytest

from oracle import oracle
from workloads import synth

pytestmark = pytest.mark.gpu


def _bits_equal(got, exp, msg=""):
    gn, en = np.isnan(got), np.isnan(exp)
    np.testing.assert_array_equal(gn, en, err_msg=msg)
    np.testing.assert_array_equal(np.where(gn, 0, got).view(np.uint64),
                                  np.where(en, 0, exp).view(np.uint64), err_msg=msg)


@pytest.mark.parametrize("keep_factor", [True, False])
def test_grad_batched_matches_oracle(mf, keep_factor):
    import torch
    rng = np.random.default_rng(21)
    n = rng.integers(1, 129, size=64).astype(np.int32)
    n[:3] = [1, 2, 128]
    mats = []
    for i, ni in enumerate(n):
        b = rng.standard_normal((ni, ni))
        s = b @ b.T + ni * np.eye(ni)
        if i == 9:
            s[1, 1] = -5.0                          # not positive definite
        mats.append(s.reshape(-1, order="F"))
    sz = n.astype(np.int64) ** 2
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]])
    a = np.concatenate(mats)
    b_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]])
    y = rng.standard_normal(int(n.sum()))

    batch = mf.CholeskyBatch(n, a_off, nrhs=1, b_off=b_off)
    dk = torch.from_numpy(a.copy()).cuda()
    dy = torch.from_numpy(y.copy()).cuda()
    dloss = torch.zeros(len(n), dtype=torch.float64, device="cuda")
    dgrad = torch.zeros_like(dk)
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    batch.loss_and_grad(dk, dy, dloss, dgrad, dinfo, keep_factor=keep_factor)
    mf.context().synchronize()

    ok, oy, og = a.copy(), y.copy(), np.zeros_like(a)
    oloss = np.zeros(len(n))
    oinfo = np.zeros(len(n), np.int32)
    oracle.chol_grad_batched(n, a_off, ok, b_off, oy, oloss, og, oinfo, 4)

    gk, gy, gg, gl, gi = (t.cpu().numpy() for t in (dk, dy, dgrad, dloss, dinfo))
    np.testing.assert_array_equal(gi, oinfo)
    assert oinfo[9] != 0
    for i in range(len(n)):
        if oinfo[i] != 0:
            assert np.isnan(gl[i])
            continue
        sl = slice(a_off[i], a_off[i] + sz[i])
        _bits_equal(gg[sl], og[sl], "grad %d" % i)
        if keep_factor:
            _bits_equal(gk[sl], ok[sl], "factor %d" % i)
        else:
            _bits_equal(gk[sl], a[sl], "k untouched %d" % i)
        _bits_equal(gy[b_off[i]:b_off[i] + n[i]], oy[b_off[i]:b_off[i] + n[i]], "alpha %d" % i)
        assert abs(gl[i] - oloss[i]) <= 1e-14 * max(1.0, abs(oloss[i])), i


def test_grad_rbf_central_differences(mf):
    """Gradient of the RBF configuration against central finite differences (h = 1e-6) taken
    through the GPU's own loss."""
    import torch
    d = synth.rbf_batch(1, 128, seed=3)
    K = d["a"].reshape(128, 128, order="F")
    y = d["b"]
    batch = mf.CholeskyBatch(d["n"], d["a_off"], nrhs=1, b_off=d["b_off"])

    def run(Kx):
        dk = torch.from_numpy(Kx.reshape(-1, order="F").copy()).cuda()
        dy = torch.from_numpy(y.copy()).cuda()
        dl = torch.zeros(1, dtype=torch.float64, device="cuda")
        dg = torch.zeros_like(dk)
        di = torch.zeros(1, dtype=torch.int32, device="cuda")
        batch.loss_and_grad(dk, dy, dl, dg, di, keep_factor=False)
        mf.context().synchronize()
        return float(dl.cpu()[0]), dg.cpu().numpy().reshape(128, 128, order="F")

    loss, G = run(K)
    h = 1e-6
    for (i, j) in [(0, 0), (7, 2), (100, 99)]:
        E = np.zeros_like(K)
        E[i, j] = 1.0
        E[j, i] = 1.0
        fd = (run(K + h * E)[0] - run(K - h * E)[0]) / (2 * h)
        an = G[i, j] * (1 if i == j else 2)
        assert abs(fd - an) <= 1e-2 * abs(an), (i, j, fd, an)


@pytest.mark.parametrize("keep_factor", [True, False])
def test_grad_structured_zeros(mf, keep_factor):
    """Exact zeros in L^-1, K^-1 and alpha (diagonal, block-diagonal and arrow matrices, y with
    zeros): the gradient's signed zeros match the oracle bit for bit."""
    import torch
    rng = np.random.default_rng(22)
    n = np.array([5, 33, 64, 97, 128, 7], np.int32)
    mats, ys = [], []
    for i, ni in enumerate(n):
        if i % 3 == 0:
            s = np.diag(rng.uniform(1.0, 3.0, ni))
        elif i % 3 == 1:
            s = np.zeros((ni, ni))
            h = ni // 2
            for lo, hi in ((0, h), (h, ni)):
                b = rng.standard_normal((hi - lo, hi - lo))
                s[lo:hi, lo:hi] = b @ b.T + (hi - lo) * np.eye(hi - lo)
        else:
            s = np.eye(ni) * ni
            s[0, 1:] = s[1:, 0] = rng.choice([-1.0, 0.0, 1.0], ni - 1)
        mats.append(s.reshape(-1, order="F"))
        yy = rng.standard_normal(ni)
        yy[rng.random(ni) < 0.3] = 0.0
        yy[rng.random(ni) < 0.1] = -0.0
        ys.append(yy)
    sz = n.astype(np.int64) ** 2
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]])
    a = np.concatenate(mats)
    b_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]])
    y = np.concatenate(ys)
    batch = mf.CholeskyBatch(n, a_off, nrhs=1, b_off=b_off)
    dk = torch.from_numpy(a.copy()).cuda()
    dy = torch.from_numpy(y.copy()).cuda()
    dloss = torch.zeros(len(n), dtype=torch.float64, device="cuda")
    dgrad = torch.zeros_like(dk)
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    batch.loss_and_grad(dk, dy, dloss, dgrad, dinfo, keep_factor=keep_factor)
    mf.context().synchronize()
    ok, oy, og = a.copy(), y.copy(), np.zeros_like(a)
    oloss = np.zeros(len(n))
    oinfo = np.zeros(len(n), np.int32)
    oracle.chol_grad_batched(n, a_off, ok, b_off, oy, oloss, og, oinfo, 1)
    assert (oinfo == 0).all()
    gg = dgrad.cpu().numpy()
    assert (og == 0).any()
    for i in range(len(n)):
        sl = slice(a_off[i], a_off[i] + sz[i])
        _bits_equal(gg[sl], og[sl], "grad %d" % i)

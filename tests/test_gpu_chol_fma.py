"""The FMA form of the batched Cholesky (mfg_plan_set_form(MFG_FORM_FMA)): fused multiply-adds in
any order, so the factors are not MatFlat's bits; checked by what the form promises instead:
normwise backward error of the factor and of the solution within 1e-13 * n, the same info as
MatFlat (the oracle) on clearly indefinite matrices, a cleared strict upper triangle, and the
exact form unchanged on the same plan afterwards."""
import numpy as np
import pytest

from oracle import oracle
from tests.test_gpu_parity import _dev, _host, assert_bits

pytestmark = pytest.mark.gpu


def _batch(rng, count, nmax=140, bad_every=0):
    n = rng.integers(1, nmax + 1, size=count).astype(np.int32)
    mats = []
    for i, ni in enumerate(n):
        bm = rng.standard_normal((ni, ni))
        s = bm @ bm.T + ni * np.eye(ni)
        if bad_every and i % bad_every == 3 and ni > 2:
            s[ni // 2, ni // 2] = -1.0      # not positive definite at column ni // 2
        mats.append(np.asfortranarray(s).reshape(-1, order="F"))
    sz = n.astype(np.int64) ** 2
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    b_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]]).astype(np.int64)
    return n, a_off, b_off, np.concatenate(mats), rng.standard_normal(int(n.sum()))


@pytest.mark.parametrize("table", [0, 2])
def test_cholesky_fma_backward_error(mf, table, monkeypatch):
    import torch
    monkeypatch.setenv("MFG_CHOL_TABLE", str(table))
    rng = np.random.default_rng(70 + table)
    n, a_off, b_off, a, b = _batch(rng, 600, bad_every=41)
    batch = mf.CholeskyBatch(n, a_off, nrhs=1, b_off=b_off)
    batch.set_form("fma")
    da, db = _dev(a), _dev(b)
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    batch.run(da, db, dinfo)
    mf.context().synchronize()
    oa, ob = a.copy(), b.copy()
    oinfo = np.zeros(len(n), np.int32)
    oracle.chol_solve_batched(n, a_off, oa, b_off, ob, oinfo, 4)
    ginfo = _host(dinfo)
    np.testing.assert_array_equal(ginfo, oinfo)
    assert (oinfo != 0).any()
    ga, gb = _host(da), _host(db)
    worst_f, worst_x, differs = 0.0, 0.0, 0
    for i in range(len(n)):
        if oinfo[i] != 0:
            continue
        ni = int(n[i])
        sl = slice(a_off[i], a_off[i] + ni * ni)
        A = a[sl].reshape(ni, ni, order="F")
        L = ga[sl].reshape(ni, ni, order="F")
        assert not np.triu(L, 1).any(), "strict upper triangle must be cleared (matrix %d)" % i
        ef = np.linalg.norm(A - L @ L.T, 1) / np.linalg.norm(A, 1)
        x = gb[b_off[i]:b_off[i] + ni]
        bi = b[b_off[i]:b_off[i] + ni]
        ex = np.linalg.norm(bi - A @ x, 1) / (np.linalg.norm(A, 1) * np.linalg.norm(x, 1) +
                                              np.linalg.norm(bi, 1))
        assert ef <= 1e-13 * ni, (i, ni, ef)
        assert ex <= 1e-13 * ni, (i, ni, ex)
        worst_f, worst_x = max(worst_f, ef / ni), max(worst_x, ex / ni)
        differs += int(not np.array_equal(ga[sl], oa[sl]))
    # the form is a different arithmetic: most factors differ from MatFlat's in the last bits
    assert differs > 0
    # a solve-only call on the FMA factors gives the fused call's solutions bit for bit
    db2 = _dev(b)
    torch.cuda.synchronize()
    batch.solve(da, db2)
    mf.context().synchronize()
    ok = oinfo == 0
    for i in np.nonzero(ok)[0][::5]:
        sl = slice(b_off[i], b_off[i] + int(n[i]))
        assert_bits(_host(db2)[sl], gb[sl], "solve-only, matrix %d" % i)
    # switching the plan back gives MatFlat's bits again
    batch.set_form("exact")
    da, db = _dev(a), _dev(b)
    batch.run(da, db, dinfo)
    mf.context().synchronize()
    ga, gb = _host(da), _host(db)
    for i in range(0, len(n), 7):
        if oinfo[i] == 0:
            sl = slice(a_off[i], a_off[i] + int(n[i]) ** 2)
            assert_bits(ga[sl], oa[sl], "matrix %d" % i)


def test_cholesky_fma_autotune(mf):
    """The autotuner times the FMA kernel for an FMA plan, and the tuned plan keeps the form."""
    import torch
    rng = np.random.default_rng(77)
    n, a_off, b_off, a, b = _batch(rng, 1500, nmax=128)
    batch = mf.CholeskyBatch(n, a_off, nrhs=1, b_off=b_off)
    batch.set_form("fma")
    cfg = batch.autotune()
    assert cfg[3] == 0
    da, db = _dev(a), _dev(b)
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    batch.run(da, db, dinfo)
    mf.context().synchronize()
    assert not _host(dinfo).any()
    ga = _host(da)
    for i in range(0, len(n), 11):
        ni = int(n[i])
        sl = slice(a_off[i], a_off[i] + ni * ni)
        A = a[sl].reshape(ni, ni, order="F")
        L = ga[sl].reshape(ni, ni, order="F")
        assert np.linalg.norm(A - L @ L.T, 1) / np.linalg.norm(A, 1) <= 1e-13 * ni


def test_set_form_rejects_other_plans(mf):
    n = np.array([3, 4], np.int32)
    a_off = np.array([0, 9], np.int64)
    piv_off = np.array([0, 3], np.int64)
    batch = mf.LuInverseBatch(n, a_off, piv_off)
    with pytest.raises(RuntimeError):      # the C call refuses a plan that is not a Cholesky
        mf.CholeskyBatch.set_form(batch, "fma")


def test_cholesky_fma_padded(mf):
    """lda > n in the FMA form: the factor is backward stable, the padding rows are untouched."""
    import torch
    rng = np.random.default_rng(79)
    count = 150
    n = rng.integers(1, 129, size=count).astype(np.int32)
    lda = (n + rng.integers(1, 5, size=count)).astype(np.int32)
    mats = []
    for i, ni in enumerate(n):
        bm = rng.standard_normal((ni, ni))
        full = np.full((int(lda[i]), ni), 7.0)
        full[:ni, :] = bm @ bm.T + ni * np.eye(ni)
        mats.append(full.reshape(-1, order="F"))
    sz = lda.astype(np.int64) * n
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    b_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]]).astype(np.int64)
    a = np.concatenate(mats)
    b = rng.standard_normal(int(n.sum()))
    batch = mf.CholeskyBatch(n, a_off, nrhs=1, b_off=b_off, lda=lda)
    batch.set_form("fma")
    da, db = _dev(a), _dev(b)
    dinfo = torch.zeros(count, dtype=torch.int32, device="cuda")
    batch.run(da, db, dinfo)
    mf.context().synchronize()
    assert not _host(dinfo).any()
    ga, gb = _host(da), _host(db)
    for i in range(count):
        ni, li = int(n[i]), int(lda[i])
        F = ga[a_off[i]:a_off[i] + li * ni].reshape(ni, li).T
        assert (F[ni:, :] == 7.0).all()
        A = a[a_off[i]:a_off[i] + li * ni].reshape(ni, li).T[:ni, :]
        L = np.tril(F[:ni, :])
        assert np.linalg.norm(A - L @ L.T, 1) / np.linalg.norm(A, 1) <= 1e-13 * ni, i
        x, bi = gb[b_off[i]:b_off[i] + ni], b[b_off[i]:b_off[i] + ni]
        assert np.linalg.norm(bi - A @ x, 1) / (np.linalg.norm(A, 1) * np.linalg.norm(x, 1) +
                                                np.linalg.norm(bi, 1)) <= 1e-13 * ni, i

"""The FMA form of the batched double LU (mfg_plan_set_form(MFG_FORM_FMA) on a getrf plan):
fused multiply-add dots and reciprocal scaling, MatFlat's pivots kept by a screen that sends the
matrices whose choice could depend on rounding (ties, near-ties, zero pivots, NaN or infinite
entries) back to MatFlat's arithmetic.  Checked against what the form promises: pivots, signs and
info identical to the oracle's (MatFlat's LuCore) on every matrix; factors and solutions within a
normwise backward error of 1e-13 n; the redone matrices bit-identical to MatFlat's factors;
solve-only and host-buffer calls equal to the fused device call; the exact form unchanged on the
same plan afterwards."""
import numpy as np
import pytest

from oracle import oracle
from tests.test_gpu_parity import _dev, _host, assert_bits

pytestmark = pytest.mark.gpu


def _batch(rng, count, nmax=128, crafted=True):
    n = rng.integers(1, nmax + 1, size=count).astype(np.int32)
    if crafted:
        n[:6] = [40, 33, 50, 64, 48, 128]
    sz = n.astype(np.int64) ** 2
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    a = rng.standard_normal(int(sz.sum()))
    special = []
    if crafted:
        def mat(i):
            return a[a_off[i]:a_off[i] + n[i] * n[i]].reshape(n[i], n[i], order="F")
        mat(0)[:] = 0.0                                   # singular: zero pivot
        mat(1)[7, 3] = np.nan                             # NaN entry
        mat(2)[11, 20] = np.inf                           # infinite entry
        mat(3)[:, 0] = 1.0                                # tied first-column candidates
        m4 = mat(4)
        m4[5, 0] = 50.0
        m4[9, 0] = -50.0 * (1.0 + 2.0 ** -45)             # near-tie, 3e-14 apart
        special = [0, 1, 2, 3, 4]
    piv_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]]).astype(np.int64)
    b_off = piv_off * 4
    b = rng.standard_normal(int(n.sum()) * 4)
    return n, a_off, a, piv_off, b_off, b, special


def _run(mf, batch, a, b, n):
    import torch
    da, db = _dev(a), _dev(b)
    dpiv = torch.zeros(int(n.sum()), dtype=torch.int32, device="cuda")
    dsign = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    batch.run(da, dpiv, db, dsign, dinfo)
    mf.context().synchronize()
    return da, db, dpiv, dsign, dinfo


@pytest.mark.parametrize("table", [0, 2])
def test_lu_fma_pivots_and_backward_error(mf, table, monkeypatch):
    import torch
    monkeypatch.setenv("MFG_LU_GROUPS", str(table))
    rng = np.random.default_rng(300 + table)
    n, a_off, a, piv_off, b_off, b, special = _batch(rng, 400)
    batch = mf.LuBatch(n, a_off, piv_off, nrhs=4, b_off=b_off)
    batch.set_form("fma")
    da, db, dpiv, dsign, dinfo = _run(mf, batch, a, b, n)
    fallbacks = batch.form_fallbacks()
    oa, ob = a.copy(), b.copy()
    opiv = np.zeros(int(n.sum()), np.int32)
    osign = np.zeros(len(n), np.int32)
    oracle.lu_solve_batched(n, a_off, oa, piv_off, opiv, b_off, ob, 4, osign, 4)
    ga, gb, gpiv = _host(da), _host(db), _host(dpiv)
    np.testing.assert_array_equal(gpiv, opiv)
    np.testing.assert_array_equal(_host(dsign), osign)
    assert _host(dinfo)[0] == 1
    assert fallbacks >= len(special), fallbacks
    differs = 0
    for i in range(len(n)):
        ni = int(n[i])
        sl = slice(a_off[i], a_off[i] + ni * ni)
        if i in special:
            # redone in MatFlat's arithmetic: the oracle's factors bit for bit
            assert_bits(ga[sl], oa[sl], "fallback matrix %d" % i)
            continue
        A = a[sl].reshape(ni, ni, order="F")
        F = ga[sl].reshape(ni, ni, order="F")
        p = gpiv[piv_off[i]:piv_off[i] + ni]
        L = np.tril(F, -1) + np.eye(ni)
        U = np.triu(F)
        ef = np.linalg.norm(A[p, :] - L @ U, 1) / np.linalg.norm(A, 1)
        assert ef <= 1e-13 * ni, (i, ni, ef)
        for r in range(4):
            bs = slice(b_off[i] + r * ni, b_off[i] + (r + 1) * ni)
            x, bi = gb[bs], b[bs]
            ex = np.linalg.norm(bi - A @ x, 1) / (np.linalg.norm(A, 1) * np.linalg.norm(x, 1) +
                                                  np.linalg.norm(bi, 1))
            assert ex <= 1e-13 * ni, (i, ni, r, ex)
        differs += int(not np.array_equal(ga[sl], oa[sl]))
    assert differs > 0
    # solve-only on the factors: the fused call's solutions bit for bit
    db2 = _dev(b)
    torch.cuda.synchronize()
    batch.solve(da, dpiv, db2)
    mf.context().synchronize()
    assert_bits(_host(db2), gb)
    # back to the exact form: MatFlat's bits
    batch.set_form("exact")
    da, db, dpiv, dsign, dinfo = _run(mf, batch, a, b, n)
    assert_bits(_host(da), oa)
    assert_bits(_host(db), ob)
    np.testing.assert_array_equal(_host(dpiv), opiv)
    assert batch.form_fallbacks() == 0


def test_lu_fma_host_buffers_and_autotune(mf):
    rng = np.random.default_rng(310)
    n, a_off, a, piv_off, b_off, b, special = _batch(rng, 6000)
    batch = mf.LuBatch(n, a_off, piv_off, nrhs=4, b_off=b_off)
    batch.set_form("fma")
    batch.autotune()
    da, db, dpiv, dsign, dinfo = _run(mf, batch, a, b, n)
    dev_fb = batch.form_fallbacks()
    ha, hb = a.copy(), b.copy()
    hpiv = np.zeros(int(n.sum()), np.int32)
    hsign = np.zeros(len(n), np.int32)
    hinfo = np.zeros(len(n), np.int32)
    batch.run_host(ha, hpiv, hb, hsign, hinfo)
    assert batch.form_fallbacks() == dev_fb >= len(special)
    assert_bits(ha, _host(da))
    assert_bits(hb, _host(db))
    np.testing.assert_array_equal(hpiv, _host(dpiv))
    np.testing.assert_array_equal(hinfo, _host(dinfo))
    opiv = np.zeros(int(n.sum()), np.int32)
    osign = np.zeros(len(n), np.int32)
    oracle.lu_solve_batched(n, a_off, a.copy(), piv_off, opiv, b_off, b.copy(), 4, osign, 8)
    np.testing.assert_array_equal(hpiv, opiv)
    np.testing.assert_array_equal(hsign, osign)


@pytest.mark.parametrize("big", [False, True], ids=["cta-bucket", "task-bucket"])
def test_lu_fma_padded_and_large_orders(mf, big):
    """lda > n, and orders above 128: up to order 152 in 32-lane tasks (scratch in global
    memory), above it in the blocked CTA kernel, few or many of them.  Pivots identical to the
    oracle's, factors backward stable."""
    import torch
    rng = np.random.default_rng(320 + big)
    count = 1400 if big else 120
    n = rng.integers(1, 141, size=count).astype(np.int32)
    if big:
        n[:1300] = rng.integers(129, 141, size=1300)
        n[1300:1350] = rng.integers(177, 201, size=50)     # the blocked CTA kernel beside them
    lda = (n + rng.integers(0, 4, size=count)).astype(np.int32)
    sz = lda.astype(np.int64) * n
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    a = rng.standard_normal(int(sz.sum()))
    piv_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]]).astype(np.int64)
    b_off = piv_off * 2
    b = rng.standard_normal(int(n.sum()) * 2)
    batch = mf.LuBatch(n, a_off, piv_off, nrhs=2, b_off=b_off, lda=lda)
    batch.set_form("fma")
    da, db = _dev(a), _dev(b)
    dpiv = torch.zeros(int(n.sum()), dtype=torch.int32, device="cuda")
    dsign = torch.zeros(count, dtype=torch.int32, device="cuda")
    dinfo = torch.zeros(count, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    batch.run(da, dpiv, db, dsign, dinfo)
    mf.context().synchronize()
    ga, gpiv = _host(da), _host(dpiv)
    for i in range(0, count, 7 if big else 1):
        ni, li = int(n[i]), int(lda[i])
        A = a[a_off[i]:a_off[i] + li * ni].reshape(ni, li).T
        oa = a[a_off[i]:a_off[i] + li * ni].copy()
        opiv = np.zeros(ni, np.int32)
        oracle.lu(ni, ni, oa, li, opiv)
        p = gpiv[piv_off[i]:piv_off[i] + ni]
        np.testing.assert_array_equal(p, opiv, err_msg="matrix %d" % i)
        F = ga[a_off[i]:a_off[i] + li * ni].reshape(ni, li).T
        np.testing.assert_array_equal(F[ni:li, :], A[ni:li, :])     # padding untouched
        F = F[:ni, :]
        L = np.tril(F, -1) + np.eye(ni)
        U = np.triu(F)
        An = A[:ni, :]
        assert np.linalg.norm(An[p, :] - L @ U, 1) / np.linalg.norm(An, 1) <= 1e-13 * ni, i


@pytest.mark.parametrize("mma", [0, 1], ids=["fma-tiles", "dmma-tiles"])
def test_lu_fma_blocked_large_orders(mf, mma, monkeypatch):
    """Orders above 128 in the FMA form run the blocked CTA kernel (panels of 32 columns, U12
    solve, 64 x 64 trailing-update tiles of fused multiply-adds, or of FP64 tensor-pipe mma with
    MFG_LU_BIG_MMA=1): pivots and signs identical to the oracle's, factors and solutions backward
    stable, padding rows untouched; a near-tie and a NaN at large orders are redone in MatFlat's
    arithmetic (the oracle's bits); solve-only calls give the fused call's bits; the exact form
    afterwards gives MatFlat's bits."""
    import torch
    monkeypatch.setenv("MFG_LU_BIG_MMA", str(mma))
    rng = np.random.default_rng(330)
    n = np.array([129, 160, 191, 200, 256, 257, 300, 333, 384, 512, 97, 64, 450, 130],
                 np.int32)
    count = len(n)
    lda = (n + rng.integers(0, 4, size=count)).astype(np.int32)
    sz = lda.astype(np.int64) * n
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    a = rng.standard_normal(int(sz.sum()))

    def mat(i):
        return a[a_off[i]:a_off[i] + sz[i]].reshape(n[i], lda[i]).T

    mat(5)[7, 0] = 50.0
    mat(5)[90, 0] = -50.0 * (1.0 + 2.0 ** -45)        # near-tie in column 0: redone exactly
    mat(7)[200, 150] = np.nan                          # NaN: redone exactly
    special = [5, 7]
    piv_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]]).astype(np.int64)
    nrhs = 2
    b_off = piv_off * nrhs
    b = rng.standard_normal(int(n.sum()) * nrhs)
    batch = mf.LuBatch(n, a_off, piv_off, nrhs=nrhs, b_off=b_off, lda=lda)
    batch.set_form("fma")
    da, db = _dev(a), _dev(b)
    dpiv = torch.zeros(int(n.sum()), dtype=torch.int32, device="cuda")
    dsign = torch.zeros(count, dtype=torch.int32, device="cuda")
    dinfo = torch.zeros(count, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    batch.run(da, dpiv, db, dsign, dinfo)
    mf.context().synchronize()
    assert batch.form_fallbacks() == len(special)
    ga, gb, gpiv, gsign = _host(da), _host(db), _host(dpiv), _host(dsign)
    assert not _host(dinfo)[[i for i in range(count) if i not in special]].any()
    for i in range(count):
        ni, li = int(n[i]), int(lda[i])
        A = mat(i)
        oa = a[a_off[i]:a_off[i] + sz[i]].copy()
        opiv = np.zeros(ni, np.int32)
        osign = oracle.lu(ni, ni, oa, li, opiv)
        p = gpiv[piv_off[i]:piv_off[i] + ni]
        np.testing.assert_array_equal(p, opiv, err_msg="matrix %d" % i)
        assert gsign[i] == osign, i
        F = ga[a_off[i]:a_off[i] + sz[i]].reshape(ni, li).T
        np.testing.assert_array_equal(F[ni:li, :], A[ni:li, :])     # padding untouched
        if i in special:
            assert_bits(ga[a_off[i]:a_off[i] + sz[i]], oa, "fallback matrix %d" % i)
            continue
        F = F[:ni, :]
        L = np.tril(F, -1) + np.eye(ni)
        U = np.triu(F)
        An = A[:ni, :]
        assert np.linalg.norm(An[p, :] - L @ U, 1) / np.linalg.norm(An, 1) <= 1e-13 * ni, i
        for r in range(nrhs):
            bs = slice(b_off[i] + r * ni, b_off[i] + (r + 1) * ni)
            x, bi = gb[bs], b[bs]
            ex = np.linalg.norm(bi - An @ x, 1) / (np.linalg.norm(An, 1) * np.linalg.norm(x, 1) +
                                                   np.linalg.norm(bi, 1))
            assert ex <= 1e-13 * ni, (i, r, ex)
    # solve-only on the factors: the fused call's solutions bit for bit
    db2 = _dev(b)
    torch.cuda.synchronize()
    batch.solve(da, dpiv, db2)
    mf.context().synchronize()
    assert_bits(_host(db2), gb)
    # back to the exact form: MatFlat's bits on every matrix
    batch.set_form("exact")
    da = _dev(a)
    torch.cuda.synchronize()
    batch.run(da, dpiv, _dev(b), dsign, dinfo)
    mf.context().synchronize()
    ga = _host(da)
    for i in (0, 4, 9):
        ni, li = int(n[i]), int(lda[i])
        oa = a[a_off[i]:a_off[i] + sz[i]].copy()
        oracle.lu(ni, ni, oa, li, np.zeros(ni, np.int32))
        assert_bits(ga[a_off[i]:a_off[i] + sz[i]], oa, "exact matrix %d" % i)
    assert batch.form_fallbacks() == 0


def test_lu_fma_large_orders_host_buffers(mf, monkeypatch):
    """Host-buffer calls (four pipelined chunk plans) give the device call's bits in the FMA form
    for orders on both sides of the blocked kernel's threshold (152)."""
    monkeypatch.setenv("MFG_PIPE_CHUNKS", "4")
    rng = np.random.default_rng(340)
    n = rng.choice([40, 150, 170, 200, 260], size=48).astype(np.int32)
    sz = n.astype(np.int64) ** 2
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    a = rng.standard_normal(int(sz.sum()))
    piv_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]]).astype(np.int64)
    b_off = piv_off * 2
    b = rng.standard_normal(int(n.sum()) * 2)
    batch = mf.LuBatch(n, a_off, piv_off, nrhs=2, b_off=b_off)
    batch.set_form("fma")
    da, db, dpiv, dsign, dinfo = _run(mf, batch, a, b, n)
    ha, hb = a.copy(), b.copy()
    hpiv = np.zeros(int(n.sum()), np.int32)
    hsign = np.zeros(len(n), np.int32)
    hinfo = np.zeros(len(n), np.int32)
    batch.run_host(ha, hpiv, hb, hsign, hinfo)
    assert_bits(ha, _host(da))
    assert_bits(hb, _host(db))
    np.testing.assert_array_equal(hpiv, _host(dpiv))
    np.testing.assert_array_equal(hsign, _host(dsign))
    for i in (0, 1, 2, 3):
        ni = int(n[i])
        oa = a[a_off[i]:a_off[i] + sz[i]].copy()
        opiv = np.zeros(ni, np.int32)
        oracle.lu(ni, ni, oa, ni, opiv)
        np.testing.assert_array_equal(hpiv[piv_off[i]:piv_off[i] + ni], opiv)

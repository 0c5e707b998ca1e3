"""The FMA form of the batched double QR (mfg_plan_set_form(MFG_FORM_FMA) on a geqrf plan):
MatFlat's Householder algorithm and storage with fused multiply-adds, so the factors are not
MatFlat's bits; checked by what the form promises instead: the reflectors and R reproduce A to a
normwise backward error within 1e-13 * m, the least-squares solutions satisfy the normal
equations to the same order as the exact form's, rdiag agrees with MatFlat's to rounding times
the condition, solve-only calls give the fused call's bits, and the exact form is unchanged on
the same plan afterwards."""
import numpy as np
import pytest

from oracle import oracle
from tests.test_gpu_parity import _dev, _host, assert_bits

pytestmark = pytest.mark.gpu


def _reconstruct(f, rd, m, n):
    """A from MatFlat's storage: v_k = f[k:, k] (v_k[0] = 1 + a_kk / norm), H_k = I - v v^T / v0,
    R = strict upper part of f plus diag(rdiag); A = H_0 H_1 ... H_{n-1} [R; 0]."""
    r = np.zeros((m, n))
    r[:n, :] = np.triu(f[:n, :], 1)
    r[np.arange(n), np.arange(n)] = rd
    for k in range(n - 1, -1, -1):
        v = f[k:, k]
        if rd[k] != 0 and v[0] != 0:
            r[k:, :] -= np.outer(v, v @ r[k:, :]) / v[0]
    return r


def test_qr_fma_backward_error(mf):
    import torch
    rng = np.random.default_rng(91)
    count = 160
    m = rng.integers(1, 300, size=count).astype(np.int32)
    n = np.minimum(rng.integers(1, 70, size=count), m).astype(np.int32)
    m[:4], n[:4] = [1, 64, 512, 40], [1, 64, 64, 12]
    sz = m.astype(np.int64) * n
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]])
    a = rng.standard_normal(int(sz.sum()))
    a[a_off[3] + 2 * 40:a_off[3] + 3 * 40] = 0.0            # a zero column: degenerate reflector
    r_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]])
    b_off = np.concatenate([[0], np.cumsum(m.astype(np.int64))[:-1]])
    b = rng.standard_normal(int(m.sum()))
    batch = mf.QrBatch(m, n, a_off, r_off, nrhs=1, b_off=b_off)
    batch.set_form("fma")
    da, db = _dev(a), _dev(b)
    dr = torch.zeros(int(n.sum()), dtype=torch.float64, device="cuda")
    batch.run(da, dr, db)
    mf.context().synchronize()
    ga, gr, gb = _host(da), _host(dr), _host(db)
    differs = 0
    for i in range(count):
        mi, ni = int(m[i]), int(n[i])
        A = a[a_off[i]:a_off[i] + mi * ni].reshape(ni, mi).T
        F = ga[a_off[i]:a_off[i] + mi * ni].reshape(ni, mi).T
        rd = gr[r_off[i]:r_off[i] + ni]
        na = np.linalg.norm(A)
        berr = np.linalg.norm(A - _reconstruct(F, rd, mi, ni)) / max(na, 1e-300)
        assert berr <= 1e-13 * mi, (i, mi, ni, berr)
        # MatFlat's factors of the same matrix: rdiag to rounding times the condition
        ao = a[a_off[i]:a_off[i] + mi * ni].copy()
        ro = np.zeros(ni)
        oracle.qr(mi, ni, ao, mi, ro)
        if i != 3:
            cond = np.linalg.cond(A)
            assert np.max(np.abs(rd - ro)) <= 1e-13 * cond * ni * max(1.0, np.max(np.abs(ro)))
        differs += int(not np.array_equal(ga[a_off[i]:a_off[i] + mi * ni], ao))
        # least squares through the normal-equation residual, as for the exact form
        bi = b[b_off[i]:b_off[i] + mi]
        x = gb[b_off[i]:b_off[i] + ni]
        if i != 3:
            res = np.linalg.norm(A.T @ (A @ x - bi))
            assert res / (na * np.linalg.norm(bi) + 1e-300) <= 1e-9, i
    assert differs > 0
    # solve-only on the FMA factors: the fused call's solutions, bit for bit
    db2 = _dev(b)
    torch.cuda.synchronize()
    batch.solve(da, dr, db2)
    mf.context().synchronize()
    for i in range(count):
        sl = slice(b_off[i], b_off[i] + int(n[i]))
        assert_bits(_host(db2)[sl], gb[sl], "solve-only, matrix %d" % i)
    # back to the exact form: MatFlat's bits
    batch.set_form("exact")
    da, db = _dev(a), _dev(b)
    batch.run(da, dr, db)
    mf.context().synchronize()
    ga, gr = _host(da), _host(dr)
    for i in range(0, count, 9):
        mi, ni = int(m[i]), int(n[i])
        ao = a[a_off[i]:a_off[i] + mi * ni].copy()
        ro = np.zeros(ni)
        oracle.qr(mi, ni, ao, mi, ro)
        assert_bits(ga[a_off[i]:a_off[i] + mi * ni], ao, "factors %d" % i)
        assert_bits(gr[r_off[i]:r_off[i] + ni], ro, "rdiag %d" % i)


def test_qr_fma_autotune_and_host(mf):
    """The autotuner keeps the form, and the pipelined host-buffer call gives the device call's
    bits."""
    import torch
    rng = np.random.default_rng(92)
    count = 3000
    m = rng.integers(64, 200, size=count).astype(np.int32)
    n = rng.integers(16, 64, size=count).astype(np.int32)
    sz = m.astype(np.int64) * n
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]])
    a = rng.standard_normal(int(sz.sum()))
    r_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]])
    b_off = np.concatenate([[0], np.cumsum(m.astype(np.int64))[:-1]])
    b = rng.standard_normal(int(m.sum()))
    batch = mf.QrBatch(m, n, a_off, r_off, nrhs=1, b_off=b_off)
    batch.set_form("fma")
    batch.autotune()
    da, db = _dev(a), _dev(b)
    dr = torch.zeros(int(n.sum()), dtype=torch.float64, device="cuda")
    batch.run(da, dr, db)
    mf.context().synchronize()
    ha, hb = a.copy(), b.copy()
    hr = np.zeros(int(n.sum()))
    batch.run_host(ha, hr, hb)
    assert_bits(ha, _host(da))
    assert_bits(hr, _host(dr))
    assert_bits(hb, _host(db))
    for i in range(0, count, 97):
        mi, ni = int(m[i]), int(n[i])
        A = a[a_off[i]:a_off[i] + mi * ni].reshape(ni, mi).T
        F = ha[a_off[i]:a_off[i] + mi * ni].reshape(ni, mi).T
        rd = hr[r_off[i]:r_off[i] + ni]
        assert np.linalg.norm(A - _reconstruct(F, rd, mi, ni)) / np.linalg.norm(A) <= 1e-13 * mi

"""Single-matrix entry points called with DEVICE arrays give the same bits as with host arrays."""
import ctypes

import numpy as np
import pytest

from tests.test_gpu_parity import assert_bits

pytestmark = pytest.mark.gpu

U, L, NT, T = 121, 122, 111, 112


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def test_device_arrays_match_host_arrays(mf):
    import torch
    ctx = mf.context()
    lib = ctx.lib
    rng = np.random.default_rng(51)
    m, n, lda = 37, 29, 41
    a = rng.standard_normal(lda * n)
    # LU
    ha, hpiv = a.copy(), np.zeros(m, np.int32)
    hsign = mf.Factorization.Lu(m, n, ha, lda, hpiv)
    da = torch.from_numpy(a.copy()).cuda()
    dpiv = torch.zeros(m, dtype=torch.int32, device="cuda")
    sign = ctypes.c_int(0)
    assert lib.mfg_dgetrf(ctx.h, m, n, _vp(da), lda, _vp(dpiv), ctypes.byref(sign)) == 0
    assert_bits(da.cpu().numpy(), ha)
    np.testing.assert_array_equal(dpiv.cpu().numpy(), hpiv)
    assert sign.value == hsign
    # Cholesky
    k = 33
    bm = rng.standard_normal((k, k))
    spd = (bm @ bm.T + k * np.eye(k)).flatten(order="F")
    hs = spd.copy()
    mf.Factorization.Cholesky(k, hs, k)
    ds = torch.from_numpy(spd.copy()).cuda()
    info = ctypes.c_int(-1)
    assert lib.mfg_dpotrf(ctx.h, k, _vp(ds), k, ctypes.byref(info)) == 0
    assert info.value == 0
    assert_bits(ds.cpu().numpy(), hs)
    # QR + Q + R
    hq_a, hrd = a.copy(), np.zeros(n)
    mf.Factorization.Qr(m, n, hq_a, lda, hrd)
    dq_a = torch.from_numpy(a.copy()).cuda()
    drd = torch.zeros(n, dtype=torch.float64, device="cuda")
    assert lib.mfg_dgeqrf(ctx.h, m, n, _vp(dq_a), lda, _vp(drd)) == 0
    assert_bits(dq_a.cpu().numpy(), hq_a)
    assert_bits(drd.cpu().numpy(), hrd)
    hq = np.zeros(m * n)
    mf.Factorization.QrOrthogonalFactor(m, n, hq_a, lda, hq, m)
    dq = torch.zeros(m * n, dtype=torch.float64, device="cuda")
    assert lib.mfg_dorgqr(ctx.h, m, n, _vp(dq_a), lda, _vp(dq), m) == 0
    assert_bits(dq.cpu().numpy(), hq)
    # SolveTriangular (upper factor of the LU above) and MulMatMat
    x = rng.standard_normal(n)
    hx = x.copy()
    mf.Blas.SolveTriangular(U, NT, n, ha, lda, hx, 1)
    dx = torch.from_numpy(x.copy()).cuda()
    assert lib.mfg_dtrsv(ctx.h, U, NT, n, _vp(da), lda, _vp(dx), 1) == 0
    assert_bits(dx.cpu().numpy(), hx)
    b = rng.standard_normal(n * 5)
    hc = np.zeros(m * 5)
    mf.Blas.MulMatMat(NT, NT, m, 5, n, a, lda, b, n, hc, m)
    dA = torch.from_numpy(a.copy()).cuda()
    dB = torch.from_numpy(b.copy()).cuda()
    dC = torch.zeros(m * 5, dtype=torch.float64, device="cuda")
    assert lib.mfg_dgemm(ctx.h, NT, NT, m, 5, n, _vp(dA), lda, _vp(dB), n, _vp(dC), m) == 0
    assert_bits(dC.cpu().numpy(), hc)
    # LuInverse of a square LU
    s = 24
    sq = rng.standard_normal(s * s)
    hpv = np.zeros(s, np.int32)
    mf.Factorization.Lu(s, s, sq, s, hpv)
    hinv = sq.copy()
    mf.Factorization.LuInverse(s, hinv, s, hpv)
    dinv = torch.from_numpy(sq.copy()).cuda()
    dpv = torch.from_numpy(hpv.copy()).cuda()
    inf = ctypes.c_int(-1)
    assert lib.mfg_dgetri(ctx.h, s, _vp(dinv), s, _vp(dpv), ctypes.byref(inf)) == 0
    assert inf.value == 0
    assert_bits(dinv.cpu().numpy(), hinv)
    # Complex LU with a device array
    z = (rng.standard_normal(m * n) + 1j * rng.standard_normal(m * n))
    hz, hzp = z.copy(), np.zeros(m, np.int32)
    mf.Factorization.Lu(m, n, hz, m, hzp)
    dz = torch.from_numpy(z.view(np.float64).copy()).cuda()
    dzp = torch.zeros(m, dtype=torch.int32, device="cuda")
    assert lib.mfg_zgetrf(ctx.h, m, n, _vp(dz), m, _vp(dzp), ctypes.byref(sign)) == 0
    assert_bits(dz.cpu().numpy(), hz.view(np.float64))
    np.testing.assert_array_equal(dzp.cpu().numpy(), hzp)


def test_context_runs_on_its_device_and_restores_the_callers(mf):
    """Every call runs on the context's device and leaves the caller's current device as it
    was.  With one visible GPU the switch itself cannot be exercised: the test checks the
    device the context reports, that a call made while another device id was current on the
    host thread still computes correctly (when a second device exists), and that the caller's
    device is unchanged after the call."""
    import torch
    ctx = mf.context()
    dev = ctx.device()
    assert dev == torch.cuda.current_device()
    rng = np.random.default_rng(77)
    n = 24
    a = rng.standard_normal(n * n)
    ref, rpiv = a.copy(), np.zeros(n, np.int32)
    rsign = mf.Factorization.Lu(n, n, ref, n, rpiv)
    other = (dev + 1) % torch.cuda.device_count()
    prev = torch.cuda.current_device()
    torch.cuda.set_device(other)
    try:
        got, gpiv = a.copy(), np.zeros(n, np.int32)
        gsign = mf.Factorization.Lu(n, n, got, n, gpiv)
        assert torch.cuda.current_device() == other
    finally:
        torch.cuda.set_device(prev)
    assert_bits(got, ref)
    np.testing.assert_array_equal(gpiv, rpiv)
    assert gsign == rsign

"""Strided batches of MulMatVec / Dot / L2Norm / Outer against the oracle, bit for bit."""
import numpy as np
import pytest

from oracle import oracle
from tests.test_gpu_parity import _dev, _host, assert_bits

pytestmark = pytest.mark.gpu

NT, T = 111, 112


@pytest.mark.parametrize("trans", [NT, T])
def test_gemv_strided(mf, trans):
    import torch
    rng = np.random.default_rng(81)
    m, n, lda, incx, incy, count = 37, 29, 41, 2, 3, 50
    sa = lda * n + 5
    lx = (n if trans == NT else m)
    ly = (m if trans == NT else n)
    sx, sy = incx * lx + 1, incy * ly + 2
    a = rng.standard_normal(sa * count)
    x = rng.standard_normal(sx * count)
    y0 = rng.standard_normal(sy * count)
    exp = y0.copy()
    for b in range(count):
        oracle.gemv(trans, m, n, a[b * sa:], lda, x[b * sx:], incx, exp[b * sy:], incy)
    dy, da, dx = _dev(y0), _dev(a), _dev(x)   # kept alive until the stream is synchronised
    mf.StridedBlas.MulMatVec(trans, m, n, da, lda, sa, dx, incx, sx, dy, incy, sy, count)
    mf.context().synchronize()
    assert_bits(_host(dy), exp)


def test_dot_nrm2_strided(mf):
    import torch
    rng = np.random.default_rng(82)
    for n, inc in ((77, 1), (64, 3), (1, 1)):
        count = 1000
        s = n * inc + 7
        x = rng.standard_normal(s * count)
        y = rng.standard_normal(s * count)
        d_out = torch.zeros(count, dtype=torch.float64, device="cuda")
        dx, dy = _dev(x), _dev(y)
        mf.StridedBlas.Dot(n, dx, inc, s, dy, inc, s, d_out, count)
        n_out = torch.zeros(count, dtype=torch.float64, device="cuda")
        mf.StridedBlas.L2Norm(n, dx, inc, s, n_out, count)
        mf.context().synchronize()
        ed = np.array([oracle.dot(n, x[b * s:], inc, y[b * s:], inc) for b in range(count)])
        en = np.array([oracle.nrm2(n, x[b * s:], inc) for b in range(count)])
        assert_bits(_host(d_out), ed)
        assert_bits(_host(n_out), en)


def test_ger_strided(mf):
    rng = np.random.default_rng(83)
    m, n, lda, count = 13, 9, 15, 20
    sx, sy, sa = 2 * m, n + 3, lda * n + 1
    x = rng.standard_normal(sx * count)
    y = rng.standard_normal(sy * count)
    a0 = rng.standard_normal(sa * count)
    exp = a0.copy()
    for b in range(count):
        oracle.ger(m, n, x[b * sx:], 2, y[b * sy:], 1, exp[b * sa:], lda)
    da, dx, dy = _dev(a0), _dev(x), _dev(y)
    mf.StridedBlas.Outer(m, n, dx, 2, sx, dy, 1, sy, da, lda, sa, count)
    mf.context().synchronize()
    assert_bits(_host(da), exp)


def test_gemv_in_place_rejected(mf):
    import torch
    z = torch.zeros(100, dtype=torch.float64, device="cuda")
    with pytest.raises(mf.ArgumentException):
        mf.StridedBlas.MulMatVec(NT, 3, 3, z, 3, 9, z, 1, 3, z, 1, 3, 1)
    with pytest.raises(mf.ArgumentException):
        mf.StridedBlas.MulMatVec(NT, 3, 3, z, 2, 9, z[50:], 1, 3, z[80:], 1, 3, 1)


def _draw(rng, k, dt):
    if dt == np.complex128:
        return rng.standard_normal(k) + 1j * rng.standard_normal(k)
    return rng.standard_normal(k).astype(dt)


def _flat(x):
    return x.view(np.float64) if x.dtype == np.complex128 else x


@pytest.mark.parametrize("dt,trans", [(np.float32, NT), (np.float32, T), (np.complex128, NT),
                                      (np.complex128, T), (np.complex128, 113),
                                      (np.complex128, 114)])
def test_gemv_strided_types(mf, dt, trans):
    rng = np.random.default_rng(84)
    m, n, lda, incx, incy, count = 37, 29, 41, 2, 3, 40
    sa = lda * n + 5
    rows = trans in (NT, 114)
    lx, ly = (n, m) if rows else (m, n)
    sx, sy = incx * lx + 1, incy * ly + 2
    a, x, y0 = _draw(rng, sa * count, dt), _draw(rng, sx * count, dt), _draw(rng, sy * count, dt)
    exp = y0.copy()
    for b in range(count):
        ey = exp[b * sy:]
        oracle.gemv(trans, m, n, a[b * sa:], lda, x[b * sx:], incx, ey, incy)
        exp[b * sy:] = ey
    dy, da, dx = _dev(y0), _dev(a), _dev(x)   # kept alive until the stream is synchronised
    mf.StridedBlas.MulMatVec(trans, m, n, da, lda, sa, dx, incx, sx, dy, incy, sy, count)
    mf.context().synchronize()
    assert_bits(_flat(_host(dy)), _flat(exp))


@pytest.mark.parametrize("dt", [np.float32, np.complex128])
def test_dot_nrm2_strided_types(mf, dt):
    import torch
    rng = np.random.default_rng(85)
    rdt = {np.float32: torch.float32, np.complex128: torch.complex128}[dt]
    for n, inc in ((77, 1), (64, 3), (1, 1)):
        count = 500
        s = n * inc + 7
        x, y = _draw(rng, s * count, dt), _draw(rng, s * count, dt)
        d_out = torch.zeros(count, dtype=rdt, device="cuda")
        dx, dy = _dev(x), _dev(y)
        mf.StridedBlas.Dot(n, dx, inc, s, dy, inc, s, d_out, count)
        n_out = torch.zeros(count, dtype=torch.float32 if dt == np.float32 else torch.float64,
                            device="cuda")
        mf.StridedBlas.L2Norm(n, dx, inc, s, n_out, count)
        mf.context().synchronize()
        ed = np.array([oracle.dot(n, x[b * s:], inc, y[b * s:], inc) for b in range(count)],
                      dtype=dt)
        en = np.array([oracle.nrm2(n, x[b * s:], inc) for b in range(count)],
                      dtype=np.float32 if dt == np.float32 else np.float64)
        assert_bits(_flat(_host(d_out)), _flat(ed))
        assert_bits(_host(n_out), en)
        if dt == np.complex128:
            c_out = torch.zeros(count, dtype=rdt, device="cuda")
            mf.StridedBlas.DotConj(n, dx, inc, s, dy, inc, s, c_out, count)
            mf.context().synchronize()
            ec = np.array([oracle.dot(n, x[b * s:], inc, y[b * s:], inc, conj=True)
                           for b in range(count)])
            assert_bits(_flat(_host(c_out)), _flat(ec))


@pytest.mark.parametrize("dt,conj", [(np.float32, False), (np.complex128, False),
                                     (np.complex128, True)])
def test_ger_strided_types(mf, dt, conj):
    rng = np.random.default_rng(86)
    m, n, lda, count = 13, 9, 15, 20
    sx, sy, sa = 2 * m, n + 3, lda * n + 1
    x, y, a0 = _draw(rng, sx * count, dt), _draw(rng, sy * count, dt), _draw(rng, sa * count, dt)
    exp = a0.copy()
    for b in range(count):
        ea = exp[b * sa:]
        oracle.ger(m, n, x[b * sx:], 2, y[b * sy:], 1, ea, lda, conj=conj)
    da, dx, dy = _dev(a0), _dev(x), _dev(y)
    fn = mf.StridedBlas.OuterConj if conj else mf.StridedBlas.Outer
    fn(m, n, dx, 2, sx, dy, 1, sy, da, lda, sa, count)
    mf.context().synchronize()
    assert_bits(_flat(_host(da)), _flat(exp))

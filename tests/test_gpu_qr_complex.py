"""Batched QR + least squares of MatFlat's Complex overload: factors and rdiag bit-identical to
the oracle's Factorization.Qr(Complex); least-squares solutions checked through the normal
equations A^H (A x - b) = 0 and against the oracle's composition (MatFlat has no QR solve, so
the reflector-applied Q^H b rounds differently from an explicit Q)."""
import numpy as np
import pytest

from oracle import oracle
from tests.test_gpu_parity import _dev, _host, assert_bits

pytestmark = pytest.mark.gpu


def _cplx(rng, k):
    return rng.standard_normal(k) + 1j * rng.standard_normal(k)


@pytest.mark.parametrize("nrhs,mmax,nmax", [(0, 80, 24), (1, 200, 64), (2, 300, 140)])
def test_qr_batched_complex(mf, nrhs, mmax, nmax):
    import torch
    rng = np.random.default_rng(500 + nrhs)
    count = 300
    n = rng.integers(1, nmax + 1, size=count).astype(np.int32)
    m = np.maximum(n, rng.integers(1, mmax + 1, size=count)).astype(np.int32)
    m[:3], n[:3] = [1, 7, mmax], [1, 7, nmax]     # 1x1, square, the largest (global scratch)
    sz = m.astype(np.int64) * n
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    r_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]]).astype(np.int64)
    b_off = np.concatenate([[0], np.cumsum(m.astype(np.int64) * max(nrhs, 1))[:-1]]).astype(np.int64)
    a = _cplx(rng, int(sz.sum()))
    o = a_off[3]
    a[o:o + m[3]] = 0                             # a zero column: no reflector
    b = _cplx(rng, int((m.astype(np.int64) * max(nrhs, 1)).sum()))
    batch = mf.QrBatch(m, n, a_off, r_off, nrhs=nrhs, b_off=b_off if nrhs else None)
    da, db = _dev(a), _dev(b)
    dr = torch.zeros(int(n.sum()), dtype=torch.float64, device="cuda")
    batch.run(da, dr, db if nrhs else None)
    mf.context().synchronize()
    ga, gr, gb = _host(da), _host(dr), _host(db)
    for i in range(count):
        mi, ni = int(m[i]), int(n[i])
        ai = a[a_off[i]:a_off[i] + mi * ni].copy()
        ri = np.zeros(ni)
        oracle.qr(mi, ni, ai, mi, ri)
        assert_bits(ga[a_off[i]:a_off[i] + mi * ni].view(np.float64), ai.view(np.float64),
                    "factors %d" % i)
        assert_bits(gr[r_off[i]:r_off[i] + ni], ri, "rdiag %d" % i)
        if nrhs == 0 or np.any(ri == 0):
            continue
        A = a[a_off[i]:a_off[i] + mi * ni].reshape(ni, mi).T
        for c in range(nrhs):
            bi = b[b_off[i] + c * mi:b_off[i] + (c + 1) * mi]
            xg = gb[b_off[i] + c * mi:b_off[i] + c * mi + ni]
            xo = np.zeros(ni, np.complex128)
            oracle.qr_ls(mi, ni, a[a_off[i]:a_off[i] + mi * ni].copy(), mi, bi.copy(), xo)
            scale = np.linalg.norm(A) * np.linalg.norm(bi) + 1e-300
            for x in (xg, xo):
                res = np.linalg.norm(A.conj().T @ (A @ x - bi))
                assert res / scale <= 1e-9, (i, res / scale)
            assert np.max(np.abs(xg - xo)) <= 1e-6 * max(1.0, np.max(np.abs(xo)))
    if nrhs:
        # The solve alone from the factors reproduces the fused solutions bit for bit.
        db2 = _dev(b)
        batch.solve(da, dr, db2)
        mf.context().synchronize()
        assert_bits(_host(db2).view(np.float64), gb.view(np.float64))
    batch.close()


def test_qr_batched_complex_interleaved_and_shared_plan(mf):
    """Complex data held as interleaved float64 (dtype="z"), and double / float / Complex launches
    of one plan, each bit-identical to its oracle."""
    import torch
    rng = np.random.default_rng(520)
    count = 120
    n = rng.integers(1, 40, size=count).astype(np.int32)
    m = (n + rng.integers(0, 60, size=count)).astype(np.int32)
    sz = m.astype(np.int64) * n
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    r_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]]).astype(np.int64)
    batch = mf.QrBatch(m, n, a_off, r_off)
    for dt in (np.complex128, np.float64, np.float32, np.complex128):
        if dt == np.complex128:
            a = _cplx(rng, int(sz.sum()))
            da = _dev(a.view(np.float64))
            dr = torch.zeros(int(n.sum()), dtype=torch.float64, device="cuda")
            batch.run(da, dr, dtype="z")
        else:
            a = rng.standard_normal(int(sz.sum())).astype(dt)
            da = _dev(a)
            dr = torch.zeros(int(n.sum()), dtype=da.dtype, device="cuda")
            batch.run(da, dr, single=(dt == np.float32))
        mf.context().synchronize()
        ga, gr = _host(da), _host(dr)
        rdt = np.float64 if dt == np.complex128 else dt
        for i in range(count):
            mi, ni = int(m[i]), int(n[i])
            ai = a[a_off[i]:a_off[i] + mi * ni].copy()
            ri = np.zeros(ni, rdt)
            oracle.qr(mi, ni, ai, mi, ri)
            got = ga[2 * a_off[i]:2 * (a_off[i] + mi * ni)] if dt == np.complex128 else \
                ga[a_off[i]:a_off[i] + mi * ni]
            exp = ai.view(np.float64) if dt == np.complex128 else ai
            assert_bits(got, exp, "%s factors %d" % (dt.__name__, i))
            assert_bits(gr[r_off[i]:r_off[i] + ni], ri, "%s rdiag %d" % (dt.__name__, i))
    batch.close()

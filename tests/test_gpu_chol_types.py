"""Batched Cholesky + solve of MatFlat's float and Complex overloads: bit-identical to the
oracle's Factorization.Cholesky float / Complex followed by SolveTriangular Lower/NoTrans and
Lower/Trans (float) or Lower/ConjTrans (Complex), through the C ABI."""
import numpy as np
import pytest

from oracle import oracle
from tests.test_gpu_parity import _dev, _host, assert_bits

pytestmark = pytest.mark.gpu


def _packed(n, cols):
    sz = n.astype(np.int64) * cols
    return np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64), int(sz.sum())


def _draw(rng, k, dt):
    if dt == np.complex128:
        return rng.standard_normal(k) + 1j * rng.standard_normal(k)
    return rng.standard_normal(k).astype(dt)


def _spd(rng, n, dt):
    mats = []
    for ni in n:
        m = _draw(rng, int(ni) * int(ni), dt).reshape(ni, ni)
        mats.append((m @ m.conj().T + ni * np.eye(ni)).astype(dt).flatten(order="F"))
    return np.concatenate(mats)


def _flat(x):
    return x.view(np.float64) if x.dtype == np.complex128 else x


def _case(rng, count, nrhs, dt, nmax):
    n = rng.integers(1, nmax + 1, size=count).astype(np.int32)
    n[:4] = [1, 2, 128, nmax]
    a_off, _ = _packed(n, n)
    b_off, btot = _packed(n, np.full_like(n, max(nrhs, 1)))
    a = _spd(rng, n, dt)
    a[a_off[4]] = -1.0                         # not positive definite at column 0
    o = a_off[5]
    a[o + int(n[5]) * (int(n[5]) - 1)] = 0     # A(0, n-1) (upper triangle) changed: still read
    return n, a_off, b_off, a, _draw(rng, btot, dt)


@pytest.mark.parametrize("dt", [np.float32, np.complex128])
@pytest.mark.parametrize("nrhs,nmax", [(0, 60), (1, 20), (5, 150)])
def test_cholesky_batched_types(mf, dt, nrhs, nmax):
    import torch
    rng = np.random.default_rng(400 + nrhs + nmax + (1 if dt == np.complex128 else 0))
    n, a_off, b_off, a, b = _case(rng, 500, nrhs, dt, nmax)
    oa, ob = a.copy(), b.copy()
    oinfo = np.zeros(len(n), np.int32)
    oracle.chol_solve_batched(n, a_off, oa, b_off, ob, oinfo, 4, nrhs=nrhs)
    assert oinfo[4] == 1
    batch = mf.CholeskyBatch(n, a_off, nrhs=nrhs, b_off=b_off if nrhs else None)
    da, db = _dev(a), _dev(b)
    dinfo = torch.full((len(n),), -1, dtype=torch.int32, device="cuda")
    batch.run(da, db if nrhs else None, dinfo)
    mf.context().synchronize()
    info = _host(dinfo)
    np.testing.assert_array_equal(info, oinfo)
    ga = _host(da)
    for i in np.flatnonzero(info == 0):        # factors are unspecified where info != 0
        sl = slice(int(a_off[i]), int(a_off[i]) + int(n[i]) ** 2)
        assert_bits(_flat(ga[sl]), _flat(oa[sl]), "matrix %d" % i)
    if nrhs:
        gb = _host(db)
        for i in np.flatnonzero(info == 0):
            sl = slice(int(b_off[i]), int(b_off[i]) + int(n[i]) * nrhs)
            assert_bits(_flat(gb[sl]), _flat(ob[sl]), "rhs %d" % i)
        # The solve alone from the factors gives the same solutions.
        db2 = _dev(b)
        batch.solve(da, db2)
        mf.context().synchronize()
        gb2 = _host(db2)
        for i in np.flatnonzero(info == 0):
            sl = slice(int(b_off[i]), int(b_off[i]) + int(n[i]) * nrhs)
            assert_bits(_flat(gb2[sl]), _flat(ob[sl]), "solve-only rhs %d" % i)
    batch.close()


def test_cholesky_types_share_a_plan(mf):
    import torch
    rng = np.random.default_rng(420)
    nrhs = 2
    n = rng.integers(1, 140, size=300).astype(np.int32)
    n[:2] = [139, 16]
    a_off, _ = _packed(n, n)
    b_off, btot = _packed(n, np.full_like(n, nrhs))
    batch = mf.CholeskyBatch(n, a_off, nrhs=nrhs, b_off=b_off)
    for dt in (np.complex128, np.float64, np.float32, np.complex128):
        a = _spd(rng, n, dt)
        b = _draw(rng, btot, dt) if dt != np.float64 else rng.standard_normal(btot)
        oa, ob = a.copy(), b.copy()
        oinfo = np.zeros(len(n), np.int32)
        if dt == np.float64:
            # The double oracle batch solves one column: compare the factors only.
            oracle.chol_solve_batched(n, a_off, oa, b_off, np.zeros(btot), oinfo, 4)
            ob = None
        else:
            oracle.chol_solve_batched(n, a_off, oa, b_off, ob, oinfo, 4, nrhs=nrhs)
        da, db = _dev(a), _dev(b)
        dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
        batch.run(da, db, dinfo)
        mf.context().synchronize()
        np.testing.assert_array_equal(_host(dinfo), oinfo)
        assert_bits(_flat(_host(da)), _flat(oa), dt.__name__)
        if ob is not None:
            assert_bits(_flat(_host(db)), _flat(ob), dt.__name__)
    batch.close()

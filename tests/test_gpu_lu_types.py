"""Batched LU + solve of MatFlat's float and Complex overloads: bit-identical to the oracle's
Factorization.Lu float / Complex followed by SolveTriangular of the same type, through the C ABI.
One plan runs all three element types in turn (the graph cache keys on the type)."""
import numpy as np
import pytest

from oracle import oracle
from tests.test_gpu_parity import _dev, _host, assert_bits

pytestmark = pytest.mark.gpu


def _packed(n, cols):
    sz = n.astype(np.int64) * cols
    return np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64), int(sz.sum())


def _batch(rng, count, nrhs, dt, nmax=150):
    n = rng.integers(1, nmax + 1, size=count).astype(np.int32)
    n[:6] = [1, 2, 3, 128, 129, nmax]            # shared-memory and global-scratch orders
    a_off, atot = _packed(n, n)
    piv_off, ptot = _packed(n, np.ones_like(n))
    b_off, btot = _packed(n, np.full_like(n, nrhs))

    def draw(k):
        if dt == np.complex128:
            return rng.standard_normal(k) + 1j * rng.standard_normal(k)
        return rng.standard_normal(k).astype(dt)

    a, b = draw(atot), draw(btot)
    # Singular and special matrices: a zero column (info), a NaN, an infinity, exact integers.
    o = a_off[6]
    a[o:o + n[6]] = 0
    a[a_off[7]] = np.nan
    a[a_off[8] + n[8] - 1] = np.inf
    o, k = a_off[9], int(n[9]) ** 2
    a[o:o + k] = rng.integers(-3, 4, size=k).astype(a.dtype)
    return n, a_off, piv_off, b_off, a, b, ptot


def _oracle(n, a_off, piv_off, b_off, a, b, nrhs, ptot):
    oa, ob = a.copy(), b.copy()
    opiv = np.zeros(ptot, np.int32)
    osign = np.zeros(len(n), np.int32)
    oracle.lu_solve_batched(n, a_off, oa, piv_off, opiv, b_off, ob, nrhs, osign, 4)
    return oa, ob, opiv, osign


def _flat(x):
    return x.view(np.float64) if x.dtype == np.complex128 else x


@pytest.mark.parametrize("dt", [np.float32, np.complex128])
@pytest.mark.parametrize("nrhs", [0, 5])
def test_lu_batched_types(mf, dt, nrhs):
    import torch
    rng = np.random.default_rng(300 + nrhs + (1 if dt == np.complex128 else 0))
    n, a_off, piv_off, b_off, a, b, ptot = _batch(rng, 700, max(nrhs, 1), dt)
    oa, ob, opiv, osign = _oracle(n, a_off, piv_off, b_off, a, b, nrhs, ptot)
    batch = mf.LuBatch(n, a_off, piv_off, nrhs=nrhs, b_off=b_off if nrhs else None)
    da, db = _dev(a), _dev(b)
    dpiv = torch.zeros(ptot, dtype=torch.int32, device="cuda")
    dsign = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    dinfo = torch.full((len(n),), -1, dtype=torch.int32, device="cuda")
    batch.run(da, dpiv, db if nrhs else None, dsign, dinfo)
    mf.context().synchronize()
    assert_bits(_flat(_host(da)), _flat(oa))
    np.testing.assert_array_equal(_host(dpiv), opiv)
    np.testing.assert_array_equal(_host(dsign), osign)
    if nrhs:
        assert_bits(_flat(_host(db)), _flat(ob))
    info = _host(dinfo)
    assert info[6] == 1                           # zero first column
    assert (info >= 0).all()
    batch.close()


def test_lu_batched_types_share_a_plan(mf):
    """double, float and Complex launches of one plan, then the solve-only forms of each."""
    import torch
    rng = np.random.default_rng(310)
    nrhs = 3
    n = rng.integers(1, 140, size=400).astype(np.int32)
    n[:2] = [139, 130]
    a_off, atot = _packed(n, n)
    piv_off, ptot = _packed(n, np.ones_like(n))
    b_off, btot = _packed(n, np.full_like(n, nrhs))
    batch = mf.LuBatch(n, a_off, piv_off, nrhs=nrhs, b_off=b_off)
    for rep in range(2):
        for dt in (np.float64, np.complex128, np.float32):
            if dt == np.complex128:
                a = rng.standard_normal(atot) + 1j * rng.standard_normal(atot)
                b = rng.standard_normal(btot) + 1j * rng.standard_normal(btot)
            else:
                a = rng.standard_normal(atot).astype(dt)
                b = rng.standard_normal(btot).astype(dt)
            oa, ob, opiv, osign = _oracle(n, a_off, piv_off, b_off, a, b, nrhs, ptot)
            da, db = _dev(a), _dev(b)
            dpiv = torch.zeros(ptot, dtype=torch.int32, device="cuda")
            dsign = torch.zeros(len(n), dtype=torch.int32, device="cuda")
            dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
            batch.run(da, dpiv, db, dsign, dinfo)
            mf.context().synchronize()
            assert_bits(_flat(_host(da)), _flat(oa), "%s rep %d" % (dt.__name__, rep))
            assert_bits(_flat(_host(db)), _flat(ob), "%s rep %d" % (dt.__name__, rep))
            np.testing.assert_array_equal(_host(dsign), osign)
            # The solve alone from the factors reproduces the fused solutions.
            db2 = _dev(b)
            batch.solve(da, dpiv, db2)
            mf.context().synchronize()
            assert_bits(_flat(_host(db2)), _flat(ob), "%s solve-only" % dt.__name__)
    # Complex held as interleaved float64 selects the Complex overload explicitly.
    a = rng.standard_normal(atot) + 1j * rng.standard_normal(atot)
    b = rng.standard_normal(btot) + 1j * rng.standard_normal(btot)
    oa, ob, opiv, osign = _oracle(n, a_off, piv_off, b_off, a, b, nrhs, ptot)
    da, db = _dev(a.view(np.float64)), _dev(b.view(np.float64))
    dpiv = torch.zeros(ptot, dtype=torch.int32, device="cuda")
    dsign = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    batch.run(da, dpiv, db, dsign, dinfo, dtype="z")
    mf.context().synchronize()
    assert_bits(_host(da), oa.view(np.float64))
    assert_bits(_host(db), ob.view(np.float64))
    batch.close()


def test_complex_unit_lower_divides_by_one(mf):
    """MatFlat's unit-lower idiom divides by an explicit Complex(1, 0); for Complex that division
    is not the identity on signed zeros, and the batched solve must reproduce it."""
    import torch
    n = np.array([1, 3, 4], np.int32)
    a_off = np.array([0, 1, 10], np.int64)
    piv_off = np.array([0, 1, 4], np.int64)
    b_off = np.array([0, 2, 8], np.int64)
    a = np.zeros(26, np.complex128)
    a[0] = 1.0
    a[1:10] = np.diag([1.0, 2.0, 1.0 + 1.0j]).flatten(order="F")
    a[10:26] = (np.eye(4) + np.tril(np.full((4, 4), 0.5), -1)).flatten(order="F")
    b = np.full(16, complex(-0.0, -0.0))
    b[3] = complex(-0.0, 1.0)
    b[9] = complex(1.0, -0.0)
    oa, ob, opiv, osign = _oracle(n, a_off, piv_off, b_off, a, b, 2, 8)
    batch = mf.LuBatch(n, a_off, piv_off, nrhs=2, b_off=b_off)
    da, db = _dev(a), _dev(b)
    dpiv = torch.zeros(8, dtype=torch.int32, device="cuda")
    dsign = torch.zeros(3, dtype=torch.int32, device="cuda")
    dinfo = torch.zeros(3, dtype=torch.int32, device="cuda")
    batch.run(da, dpiv, db, dsign, dinfo)
    mf.context().synchronize()
    assert_bits(_host(da).view(np.float64), oa.view(np.float64))
    assert_bits(_host(db).view(np.float64), ob.view(np.float64))
    assert np.signbit(ob.view(np.float64)).any() and not np.signbit(ob.view(np.float64)).all()


@pytest.mark.parametrize("dt", [np.float32, np.complex128])
def test_lu_inverse_batched_types(mf, dt):
    """Batched LuInverse, float and Complex: the inverse of the factors of every matrix, bit for
    bit against the oracle, with singular factors (info) and a double run on the same plan."""
    import torch
    rng = np.random.default_rng(330 + (dt == np.complex128))
    n = rng.integers(1, 150, size=300).astype(np.int32)
    n[:3] = [1, 129, 149]
    a_off, atot = _packed(n, n)
    piv_off, ptot = _packed(n, np.ones_like(n))
    if dt == np.complex128:
        a = rng.standard_normal(atot) + 1j * rng.standard_normal(atot)
    else:
        a = rng.standard_normal(atot).astype(dt)
    piv = np.zeros(ptot, np.int32)
    for i in range(len(n)):
        ni = int(n[i])
        ai = a[a_off[i]:a_off[i] + ni * ni]
        oracle.lu(ni, ni, ai, ni, piv[piv_off[i]:piv_off[i] + ni])
    a[a_off[5] + int(n[5]) * 2 + 2 if n[5] > 2 else a_off[5]] = 0    # a zero diagonal entry
    oa = a.copy()
    oinfo = np.zeros(len(n), np.int32)
    oracle.lu_inverse_batched(n, a_off, oa, piv_off, piv, oinfo, 4)
    assert oinfo[5] > 0
    batch = mf.LuInverseBatch(n, a_off, piv_off)
    da, dpiv = _dev(a), _dev(piv)
    dinfo = torch.full((len(n),), -7, dtype=torch.int32, device="cuda")
    batch.run(da, dpiv, dinfo)
    mf.context().synchronize()
    np.testing.assert_array_equal(_host(dinfo), oinfo)
    assert_bits(_flat(_host(da)), _flat(oa))
    # The double overload on the same plan afterwards.
    d = rng.standard_normal(atot)
    dp = np.zeros(ptot, np.int32)
    for i in range(len(n)):
        ni = int(n[i])
        oracle.lu(ni, ni, d[a_off[i]:a_off[i] + ni * ni], ni, dp[piv_off[i]:piv_off[i] + ni])
    od = d.copy()
    oinfo = np.zeros(len(n), np.int32)
    oracle.lu_inverse_batched(n, a_off, od, piv_off, dp, oinfo, 4)
    dd, ddp = _dev(d), _dev(dp)
    batch.run(dd, ddp, dinfo)
    mf.context().synchronize()
    assert_bits(_host(dd), od)
    batch.close()

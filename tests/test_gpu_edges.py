"""Edge cases of the batched paths: special values inside batches (NaN, infinities, signed zeros,
subnormals, products that overflow or underflow — the integer-pipe product's fallbacks) and empty
batches."""
import numpy as np
import pytest

from oracle import oracle
from tests.test_gpu_parity import _dev, _host, assert_bits

pytestmark = pytest.mark.gpu


def _special_batch(rng, count):
    n = rng.integers(1, 70, size=count).astype(np.int32)
    sz = n.astype(np.int64) ** 2
    off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    a = rng.standard_normal(int(sz.sum()))
    kinds = [np.nan, np.inf, -np.inf, 0.0, -0.0, 1e-310, -4e-320, 1e300, -1e300, 1e-300, 5e-324]
    for i in range(count):
        blk = a[off[i]:off[i] + sz[i]]
        if i % 3 == 0:
            continue                                   # ordinary matrices between the others
        k = int(rng.integers(1, 4))
        pos = rng.integers(0, sz[i], size=k)
        blk[pos] = rng.choice(kinds, size=k)
        if i % 5 == 1:
            with np.errstate(over="ignore"):
                blk *= rng.choice([1e150, 1e-150])     # products near the exponent limits
    return n, off, a


def test_lu_batched_special_values(mf):
    import torch
    rng = np.random.default_rng(91)
    n, off, a = _special_batch(rng, 400)
    piv_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]]).astype(np.int64)
    b_off = piv_off * 2
    b = rng.standard_normal(int(n.sum()) * 2)
    oa, ob = a.copy(), b.copy()
    opiv = np.zeros(int(n.sum()), np.int32)
    osign = np.zeros(len(n), np.int32)
    oracle.lu_solve_batched(n, off, oa, piv_off, opiv, b_off, ob, 2, osign, 4)
    batch = mf.LuBatch(n, off, piv_off, nrhs=2, b_off=b_off)
    for mode in ("default", "autotuned"):
        if mode == "autotuned":
            batch.autotune()
        da, db = _dev(a), _dev(b)
        dpiv = torch.zeros(int(n.sum()), dtype=torch.int32, device="cuda")
        dsign = torch.zeros(len(n), dtype=torch.int32, device="cuda")
        dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
        batch.run(da, dpiv, db, dsign, dinfo)
        mf.context().synchronize()
        assert_bits(_host(da), oa, mode)
        np.testing.assert_array_equal(_host(dpiv), opiv)
        np.testing.assert_array_equal(_host(dsign), osign)
        assert_bits(_host(db), ob, mode)


def test_cholesky_batched_special_values(mf):
    import torch
    rng = np.random.default_rng(92)
    n = rng.integers(1, 60, size=300).astype(np.int32)
    mats = []
    for i, ni in enumerate(n):
        m = rng.standard_normal((ni, ni))
        s = m @ m.T + ni * np.eye(ni)
        if i % 4 == 1:
            s[rng.integers(0, ni), rng.integers(0, ni)] = rng.choice([np.nan, np.inf, -np.inf])
        elif i % 4 == 2:
            s *= rng.choice([1e-300, 1e300, 1e-160])
        mats.append(s.flatten(order="F"))
    sz = n.astype(np.int64) ** 2
    off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    a = np.concatenate(mats)
    b_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]]).astype(np.int64)
    b = rng.standard_normal(int(n.sum()))
    oa, ob = a.copy(), b.copy()
    oinfo = np.zeros(len(n), np.int32)
    oracle.chol_solve_batched(n, off, oa, b_off, ob, oinfo, 4)
    batch = mf.CholeskyBatch(n, off, nrhs=1, b_off=b_off)
    da, db = _dev(a), _dev(b)
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    batch.run(da, db, dinfo)
    mf.context().synchronize()
    info = _host(dinfo)
    np.testing.assert_array_equal(info, oinfo)
    ga, gb = _host(da), _host(db)
    for i in range(len(n)):
        if oinfo[i] == 0:
            s = slice(off[i], off[i] + sz[i])
            assert_bits(ga[s], oa[s], "L %d" % i)
            bs = slice(b_off[i], b_off[i] + n[i])
            assert_bits(gb[bs], ob[bs], "x %d" % i)


def test_empty_batches(mf):
    import torch
    z = np.zeros(0, np.int32)
    zl = np.zeros(0, np.int64)
    t = torch.zeros(1, dtype=torch.float64, device="cuda")
    ti = torch.zeros(1, dtype=torch.int32, device="cuda")
    mf.LuBatch(z, zl, zl, nrhs=1, b_off=zl).run(t, ti, t, ti, ti)
    mf.CholeskyBatch(z, zl, nrhs=1, b_off=zl).run(t, t, ti)
    mf.QrBatch(z, z, zl, zl, nrhs=1, b_off=zl).run(t, t, t)
    mf.LuInverseBatch(z, zl, zl).run(t, ti, ti)
    mf.GevdFrontBatch(z, zl, zl, zl).run(t, t, t, ti)
    lb = mf.LuBatch(z, zl, zl)
    lb.run_host(np.zeros(1), np.zeros(1, np.int32), None, np.zeros(1, np.int32),
                np.zeros(1, np.int32))
    mf.context().synchronize()

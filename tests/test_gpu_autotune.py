"""The launch-shape autotuner: whatever shape it picks, results stay bit-identical to the oracle,
and later plans of the same size bucket (which start from the recorded shape) do too."""
import numpy as np
import pytest

from oracle import oracle
from tests.test_gpu_parity import _dev, _host, assert_bits

pytestmark = pytest.mark.gpu


def _packed(n, cols):
    sz = n.astype(np.int64) * cols
    return np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64), int(sz.sum())


def _lu_case(rng, count):
    n = rng.integers(1, 141, size=count).astype(np.int32)
    n[:2] = [129, 140]                          # global scratch, which a reshape must regrow
    a_off, atot = _packed(n, n)
    piv_off, ptot = _packed(n, np.ones_like(n))
    b_off, btot = _packed(n, np.full_like(n, 2))
    return n, a_off, piv_off, b_off, rng.standard_normal(atot), rng.standard_normal(btot), ptot


def test_autotune_getrf(mf):
    import torch
    rng = np.random.default_rng(41)
    n, a_off, piv_off, b_off, a, b, ptot = _lu_case(rng, 3000)
    oa, ob = a.copy(), b.copy()
    opiv = np.zeros(ptot, np.int32)
    osign = np.zeros(len(n), np.int32)
    oracle.lu_solve_batched(n, a_off, oa, piv_off, opiv, b_off, ob, 2, osign, 4)
    for round_ in range(2):      # the second plan starts from the recorded shape
        batch = mf.LuBatch(n, a_off, piv_off, nrhs=2, b_off=b_off)
        if round_ == 0:
            cfg = batch.autotune()
            assert len(cfg) == 5 and cfg[0] in (4, 8) and cfg[1] in (24, 28, 32)
            assert cfg[2] in (0, 2, 4, 5, 6)           # the lanes table of the size buckets
            assert cfg[3] in (0, 2) and cfg[4] in (2, 4)
        da, db = _dev(a), _dev(b)
        dpiv = torch.zeros(ptot, dtype=torch.int32, device="cuda")
        dsign = torch.zeros(len(n), dtype=torch.int32, device="cuda")
        dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
        batch.run(da, dpiv, db, dsign, dinfo)
        mf.context().synchronize()
        assert_bits(_host(da), oa)
        np.testing.assert_array_equal(_host(dpiv), opiv)
        assert_bits(_host(db), ob)
        batch.close()


def test_autotune_potrf(mf):
    import torch
    rng = np.random.default_rng(42)
    n = rng.integers(1, 140, size=1500).astype(np.int32)
    mats = []
    for ni in n:
        bm = rng.standard_normal((ni, ni))
        mats.append((bm @ bm.T + ni * np.eye(ni)).flatten(order="F"))
    a = np.concatenate(mats)
    a_off, _ = _packed(n, n)
    b_off, btot = _packed(n, np.ones_like(n))
    b = rng.standard_normal(btot)
    oa, ob = a.copy(), b.copy()
    oinfo = np.zeros(len(n), np.int32)
    oracle.chol_solve_batched(n, a_off, oa, b_off, ob, oinfo, 4)
    batch = mf.CholeskyBatch(n, a_off, nrhs=1, b_off=b_off)
    cfg = batch.autotune()
    assert cfg[2] in (4, 8, 16, 32, -1, -2) and cfg[3] in (0, 1)   # -t: lanes by size bucket
    da, db = _dev(a), _dev(b)
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    batch.run(da, db, dinfo)
    mf.context().synchronize()
    assert_bits(_host(da), oa)
    assert_bits(_host(db), ob)
    np.testing.assert_array_equal(_host(dinfo), oinfo)


def test_autotune_rejects_other_plans(mf):
    n = np.array([3, 4], np.int32)
    a_off, _ = _packed(n, n)
    piv_off, _ = _packed(n, np.ones_like(n))
    batch = mf.LuInverseBatch(n, a_off, piv_off)
    with pytest.raises(RuntimeError):
        batch.autotune()


def test_autotune_geqrf(mf):
    """QR plans: the autotuner picks lanes per matrix and warps per SM for the plan's (m, n) mix;
    the factors stay bit-identical to the oracle (double and float overloads), and a later plan
    of the same size bucket, which starts from the recorded shape, too."""
    import torch
    rng = np.random.default_rng(43)
    count = 600
    m = rng.integers(64, 300, size=count).astype(np.int32)
    n = np.minimum(rng.integers(16, 65, size=count), m).astype(np.int32)
    a_off, atot = _packed(m, n)
    r_off, rtot = _packed(n, np.ones_like(n))
    b_off, btot = _packed(m, np.ones_like(m))
    a = rng.standard_normal(atot)
    b = rng.standard_normal(btot)
    exp_a, exp_r = a.copy(), np.zeros(rtot)
    for i in range(count):
        ai = exp_a[a_off[i]:a_off[i] + m[i] * n[i]]
        ri = exp_r[r_off[i]:r_off[i] + n[i]]
        oracle.qr(int(m[i]), int(n[i]), ai, int(m[i]), ri)
    for round_ in range(2):
        batch = mf.QrBatch(m, n, a_off, r_off, nrhs=1, b_off=b_off)
        if round_ == 0:
            cfg = batch.autotune()
            assert cfg[2] in (4, 8, 16, 32) and cfg[1] in (8, 12, 16, 24)
        for dtype in (np.float64, np.float32):
            da, db = _dev(a.astype(dtype)), _dev(b.astype(dtype))
            dr = torch.zeros(rtot, dtype=da.dtype, device="cuda")
            batch.run(da, dr, db, single=(dtype == np.float32))
            mf.context().synchronize()
            if dtype == np.float64:
                assert_bits(_host(da), exp_a)
                assert_bits(_host(dr), exp_r)
            else:
                ea, er = a.astype(np.float32), np.zeros(rtot, np.float32)
                for i in range(0, count, 37):
                    ai = ea[a_off[i]:a_off[i] + m[i] * n[i]]
                    ri = er[r_off[i]:r_off[i] + n[i]]
                    oracle.qr(int(m[i]), int(n[i]), ai, int(m[i]), ri)
                    assert_bits(_host(da)[a_off[i]:a_off[i] + m[i] * n[i]], ai)
        batch.close()

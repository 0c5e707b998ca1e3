"""Solve-only batched entry points (getrs / potrs / geqrs) against the fused factor+solve path.

Solving with the factors of an earlier call must give the same bits as the fused path, which is
itself checked against the oracle in test_gpu_parity.
"""
import numpy as np
import pytest

from oracle import oracle
from tests.test_gpu_parity import _dev, _host, assert_bits

pytestmark = pytest.mark.gpu


def _packed(n, cols):
    sz = n.astype(np.int64) * cols
    return np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64), int(sz.sum())


def test_getrs_batched_matches_fused(mf):
    import torch
    rng = np.random.default_rng(31)
    n = rng.integers(1, 150, size=150).astype(np.int32)
    nrhs = 3
    a_off, atot = _packed(n, n)
    piv_off, ptot = _packed(n, np.ones_like(n))
    b_off, btot = _packed(n, np.full_like(n, nrhs))
    a = rng.standard_normal(atot)
    b = rng.standard_normal(btot)
    batch = mf.LuBatch(n, a_off, piv_off, nrhs=nrhs, b_off=b_off)
    da, db = _dev(a), _dev(b)
    dpiv = torch.zeros(ptot, dtype=torch.int32, device="cuda")
    dsign = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    batch.run(da, dpiv, db, dsign, dinfo)
    mf.context().synchronize()
    fused = _host(db)
    b2 = _dev(b)
    for _ in range(2):          # the second call replays the captured graph
        b2.copy_(_dev(b))
        torch.cuda.synchronize()     # the copy runs on torch's stream, the plan on its own
        batch.solve(da, dpiv, b2)
        mf.context().synchronize()
    assert_bits(_host(b2), fused)
    # and the oracle's composition
    oa, ob = a.copy(), b.copy()
    opiv = np.zeros(ptot, np.int32)
    osign = np.zeros(len(n), np.int32)
    oracle.lu_solve_batched(n, a_off, oa, piv_off, opiv, b_off, ob, nrhs, osign, 4)
    assert_bits(_host(b2), ob)
    # factoring again after a solve recaptures the factorization graph
    da.copy_(_dev(a))
    db.copy_(_dev(b))
    torch.cuda.synchronize()
    batch.run(da, dpiv, db, dsign, dinfo)
    mf.context().synchronize()
    assert_bits(_host(db), fused)


def test_potrs_batched_matches_fused(mf):
    import torch
    rng = np.random.default_rng(32)
    n = rng.integers(1, 100, size=120).astype(np.int32)
    nrhs = 2
    mats = []
    for ni in n:
        bm = rng.standard_normal((ni, ni))
        mats.append((bm @ bm.T + ni * np.eye(ni)).flatten(order="F"))
    a_off, atot = _packed(n, n)
    a = np.concatenate(mats)
    b_off, btot = _packed(n, np.full_like(n, nrhs))
    b = rng.standard_normal(btot)
    batch = mf.CholeskyBatch(n, a_off, nrhs=nrhs, b_off=b_off)
    da, db = _dev(a), _dev(b)
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    batch.run(da, db, dinfo)
    mf.context().synchronize()
    assert (_host(dinfo) == 0).all()
    fused = _host(db)
    b2 = _dev(b)
    batch.solve(da, b2)
    mf.context().synchronize()
    assert_bits(_host(b2), fused)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_geqrs_batched_matches_fused(mf, dtype):
    import torch
    rng = np.random.default_rng(33)
    count = 100
    m = rng.integers(1, 300, size=count).astype(np.int32)
    n = np.minimum(rng.integers(1, 70, size=count), m).astype(np.int32)
    nrhs = 2
    a_off, atot = _packed(m, n)
    r_off, rtot = _packed(n, np.ones_like(n))
    b_off, btot = _packed(m, np.full_like(m, nrhs))
    a = rng.standard_normal(atot).astype(dtype)
    b = rng.standard_normal(btot).astype(dtype)
    a[a_off[5]:a_off[5] + m[5] * n[5]] = 0.0      # zero matrix: no reflectors
    batch = mf.QrBatch(m, n, a_off, r_off, nrhs=nrhs, b_off=b_off)
    single = dtype == np.float32
    da, db = _dev(a), _dev(b)
    dr = torch.zeros(rtot, dtype=da.dtype, device="cuda")
    batch.run(da, dr, db, single=single)
    mf.context().synchronize()
    fused = _host(db)
    b2 = _dev(b)
    batch.solve(da, dr, b2, single=single)
    mf.context().synchronize()
    assert_bits(_host(b2), fused)


def test_solve_needs_right_hand_sides(mf):
    import torch
    n = np.array([4, 5], np.int32)
    a_off, _ = _packed(n, n)
    piv_off, _ = _packed(n, np.ones_like(n))
    batch = mf.LuBatch(n, a_off, piv_off)
    z = torch.zeros(64, dtype=torch.float64, device="cuda")
    zi = torch.zeros(16, dtype=torch.int32, device="cuda")
    with pytest.raises(RuntimeError):
        batch.solve(z, zi, z)

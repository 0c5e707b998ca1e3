"""Host-buffer batched LU (pipelined copies and compute) against the device-buffer path."""
import numpy as np
import pytest

from tests.test_gpu_parity import _dev, _host, assert_bits

pytestmark = pytest.mark.gpu


def _case(rng, count, reverse=False):
    n = rng.integers(1, 141, size=count).astype(np.int32)
    sz = n.astype(np.int64) ** 2
    order = np.arange(count)[::-1] if reverse else np.arange(count)
    a_off = np.zeros(count, np.int64)
    piv_off = np.zeros(count, np.int64)
    b_off = np.zeros(count, np.int64)
    at = pt = bt = 0
    for i in order:                        # reversed: later matrices first in memory
        a_off[i], piv_off[i], b_off[i] = at, pt, bt
        at += sz[i]
        pt += n[i]
        bt += 2 * n[i]
    return n, a_off, piv_off, b_off, rng.standard_normal(at), rng.standard_normal(bt), pt


@pytest.mark.parametrize("reverse", [False, True])
def test_host_pipeline_matches_device_path(mf, reverse):
    import torch
    rng = np.random.default_rng(61 + reverse)
    n, a_off, piv_off, b_off, a, b, ptot = _case(rng, 20000 if not reverse else 9000, reverse)
    count = len(n)
    batch = mf.LuBatch(n, a_off, piv_off, nrhs=2, b_off=b_off)
    da, db = _dev(a), _dev(b)
    dpiv = torch.zeros(ptot, dtype=torch.int32, device="cuda")
    dsign = torch.zeros(count, dtype=torch.int32, device="cuda")
    dinfo = torch.zeros(count, dtype=torch.int32, device="cuda")
    batch.run(da, dpiv, db, dsign, dinfo)
    mf.context().synchronize()
    # pageable numpy arrays
    ha, hb = a.copy(), b.copy()
    hpiv = np.zeros(ptot, np.int32)
    hsign = np.zeros(count, np.int32)
    hinfo = np.zeros(count, np.int32)
    batch.run_host(ha, hpiv, hb, hsign, hinfo)
    assert_bits(ha, _host(da))
    assert_bits(hb, _host(db))
    np.testing.assert_array_equal(hpiv, _host(dpiv))
    np.testing.assert_array_equal(hsign, _host(dsign))
    np.testing.assert_array_equal(hinfo, _host(dinfo))
    # page-locked tensors, twice (the second call reuses the chunk plans)
    for _ in range(2):
        ta = torch.from_numpy(a.copy()).pin_memory()
        tb = torch.from_numpy(b.copy()).pin_memory()
        tp = torch.zeros(ptot, dtype=torch.int32).pin_memory()
        ts = torch.zeros(count, dtype=torch.int32).pin_memory()
        ti = torch.zeros(count, dtype=torch.int32).pin_memory()
        batch.run_host(ta, tp, tb, ts, ti)
        assert_bits(ta.numpy(), ha)
        assert_bits(tb.numpy(), hb)
        np.testing.assert_array_equal(tp.numpy(), hpiv)


def _pinned(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x).copy()).pin_memory()


def test_host_pipeline_other_operations(mf):
    """Every batched operation's host-buffer form equals its device-buffer form bit for bit
    (batches above 8,192 matrices, so the pipeline has at least two chunks)."""
    import torch
    from workloads import synth
    count = 9000
    # Cholesky + solve
    d = synth.spd_batch(count, 24, nrhs=1, seed=5)
    plan = mf.CholeskyBatch(d["n"], d["a_off"], nrhs=1, b_off=d["b_off"])
    da, db = _dev(d["a"]), _dev(d["b"])
    di = torch.zeros(count, dtype=torch.int32, device="cuda")
    plan.run(da, db, di)
    ha, hb, hi = _pinned(d["a"]), _pinned(d["b"]), _pinned(np.zeros(count, np.int32))
    plan.run_host(ha, hb, hi)
    assert_bits(ha.numpy(), _host(da))
    assert_bits(hb.numpy(), _host(db))
    # loss and gradient, both factor modes
    r = synth.rbf_batch(count, 24, seed=6)
    gp = mf.CholeskyBatch(r["n"], r["a_off"], nrhs=1, b_off=r["b_off"])
    for keep in (True, False):
        dk, dy = _dev(r["a"]), _dev(r["b"])
        dl = torch.zeros(count, dtype=torch.float64, device="cuda")
        dg = torch.zeros_like(dk)
        dinf = torch.zeros(count, dtype=torch.int32, device="cuda")
        gp.loss_and_grad(dk, dy, dl, dg, dinf, keep_factor=keep)
        hk, hy = _pinned(r["a"]), _pinned(r["b"])
        hl = _pinned(np.zeros(count))
        hg = _pinned(np.zeros_like(r["a"]))
        hinf = _pinned(np.zeros(count, np.int32))
        gp.loss_and_grad_host(hk, hy, hl, hg, hinf, keep_factor=keep)
        assert_bits(hk.numpy(), _host(dk))
        assert_bits(hy.numpy(), _host(dy))
        assert_bits(hl.numpy(), _host(dl))
        assert_bits(hg.numpy(), _host(dg))
        np.testing.assert_array_equal(hinf.numpy(), _host(dinf))
    # LuInverse of LU factors
    lu = synth.lu_batch(count, 4, 40, 0, seed=7)
    lp = mf.LuBatch(lu["n"], lu["a_off"], lu["piv_off"])
    fa = _dev(lu["a"])
    fp = torch.zeros(lu["piv_total"], dtype=torch.int32, device="cuda")
    fs = torch.zeros(count, dtype=torch.int32, device="cuda")
    fi = torch.zeros(count, dtype=torch.int32, device="cuda")
    lp.run(fa, fp, None, fs, fi)
    mf.context().synchronize()
    fac, piv = _host(fa), _host(fp)
    ip = mf.LuInverseBatch(lu["n"], lu["a_off"], lu["piv_off"])
    ia, ipv = _dev(fac), _dev(piv)
    iinf = torch.zeros(count, dtype=torch.int32, device="cuda")
    ip.run(ia, ipv, iinf)
    ha, hinf = _pinned(fac), _pinned(np.zeros(count, np.int32))
    ip.run_host(ha, _pinned(piv), hinf)
    assert_bits(ha.numpy(), _host(ia))
    np.testing.assert_array_equal(hinf.numpy(), _host(iinf))
    # QR + least squares, double and float
    q = synth.qr_batch(count, 16, 96, 4, 16, nrhs=1, seed=8)
    qp = mf.QrBatch(q["m"], q["n"], q["a_off"], q["rdiag_off"], nrhs=1, b_off=q["b_off"])
    for dt, single in ((np.float64, False), (np.float32, True)):
        qa, qb = _dev(q["a"].astype(dt)), _dev(q["b"].astype(dt))
        qr_ = torch.zeros(q["rdiag_total"], dtype=qa.dtype, device="cuda")
        qp.run(qa, qr_, qb, single=single)
        ha, hb = _pinned(q["a"].astype(dt)), _pinned(q["b"].astype(dt))
        hr = _pinned(np.zeros(q["rdiag_total"], dt))
        qp.run_host(ha, hr, hb, single=single)
        assert_bits(ha.numpy(), _host(qa))
        assert_bits(hr.numpy(), _host(qr_))
        assert_bits(hb.numpy(), _host(qb))
    # GEVD front half
    g = synth.gevd_batch(count, 12, seed=9)
    vp = mf.GevdFrontBatch(g["n"], g["a_off"], g["b_off"], g["a_off"])
    va, vb = _dev(g["a"]), _dev(g["b"])
    vc = torch.zeros_like(va)
    vi = torch.zeros(count, dtype=torch.int32, device="cuda")
    vp.run(va, vb, vc, vi)
    hb, hc, hinf = _pinned(g["b"]), _pinned(np.zeros_like(g["a"])), _pinned(np.zeros(count, np.int32))
    vp.run_host(_pinned(g["a"]), hb, hc, hinf)
    assert_bits(hb.numpy(), _host(vb))
    assert_bits(hc.numpy(), _host(vc))
    np.testing.assert_array_equal(hinf.numpy(), _host(vi))


def _flat(x):
    return x.view(np.float64) if x.dtype == np.complex128 else x


def _draw(rng, k, dt):
    if dt == np.complex128:
        return rng.standard_normal(k) + 1j * rng.standard_normal(k)
    return rng.standard_normal(k).astype(dt)


@pytest.mark.parametrize("dt", [np.float32, np.complex128])
def test_host_pipeline_float_complex(mf, dt):
    """The float and Complex host-buffer forms of the batched LU, Cholesky and (Complex) QR
    equal their device-buffer forms bit for bit (orders above 128 use the global scratch)."""
    import torch
    rng = np.random.default_rng(66 + (dt == np.complex128))
    count = 9000
    n = rng.integers(1, 141, size=count).astype(np.int32)
    a_off = np.concatenate([[0], np.cumsum(n.astype(np.int64) ** 2)[:-1]]).astype(np.int64)
    piv_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]]).astype(np.int64)
    b_off = np.concatenate([[0], np.cumsum(2 * n.astype(np.int64))[:-1]]).astype(np.int64)
    atot, ptot, btot = int((n.astype(np.int64) ** 2).sum()), int(n.sum()), int(2 * n.sum())
    # LU + 2-RHS solve
    a, b = _draw(rng, atot, dt), _draw(rng, btot, dt)
    lu = mf.LuBatch(n, a_off, piv_off, nrhs=2, b_off=b_off)
    da, db = _dev(a), _dev(b)
    dpiv = torch.zeros(ptot, dtype=torch.int32, device="cuda")
    dsign = torch.zeros(count, dtype=torch.int32, device="cuda")
    dinfo = torch.zeros(count, dtype=torch.int32, device="cuda")
    lu.run(da, dpiv, db, dsign, dinfo)
    mf.context().synchronize()
    ha, hb = a.copy(), b.copy()
    hpiv = np.zeros(ptot, np.int32)
    hsign = np.zeros(count, np.int32)
    hinfo = np.zeros(count, np.int32)
    lu.run_host(ha, hpiv, hb, hsign, hinfo)
    assert_bits(_flat(ha), _flat(_host(da)))
    assert_bits(_flat(hb), _flat(_host(db)))
    np.testing.assert_array_equal(hpiv, _host(dpiv))
    np.testing.assert_array_equal(hsign, _host(dsign))
    lu.close()
    # Cholesky + 2-RHS solve of Hermitian positive definite matrices
    mats = []
    for ni in n:                                # (B + B^H) / 2 + 2n I: positive definite
        m = _draw(rng, int(ni) * int(ni), dt).reshape(ni, ni)
        mats.append(((m + m.conj().T) / 2 + 2 * ni * np.eye(ni)).astype(dt).flatten(order="F"))
    s = np.concatenate(mats)
    ch = mf.CholeskyBatch(n, a_off, nrhs=2, b_off=b_off)
    ds, db = _dev(s), _dev(b)
    dinfo = torch.zeros(count, dtype=torch.int32, device="cuda")
    ch.run(ds, db, dinfo)
    mf.context().synchronize()
    hs, hb = s.copy(), b.copy()
    hinfo = np.zeros(count, np.int32)
    ch.run_host(hs, hb, hinfo)
    np.testing.assert_array_equal(hinfo, _host(dinfo))
    assert_bits(_flat(hs), _flat(_host(ds)))
    assert_bits(_flat(hb), _flat(_host(db)))
    ch.close()
    if dt != np.complex128:
        return
    # Complex QR + least squares (rdiag real)
    qn = rng.integers(1, 40, size=3000).astype(np.int32)
    qm = (qn + rng.integers(0, 100, size=3000)).astype(np.int32)
    sz = qm.astype(np.int64) * qn
    qa_off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    r_off = np.concatenate([[0], np.cumsum(qn.astype(np.int64))[:-1]]).astype(np.int64)
    qb_off = np.concatenate([[0], np.cumsum(qm.astype(np.int64))[:-1]]).astype(np.int64)
    qa, qb = _draw(rng, int(sz.sum()), dt), _draw(rng, int(qm.sum()), dt)
    qr = mf.QrBatch(qm, qn, qa_off, r_off, nrhs=1, b_off=qb_off)
    da, db = _dev(qa), _dev(qb)
    dr = torch.zeros(int(qn.sum()), dtype=torch.float64, device="cuda")
    qr.run(da, dr, db)
    mf.context().synchronize()
    ha, hb, hr = qa.copy(), qb.copy(), np.zeros(int(qn.sum()))
    qr.run_host(ha, hr, hb)
    assert_bits(_flat(ha), _flat(_host(da)))
    assert_bits(hr, _host(dr))
    assert_bits(_flat(hb), _flat(_host(db)))
    qr.close()

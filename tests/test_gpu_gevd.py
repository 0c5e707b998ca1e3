"""Batched GEVD front half on the GPU against the oracle, bit for bit (L and C)."""
import numpy as np
import pytest

from oracle import oracle
from tests.test_gpu_parity import _dev, _host, assert_bits

pytestmark = pytest.mark.gpu


def test_gevd_front_batched(mf):
    import torch
    rng = np.random.default_rng(71)
    n = rng.integers(1, 129, size=150).astype(np.int32)
    n[:4] = [1, 2, 127, 128]
    sz = n.astype(np.int64) ** 2
    off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    As, Bs = [], []
    for i, ni in enumerate(n):
        A = rng.standard_normal((ni, ni))
        M = rng.standard_normal((ni, ni))
        B = M @ M.T + ni * np.eye(ni)
        if i == 7:
            B[0, 0] = -1.0                       # not positive definite
        As.append(A.flatten(order="F"))
        Bs.append(B.flatten(order="F"))
    a, b = np.concatenate(As), np.concatenate(Bs)
    ob, oc = b.copy(), np.zeros_like(a)
    oinfo = np.zeros(len(n), np.int32)
    oracle.gevd_front_batched(n, off, a, off, ob, oc, oinfo, 4)
    plan = mf.GevdFrontBatch(n, off, off, off)
    da, db = _dev(a), _dev(b)
    dc = torch.zeros_like(da)
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    for _ in range(2):          # the second call replays the captured graph
        db.copy_(_dev(b))
        torch.cuda.synchronize()     # the copy runs on torch's stream, the plan on its own
        plan.run(da, db, dc, dinfo)
        mf.context().synchronize()
    info = _host(dinfo)
    np.testing.assert_array_equal(info, oinfo)
    assert info[7] == 1
    gb, gc = _host(db), _host(dc)
    assert_bits(_host(da), a)                     # A is read only
    for i in range(len(n)):
        s = slice(off[i], off[i] + sz[i])
        assert_bits(gb[s], ob[s], "L %d" % i)
        if info[i] == 0:
            assert_bits(gc[s], oc[s], "C %d" % i)


def test_gevd_front_leading_dimensions(mf):
    import torch
    rng = np.random.default_rng(72)
    n = np.array([3, 20, 45, 128], np.int32)
    lda = n + np.array([2, 0, 5, 1], np.int32)
    ldb = n + np.array([0, 3, 1, 4], np.int32)
    a_sz = lda.astype(np.int64) * n
    b_sz = ldb.astype(np.int64) * n
    a_off = np.concatenate([[0], np.cumsum(a_sz)[:-1]]).astype(np.int64)
    b_off = np.concatenate([[0], np.cumsum(b_sz)[:-1]]).astype(np.int64)
    c_off = np.concatenate([[0], np.cumsum(n.astype(np.int64) ** 2)[:-1]]).astype(np.int64)
    a = rng.standard_normal(int(a_sz.sum()))
    b = np.zeros(int(b_sz.sum()))
    for i, ni in enumerate(n):
        M = rng.standard_normal((ni, ni))
        B = np.full((ldb[i], ni), 99.0)
        B[:ni, :] = M @ M.T + ni * np.eye(ni)
        b[b_off[i]:b_off[i] + b_sz[i]] = B.flatten(order="F")
    ob, oc = b.copy(), np.zeros(int((n.astype(np.int64) ** 2).sum()))
    for i, ni in enumerate(n):
        assert oracle.gevd_front(int(ni), a[a_off[i]:a_off[i] + a_sz[i]], int(lda[i]),
                                 ob[b_off[i]:b_off[i] + b_sz[i]], int(ldb[i]),
                                 oc[c_off[i]:c_off[i] + ni * ni]) == 0
    plan = mf.GevdFrontBatch(n, a_off, b_off, c_off, lda=lda, ldb=ldb)
    da, db = _dev(a), _dev(b)
    dc = torch.zeros(len(oc), dtype=torch.float64, device="cuda")
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    plan.run(da, db, dc, dinfo)
    mf.context().synchronize()
    assert (_host(dinfo) == 0).all()
    assert_bits(_host(db), ob)                     # includes the padding rows, unchanged
    assert_bits(_host(dc), oc)


def _pairs(rng, n, dt, bad=()):
    """A (any values; only its upper triangle is read) and B (SPD / HPD) per pair, column-major."""
    As, Bs = [], []
    for i, ni in enumerate(n):
        if dt == np.complex128:
            A = rng.standard_normal((ni, ni)) + 1j * rng.standard_normal((ni, ni))
            M = rng.standard_normal((ni, ni)) + 1j * rng.standard_normal((ni, ni))
            B = M @ M.conj().T + ni * np.eye(ni)
        else:
            A = rng.standard_normal((ni, ni))
            M = rng.standard_normal((ni, ni))
            B = M @ M.T + ni * np.eye(ni)
        if i in bad:
            B[min(2, ni - 1), min(2, ni - 1)] = -1.0      # not positive definite
        As.append(A.astype(dt).flatten(order="F"))
        Bs.append(B.astype(dt).flatten(order="F"))
    return np.concatenate(As), np.concatenate(Bs)


def _flat(x):
    return x.view(np.float64) if x.dtype == np.complex128 else x


@pytest.mark.parametrize("dt", [np.float32, np.complex128])
def test_gevd_front_batched_types(mf, dt):
    """The float and Complex overloads (GevdCore float / Complex), bit for bit against the oracle,
    on one plan that also runs the double overload before and after (the graph is re-captured
    for each element type)."""
    import torch
    rng = np.random.default_rng(73 + (dt == np.complex128))
    n = rng.integers(1, 129, size=120).astype(np.int32)
    n[:5] = [1, 2, 8, 127, 128]
    sz = n.astype(np.int64) ** 2
    off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    plan = mf.GevdFrontBatch(n, off, off, off)
    for kind in (np.float64, dt, np.float64, dt):
        a, b = _pairs(rng, n, kind, bad=(9,))
        ob, oc = b.copy(), np.zeros_like(a)
        oinfo = np.zeros(len(n), np.int32)
        oracle.gevd_front_batched(n, off, a, off, ob, oc, oinfo, 4)
        assert oinfo[9] == min(3, n[9])
        da, db = _dev(a), _dev(b)
        dc = torch.zeros_like(da)
        dinfo = torch.full((len(n),), -5, dtype=torch.int32, device="cuda")
        plan.run(da, db, dc, dinfo)
        mf.context().synchronize()
        info = _host(dinfo)
        np.testing.assert_array_equal(info, oinfo)
        gb, gc = _host(db), _host(dc)
        assert_bits(_flat(_host(da)), _flat(a))           # A is read only
        for i in range(len(n)):
            # A pair whose B is not positive definite leaves B and C unspecified (MatFlat throws
            # with B partly factored, row by row; the kernel factors column by column).
            if info[i] == 0:
                s = slice(off[i], off[i] + sz[i])
                assert_bits(_flat(gb[s]), _flat(ob[s]), "%s L %d" % (kind.__name__, i))
                assert_bits(_flat(gc[s]), _flat(oc[s]), "%s C %d" % (kind.__name__, i))
    plan.close()


@pytest.mark.parametrize("dt", [np.float32, np.complex128])
def test_gevd_front_types_leading_dimensions(mf, dt):
    import torch
    rng = np.random.default_rng(75 + (dt == np.complex128))
    n = np.array([3, 20, 45, 128, 1], np.int32)
    lda = n + np.array([2, 0, 5, 1, 3], np.int32)
    ldb = n + np.array([0, 3, 1, 4, 2], np.int32)
    a_sz = lda.astype(np.int64) * n
    b_sz = ldb.astype(np.int64) * n
    a_off = np.concatenate([[0], np.cumsum(a_sz)[:-1]]).astype(np.int64)
    b_off = np.concatenate([[0], np.cumsum(b_sz)[:-1]]).astype(np.int64)
    c_off = np.concatenate([[0], np.cumsum(n.astype(np.int64) ** 2)[:-1]]).astype(np.int64)
    if dt == np.complex128:
        a = rng.standard_normal(int(a_sz.sum())) + 1j * rng.standard_normal(int(a_sz.sum()))
    else:
        a = rng.standard_normal(int(a_sz.sum())).astype(dt)
    b = np.zeros(int(b_sz.sum()), dt)
    for i, ni in enumerate(n):
        _, bi = _pairs(rng, [ni], dt)
        B = np.full((ldb[i], ni), 99.0, dt)
        B[:ni, :] = bi.reshape(ni, ni, order="F")
        b[b_off[i]:b_off[i] + b_sz[i]] = B.flatten(order="F")
    ob, oc = b.copy(), np.zeros(int((n.astype(np.int64) ** 2).sum()), dt)
    for i, ni in enumerate(n):
        assert oracle.gevd_front(int(ni), a[a_off[i]:a_off[i] + a_sz[i]], int(lda[i]),
                                 ob[b_off[i]:b_off[i] + b_sz[i]], int(ldb[i]),
                                 oc[c_off[i]:c_off[i] + ni * ni]) == 0
    plan = mf.GevdFrontBatch(n, a_off, b_off, c_off, lda=lda, ldb=ldb)
    da, db = _dev(a), _dev(b)
    dc = _dev(np.zeros_like(oc))
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    plan.run(da, db, dc, dinfo)
    mf.context().synchronize()
    assert (_host(dinfo) == 0).all()
    assert_bits(_flat(_host(db)), _flat(ob))       # includes the padding rows, unchanged
    assert_bits(_flat(_host(dc)), _flat(oc))
    # Complex held as interleaved float64 selects the Complex overload explicitly.
    if dt == np.complex128:
        da2, db2, dc2 = _dev(a.view(np.float64)), _dev(b.view(np.float64)), _dev(np.zeros(2 * len(oc)))
        plan.run(da2, db2, dc2, dinfo, dtype="z")
        mf.context().synchronize()
        assert_bits(_host(db2), ob.view(np.float64))
        assert_bits(_host(dc2), oc.view(np.float64))
    plan.close()


@pytest.mark.parametrize("dt", [np.float32, np.complex128])
def test_gevd_front_types_host(mf, dt):
    """The host-buffer forms (copies pipelined with compute) give the device forms' bits."""
    import torch
    rng = np.random.default_rng(77 + (dt == np.complex128))
    count = 2500
    n = rng.integers(1, 33, size=count).astype(np.int32)
    sz = n.astype(np.int64) ** 2
    off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    a, b = _pairs(rng, n, dt, bad=(4,))
    plan = mf.GevdFrontBatch(n, off, off, off)
    da, db = _dev(a), _dev(b)
    dc = torch.zeros_like(da)
    dinfo = torch.zeros(count, dtype=torch.int32, device="cuda")
    plan.run(da, db, dc, dinfo)
    mf.context().synchronize()
    hb, hc, hinf = b.copy(), np.zeros_like(a), np.zeros(count, np.int32)
    plan.run_host(a, hb, hc, hinf)
    np.testing.assert_array_equal(hinf, _host(dinfo))
    assert hinf[4] > 0
    ok = np.repeat(hinf == 0, sz)
    assert_bits(_flat(hb[ok]), _flat(_host(db)[ok]))
    assert_bits(_flat(hc[ok]), _flat(_host(dc)[ok]))
    plan.close()

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

"""Batched Factorization.LuInverse on the GPU against the oracle, bit for bit, through the C ABI.

The reference test (MatFlatTest/LuInverseTests.cs:85-135) checks A * A^-1 = I within 1e-12 and
that the padding beyond n rows is untouched; here the inverse is compared bit for bit with the
oracle's LuInverse (itself pinned to LAPACK by test_oracle_pin), including the sign of exact
zeros, NaN propagation through L, singular factors and leading dimensions larger than n.
"""
import numpy as np
import pytest

from oracle import oracle
from tests.test_gpu_parity import _dev, _host, assert_bits

pytestmark = pytest.mark.gpu


def _offsets(n, lda=None):
    lda = n if lda is None else lda
    sz = lda.astype(np.int64) * n
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    piv_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]]).astype(np.int64)
    return a_off, int(sz.sum()), piv_off


def _factor(mf, n, a_off, a, piv_off):
    """LU on the GPU (bit-identical to the oracle's); returns device factors and pivots."""
    import torch
    da = _dev(a)
    dpiv = torch.zeros(int(n.sum()), dtype=torch.int32, device="cuda")
    dsign = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    mf.LuBatch(n, a_off, piv_off).run(da, dpiv, None, dsign, dinfo)
    return da, dpiv


def _structured(rng, ni, kind):
    if kind == "perm":
        m = np.zeros((ni, ni))
        m[rng.permutation(ni), np.arange(ni)] = 1.0
    elif kind == "ternary":
        m = rng.integers(-1, 2, size=(ni, ni)).astype(np.float64) + 3.0 * np.eye(ni)
    elif kind == "lower":
        m = np.tril(rng.standard_normal((ni, ni))) + ni * np.eye(ni)
    elif kind == "blockdiag":
        h = ni // 2
        m = np.zeros((ni, ni))
        m[:h, :h] = rng.standard_normal((h, h))
        m[h:, h:] = rng.standard_normal((ni - h, ni - h))
    return m.flatten(order="F")


def test_lu_inverse_batched(mf):
    import torch
    rng = np.random.default_rng(21)
    n = rng.integers(1, 161, size=240).astype(np.int32)    # n > 128 stages columns in global
    n[:8] = [1, 2, 3, 31, 32, 33, 128, 129]
    a_off, total, piv_off = _offsets(n)
    a = rng.standard_normal(total)
    special = {10: "zero", 11: "zerocol", 12: "nan", 13: "perm", 14: "ternary", 15: "lower",
               16: "blockdiag", 17: "perm", 18: "inf"}
    for i, kind in special.items():
        ni = int(n[i])
        blk = a[a_off[i]:a_off[i] + ni * ni]
        if kind == "zero":
            blk[:] = 0.0
        elif kind == "zerocol":
            c = ni // 2
            blk[c * ni:(c + 1) * ni] = 0.0
        elif kind == "nan":
            blk[ni * (ni // 3) + ni - 1] = np.nan              # lands in L after pivoting
        elif kind == "inf":
            blk[ni * (ni // 4) + ni // 2] = np.inf
        else:
            blk[:] = _structured(rng, ni, kind)
    da, dpiv = _factor(mf, n, a_off, a, piv_off)
    fac, piv = _host(da), _host(dpiv)
    exp = fac.copy()
    einfo = np.zeros(len(n), np.int32)
    oracle.lu_inverse_batched(n, a_off, exp, piv_off, piv, einfo, 4)

    batch = mf.LuInverseBatch(n, a_off, piv_off)
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    for _ in range(2):   # twice: the second run replays the captured graph
        da.copy_(_dev(fac))
        torch.cuda.synchronize()     # the copy runs on torch's stream, the plan on its own
        batch.run(da, dpiv, dinfo)
        mf.context().synchronize()
    info = _host(dinfo)
    np.testing.assert_array_equal(info, einfo)
    assert info[10] == 1 and info[11] > 0 and info[0] == 0
    assert_bits(_host(da), exp)
    # Singular matrices are left untouched.
    got = _host(da)
    for i in (10, 11):
        ni = int(n[i])
        assert_bits(got[a_off[i]:a_off[i] + ni * ni], fac[a_off[i]:a_off[i] + ni * ni])
    # The reference suite's property: A * A^-1 = I within 1e-12 for well-conditioned inputs.
    for i in (0, 3, 6, 7, 14, 15):
        ni = int(n[i])
        m = a[a_off[i]:a_off[i] + ni * ni].reshape(ni, ni, order="F")
        inv = got[a_off[i]:a_off[i] + ni * ni].reshape(ni, ni, order="F")
        if np.linalg.cond(m) < 1e4:
            np.testing.assert_allclose(m @ inv, np.eye(ni), atol=1e-10 * ni)


def test_lu_inverse_lda_padding(mf):
    import torch
    rng = np.random.default_rng(22)
    n = np.array([5, 17, 40, 64, 130], np.int32)
    lda = n + np.array([3, 1, 8, 2, 5], np.int32)
    a_off, total, piv_off = _offsets(n, lda)
    a = rng.standard_normal(total)
    # Factor each matrix with the oracle (lda > n) and invert it there.
    piv = np.zeros(int(n.sum()), np.int32)
    fac = a.copy()
    for i, ni in enumerate(n):
        blk = fac[a_off[i]:a_off[i] + lda[i] * ni]
        oracle.lu(int(ni), int(ni), blk, int(lda[i]), piv[piv_off[i]:piv_off[i] + ni])
    exp = fac.copy()
    for i, ni in enumerate(n):
        blk = exp[a_off[i]:a_off[i] + lda[i] * ni]
        assert oracle.lu_inverse(int(ni), blk, int(lda[i]), piv[piv_off[i]:piv_off[i] + ni]) == 0
    batch = mf.LuInverseBatch(n, a_off, piv_off, lda=lda)
    da, dpiv = _dev(fac), _dev(piv)
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    batch.run(da, dpiv, dinfo)
    mf.context().synchronize()
    assert (_host(dinfo) == 0).all()
    got = _host(da)
    assert_bits(got, exp)                      # includes the padding rows, unchanged
    for i, ni in enumerate(n):
        pad = got[a_off[i]:a_off[i] + lda[i] * ni].reshape(ni, lda[i])[:, ni:]
        np.testing.assert_array_equal(pad, fac[a_off[i]:a_off[i] + lda[i] * ni]
                                      .reshape(ni, lda[i])[:, ni:])


def test_lu_inverse_bad_pivots(mf):
    import torch
    rng = np.random.default_rng(23)
    n = np.array([6, 6, 6, 40], np.int32)
    a_off, total, piv_off = _offsets(n)
    a = rng.standard_normal(total) + 0.0
    for i, ni in enumerate(n):                 # well-conditioned factors: diagonal dominant
        a[a_off[i]:a_off[i] + ni * ni:ni + 1] += 10.0
    piv = np.concatenate([np.arange(ni, dtype=np.int32) for ni in n])
    piv[piv_off[1] + 2] = piv[piv_off[1] + 3]  # duplicate
    piv[piv_off[2] + 5] = 6                    # out of range
    batch = mf.LuInverseBatch(n, a_off, piv_off)
    da, dpiv = _dev(a), _dev(piv)
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    batch.run(da, dpiv, dinfo)
    mf.context().synchronize()
    info = _host(dinfo)
    np.testing.assert_array_equal(info, [0, -1, -1, 0])
    got = _host(da)
    for i in (1, 2):
        s = slice(a_off[i], a_off[i] + n[i] * n[i])
        assert_bits(got[s], a[s])
    exp = a.copy()
    einfo = np.zeros(len(n), np.int32)
    oracle.lu_inverse_batched(n[[0]], a_off[[0]], exp, piv_off[[0]], piv, einfo[:1], 1)
    s = slice(a_off[0], a_off[0] + 36)
    assert_bits(got[s], exp[s])


def test_lu_inverse_batch_arguments(mf):
    with pytest.raises(mf.ArgumentException):
        mf.LuInverseBatch(np.array([3, 0], np.int32), np.array([0, 9]), np.array([0, 3]))
    with pytest.raises(mf.ArgumentException):
        mf.LuInverseBatch(np.array([3], np.int32), np.array([0]), np.array([-1]))

"""The allocation-free batched LU + solve (mfg_dgetrf_strided_batched_noalloc).

Callers that cannot allocate device memory (inside someone else's stream capture, fixed-budget
real-time paths, hosts handing the library a fixed arena) use this entry point; its scratch is a
static device array shared by all calls.  It must give exactly what the allocating plan entry
point (mfg_dgetrf_batched) gives, on two calls in a row (the second call runs with the scratch
left over from the first), and refuse sizes beyond its limit before launching anything.

This file is collected last on purpose, so a failure here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _same(got, exp):
    gn, en = np.isnan(got), np.isnan(exp)
    np.testing.assert_array_equal(gn, en)
    np.testing.assert_array_equal(np.where(gn, 0, got).view(np.uint8),
                                  np.where(en, 0, exp).view(np.uint8))


# 48: per-warp vectors in shared memory; 200: in the static array; 256: the largest order
# accepted; 136 with 700 matrices: more matrices than the 608 warps the static array serves, so
# the grid is capped and warps take several matrices each.
@pytest.mark.parametrize("n,count", [(48, 300), (200, 300), (256, 40), (136, 700)])
def test_noalloc_matches_plan_entry_point(mf, n, count):
    import torch
    nrhs = 4
    lda = n + 3
    stride_a = lda * n + 5
    stride_piv = n + 1
    stride_b = n * nrhs + 7
    rng = np.random.default_rng(n)
    a_host = rng.standard_normal(stride_a * count)
    b_host = rng.standard_normal(stride_b * count)
    a_host[stride_a * 3:stride_a * 3 + lda * n] = 0.0      # one singular matrix

    # Existing entry point: a plan over the same layout.
    a_off = np.arange(count, dtype=np.int64) * stride_a
    piv_off = np.arange(count, dtype=np.int64) * stride_piv
    b_off = np.arange(count, dtype=np.int64) * stride_b
    plan = mf.LuBatch(np.full(count, n, np.int32), a_off, piv_off, nrhs=nrhs, b_off=b_off,
                      lda=np.full(count, lda, np.int32))
    ra = torch.from_numpy(a_host.copy()).cuda()
    rb = torch.from_numpy(b_host.copy()).cuda()
    rpiv = torch.zeros(stride_piv * count, dtype=torch.int32, device="cuda")
    rsign = torch.zeros(count, dtype=torch.int32, device="cuda")
    rinfo = torch.zeros(count, dtype=torch.int32, device="cuda")
    plan.run(ra, rpiv, rb, rsign, rinfo)
    mf.context().synchronize()
    ref = [t.cpu().numpy() for t in (ra, rb, rpiv, rsign, rinfo)]
    assert ref[4][3] == 1

    ctx = mf.context()
    lib = mf.library()
    a = torch.empty_like(ra)
    b = torch.empty_like(rb)
    piv = torch.zeros_like(rpiv)
    sign = torch.zeros_like(rsign)
    info = torch.zeros_like(rinfo)
    for call in range(2):
        a.copy_(torch.from_numpy(a_host))
        b.copy_(torch.from_numpy(b_host))
        piv.zero_()
        sign.zero_()
        info.fill_(-7)
        torch.cuda.synchronize()
        rc = lib.mfg_dgetrf_strided_batched_noalloc(
            ctx.h, n, count, _ptr(a), lda, stride_a, _ptr(piv), stride_piv, nrhs, _ptr(b),
            stride_b, _ptr(sign), _ptr(info))
        assert rc == 0, ctx.last_error()
        ctx.synchronize()
        got = [t.cpu().numpy() for t in (a, b, piv, sign, info)]
        for g, r in zip(got[:2], ref[:2]):
            _same(g, r)
        for g, r in zip(got[2:], ref[2:]):
            np.testing.assert_array_equal(g, r, err_msg="call %d" % call)


def test_noalloc_rejects_sizes_beyond_limit(mf):
    import torch
    n = 257
    a = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    piv = torch.full((n,), 5, dtype=torch.int32, device="cuda")
    sign = torch.zeros(1, dtype=torch.int32, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    ctx = mf.context()
    rc = mf.library().mfg_dgetrf_strided_batched_noalloc(
        ctx.h, n, 1, _ptr(a), n, n * n, _ptr(piv), n, 0, None, 0, _ptr(sign), _ptr(info))
    assert rc == -1005
    assert "allocation-free limit" in ctx.last_error()
    ctx.synchronize()
    assert bool((piv == 5).all())

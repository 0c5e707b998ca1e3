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

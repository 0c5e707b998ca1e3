"""The integer-pipe double product (used by every dot product of the factorizations) must equal
the IEEE 754 round-to-nearest-even product bit for bit, on every class of operand.  Both variants
(with and without the integer path for exact zeros) are checked: the self-test kernel turns any
disagreement between them into a NaN."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _operands(rng, n):
    parts = []
    # ordinary values
    parts.append((rng.standard_normal(n), rng.standard_normal(n)))
    # uniformly random bit patterns: every exponent, subnormals, infinities, NaNs
    parts.append((rng.integers(0, 2 ** 64, n, dtype=np.uint64).view(np.float64),
                  rng.integers(0, 2 ** 64, n, dtype=np.uint64).view(np.float64)))
    # short significands: products with <= 54 significant bits hit exact halfway cases
    def short(k):
        bits = rng.integers(0, 2 ** 64, n, dtype=np.uint64)
        bits &= ~np.uint64((1 << (52 - k)) - 1)
        bits = (bits & np.uint64(0x800FFFFFFFFFFFFF)) | np.uint64(0x3FF0000000000000)
        return bits.view(np.float64) * rng.choice([1.0, -1.0, 2.0 ** 40, 2.0 ** -40], n)
    parts.append((short(26), short(27)))
    parts.append((short(20), short(33)))
    # signed zeros against every class of operand (the zero-aware variant's integer path)
    z = rng.choice([0.0, -0.0], n)
    other = rng.integers(0, 2 ** 64, n, dtype=np.uint64).view(np.float64)
    parts.append((z, other))
    parts.append((other, z))
    # exponents at the edges of the normal range (overflow / underflow / subnormal results)
    e1 = rng.integers(-1100, 1100, n).astype(np.float64)
    e2 = -e1 + rng.integers(-60, 60, n)
    with np.errstate(over="ignore"):
        parts.append((np.ldexp(1.0 + rng.random(n), e1.astype(int)),
                      np.ldexp(1.0 + rng.random(n), np.clip(e2, -1100, 1100).astype(int))))
    a = np.concatenate([p[0] for p in parts] + [np.array([0.0, -0.0, np.inf, -np.inf, np.nan,
                                                          5e-324, 1.0, 2.0 ** 1023, 2.0 ** -1022])])
    b = np.concatenate([p[1] for p in parts] + [np.array([3.0, -2.0, 0.0, -1.0, 1.0, 0.5, 5e-324,
                                                          2.0, 0.5])])
    return a, b


def test_integer_product_is_ieee(mf):
    import torch
    rng = np.random.default_rng(99)
    a, b = _operands(rng, 1 << 20)
    da = torch.from_numpy(a).cuda()
    db = torch.from_numpy(b).cuda()
    out = torch.empty_like(da)
    mf.selftest_dmul(da, db, out)
    mf.context().synchronize()
    got = out.cpu().numpy()
    with np.errstate(all="ignore"):
        exp = a * b          # host IEEE multiply, round to nearest even
    gn, en = np.isnan(got), np.isnan(exp)
    np.testing.assert_array_equal(gn, en)
    bad = np.nonzero(got.view(np.uint64)[~gn] != exp.view(np.uint64)[~en])[0]
    assert bad.size == 0, (a[~gn][bad[:5]], b[~gn][bad[:5]], got[~gn][bad[:5]], exp[~en][bad[:5]])


def _div_operands(rng, n):
    parts = []
    # values as the column scalings see them
    parts.append((rng.standard_normal(n), rng.standard_normal(n) * 10))
    # uniformly random bit patterns: every exponent, subnormals, infinities, NaNs
    parts.append((rng.integers(0, 2 ** 64, n, dtype=np.uint64).view(np.float64),
                  rng.integers(0, 2 ** 64, n, dtype=np.uint64).view(np.float64)))
    # dividends one ulp around a rounded product q * b: quotients next to rounding boundaries
    q = 1.0 + rng.random(n)
    b = (1.0 + rng.random(n)) * rng.choice([1.0, -1.0, 2.0 ** 300, 2.0 ** -300], n)
    prod = q * b
    for d in (-1, 0, 1):
        parts.append(((prod.view(np.int64) + d).view(np.float64), b))
    # divisors that are powers of two or have all-ones significands, short significands
    pw = np.ldexp(1.0, rng.integers(-1000, 1000, n))
    ones = np.ldexp(2.0 - 2.0 ** -52, rng.integers(-1000, 1000, n))
    parts.append((rng.standard_normal(n), pw))
    parts.append((rng.standard_normal(n), ones))
    parts.append((ones, rng.standard_normal(n)))
    # exponents at the edges of the normal range (overflow / underflow / subnormal quotients)
    e1 = rng.integers(-1100, 1100, n)
    e2 = np.clip(e1 + rng.integers(-60, 60, n), -1100, 1100)
    with np.errstate(over="ignore"):
        parts.append((np.ldexp(1.0 + rng.random(n), e1), np.ldexp(1.0 + rng.random(n), e2)))
        parts.append((np.ldexp(1.0 + rng.random(n), e1), np.ldexp(1.0 + rng.random(n), -e2)))
    # signed zeros against every class of divisor
    z = rng.choice([0.0, -0.0], n)
    parts.append((z, rng.integers(0, 2 ** 64, n, dtype=np.uint64).view(np.float64)))
    a = np.concatenate([p[0] for p in parts] + [np.array([0.0, -0.0, np.inf, 1.0, np.nan, 1.0,
                                                          5e-324, 2.0 ** 1023, 3.0])])
    b = np.concatenate([p[1] for p in parts] + [np.array([3.0, 0.0, 2.0, np.inf, 1.0, 5e-324,
                                                          1.0, 2.0 ** -2, 2.0 ** 1023])])
    return a, b


def test_integer_quotient_is_ieee(mf):
    """The integer-pipe quotient (LU and Cholesky column scalings) equals IEEE division."""
    import torch
    rng = np.random.default_rng(98)
    a, b = _div_operands(rng, 1 << 20)
    da = torch.from_numpy(a).cuda()
    db = torch.from_numpy(b).cuda()
    out = torch.empty_like(da)
    mf.selftest_ddiv(da, db, out)
    mf.context().synchronize()
    got = out.cpu().numpy()
    with np.errstate(all="ignore"):
        exp = a / b          # host IEEE division, round to nearest even
    gn, en = np.isnan(got), np.isnan(exp)
    np.testing.assert_array_equal(gn, en)
    bad = np.nonzero(got.view(np.uint64)[~gn] != exp.view(np.uint64)[~en])[0]
    assert bad.size == 0, (a[~gn][bad[:5]], b[~gn][bad[:5]], got[~gn][bad[:5]], exp[~en][bad[:5]])

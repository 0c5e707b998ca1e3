"""Float and Complex overloads on the GPU against the oracle, bit for bit, on the golden
vectors (the reference suite's shapes) and on larger seeded cases."""
import numpy as np
import pytest

from oracle import oracle
from tests.conftest import cases

pytestmark = pytest.mark.gpu


def _same(got, exp, msg=""):
    got = np.ascontiguousarray(got)
    exp = np.ascontiguousarray(exp)
    fl = got.view(np.float32 if got.dtype == np.float32 else np.float64)
    fe = exp.view(np.float32 if exp.dtype == np.float32 else np.float64)
    gn, en = np.isnan(fl), np.isnan(fe)
    np.testing.assert_array_equal(gn, en, err_msg=msg)
    np.testing.assert_array_equal(np.where(gn, 0, fl).view(np.uint8),
                                  np.where(en, 0, fe).view(np.uint8), err_msg=msg)


@pytest.mark.parametrize("prec", ["s", "z"])
def test_lu_overloads_golden(mf, golden, prec):
    for key in cases(golden, "lu_%s/" % prec):
        m, n, lda = map(int, key.split("/")[1].split("_"))
        a = golden[key + "/in"].copy()
        piv = np.zeros(m, np.int32)
        sign = mf.Factorization.Lu(m, n, a, lda, piv)
        _same(a, golden[key + "/oracle"], key)
        np.testing.assert_array_equal(piv, golden[key + "/oracle_piv"], err_msg=key)
        assert sign == golden[key + "/oracle_sign"][0], key


@pytest.mark.parametrize("prec", ["s", "z"])
def test_cholesky_overloads_golden(mf, golden, prec):
    for key in cases(golden, "chol_%s/" % prec):
        _, n, lda = key.split("/")[1].split("_")
        n, lda = int(n), int(lda)
        a = golden[key + "/in"].copy()
        if golden[key + "/oracle_info"][0] != 0:
            with pytest.raises(mf.MatrixFactorizationException):
                mf.Factorization.Cholesky(n, a, lda)
        else:
            mf.Factorization.Cholesky(n, a, lda)
            _same(a, golden[key + "/oracle"], key)


def test_qr_complex_golden(mf, golden):
    for key in cases(golden, "qr_z/"):
        m, n, lda, ldq, ldr = map(int, key.split("/")[1].split("_"))
        a = golden[key + "/in"].copy()
        rd = np.zeros(n)
        mf.Factorization.Qr(m, n, a, lda, rd)
        _same(a, golden[key + "/oracle"], key)
        _same(rd, golden[key + "/oracle_rdiag"], key)
        q = golden[key + "/q_in"].copy()
        mf.Factorization.QrOrthogonalFactor(m, n, a, lda, q, ldq)
        _same(q, golden[key + "/oracle_q"], key)
        r = golden[key + "/r_in"].copy()
        mf.Factorization.QrUpperTriangularFactor(m, n, a, lda, r, ldr, rd)
        _same(r, golden[key + "/oracle_r"], key)


@pytest.mark.parametrize("prec", ["s", "z"])
def test_trsv_overloads_golden(mf, golden, prec):
    for key in cases(golden, "trsv_%s/" % prec):
        uplo, trans, n, lda, incx = map(int, key.split("/")[1].split("_"))
        x = golden[key + "/x"].copy()
        mf.Blas.SolveTriangular(uplo, trans, n, golden[key + "/a"], lda, x, incx)
        _same(x, golden[key + "/oracle"], key)


@pytest.mark.parametrize("prec", ["s", "z"])
def test_gemm_overloads_golden(mf, golden, prec):
    for key in cases(golden, "gemm_%s/" % prec):
        ta, tb, m, n, k, lda, ldb, ldc = map(int, key.split("/")[1].split("_"))
        c = golden[key + "/c"].copy()
        mf.Blas.MulMatMat(ta, tb, m, n, k, golden[key + "/a"], lda, golden[key + "/b"], ldb, c, ldc)
        _same(c, golden[key + "/oracle"], key)


@pytest.mark.parametrize("dtype", [np.float32, np.complex128])
@pytest.mark.parametrize("m,n", [(100, 100), (130, 70), (64, 129)])
def test_lu_overloads_large(mf, dtype, m, n):
    rng = np.random.default_rng(m + n)
    a0 = rng.standard_normal(m * n).astype(dtype)
    if dtype == np.complex128:
        a0 = a0 + 1j * rng.standard_normal(m * n)
    a, b = a0.copy(), a0.copy()
    pg, po = np.zeros(m, np.int32), np.zeros(m, np.int32)
    sg = mf.Factorization.Lu(m, n, a, m, pg)
    so = oracle.lu(m, n, b, m, po)
    _same(a, b)
    np.testing.assert_array_equal(pg, po)
    assert sg == so


@pytest.mark.parametrize("dtype", [np.float32, np.complex128])
def test_cholesky_overloads_large(mf, dtype):
    n = 120
    rng = np.random.default_rng(5)
    bm = rng.standard_normal((n, n))
    if dtype == np.complex128:
        bm = bm + 1j * rng.standard_normal((n, n))
    s = (bm @ bm.conj().T + n * np.eye(n)).astype(dtype)
    a0 = s.reshape(-1, order="F").copy()
    a, b = a0.copy(), a0.copy()
    mf.Factorization.Cholesky(n, a, n)
    assert oracle.cholesky(n, b, n) == 0
    _same(a, b)


def test_qr_complex_large(mf):
    m, n = 150, 60
    rng = np.random.default_rng(9)
    a0 = rng.standard_normal(m * n) + 1j * rng.standard_normal(m * n)
    a, b = a0.copy(), a0.copy()
    rg, ro = np.zeros(n), np.zeros(n)
    mf.Factorization.Qr(m, n, a, m, rg)
    oracle.qr(m, n, b, m, ro)
    _same(a, b)
    _same(rg, ro)


@pytest.mark.parametrize("dt", [np.float32, np.complex128])
@pytest.mark.parametrize("n,lda", [(1, 1), (5, 7), (33, 33), (70, 71)])
def test_lu_inverse_overloads(mf, dt, n, lda):
    """Factorization.LuInverse's float and Complex overloads, bit for bit against the oracle,
    including the singular case (no write, MatrixFactorizationException)."""
    rng = np.random.default_rng(700 + n)
    if dt == np.complex128:
        a0 = rng.standard_normal(lda * n) + 1j * rng.standard_normal(lda * n)
    else:
        a0 = rng.standard_normal(lda * n).astype(dt)
    piv = np.zeros(n, np.int32)
    oracle.lu(n, n, a0, lda, piv)
    g, o = a0.copy(), a0.copy()
    mf.Factorization.LuInverse(n, g, lda, piv)
    assert oracle.lu_inverse(n, o, lda, piv) == 0
    _same(g, o, "n=%d" % n)
    s = a0.copy()
    s[(n - 1) * lda + n - 1] = 0
    keep = s.copy()
    with pytest.raises(mf.MatrixFactorizationException):
        mf.Factorization.LuInverse(n, s, lda, piv)
    _same(s, keep)

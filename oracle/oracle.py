"""ctypes front end of the MatFlat CPU oracle — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py may import this module.
Every function takes numpy arrays in MatFlat's layout (column-major storage with a leading
dimension, flattened to 1-D exactly like the C# pointer arguments) and works in place, as the
reference does.  The arithmetic lives in matflat_oracle.cpp, which cites the reference lines.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

UPPER, LOWER = 121, 122
NOTRANS, TRANS, CONJTRANS, CONJNOTRANS = 111, 112, 113, 114

_d = ctypes.POINTER(ctypes.c_double)
_f = ctypes.POINTER(ctypes.c_float)
_i = ctypes.POINTER(ctypes.c_int)
_l = ctypes.POINTER(ctypes.c_int64)
_I = ctypes.c_int
_L = ctypes.c_long


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = ctypes.CDLL(path)
        sigs = {
            "orc_dlu": (_I, [_I, _I, _d, _I, _i]),
            "orc_slu": (_I, [_I, _I, _f, _I, _i]),
            "orc_zlu": (_I, [_I, _I, _d, _I, _i]),
            "orc_dcholesky": (_I, [_I, _d, _I]),
            "orc_scholesky": (_I, [_I, _f, _I]),
            "orc_zcholesky": (_I, [_I, _d, _I]),
            "orc_dqr": (None, [_I, _I, _d, _I, _d]),
            "orc_sqr": (None, [_I, _I, _f, _I, _f]),
            "orc_zqr": (None, [_I, _I, _d, _I, _d]),
            "orc_dqr_q": (None, [_I, _I, _d, _I, _d, _I]),
            "orc_sqr_q": (None, [_I, _I, _f, _I, _f, _I]),
            "orc_zqr_q": (None, [_I, _I, _d, _I, _d, _I]),
            "orc_dqr_r": (None, [_I, _I, _d, _I, _d, _I, _d]),
            "orc_sqr_r": (None, [_I, _I, _f, _I, _f, _I, _f]),
            "orc_zqr_r": (None, [_I, _I, _d, _I, _d, _I, _d]),
            "orc_dtrsv": (_I, [_I, _I, _I, _d, _I, _d, _I]),
            "orc_strsv": (_I, [_I, _I, _I, _f, _I, _f, _I]),
            "orc_ztrsv": (_I, [_I, _I, _I, _d, _I, _d, _I]),
            "orc_dgemm": (_I, [_I, _I, _I, _I, _I, _d, _I, _d, _I, _d, _I]),
            "orc_sgemm": (_I, [_I, _I, _I, _I, _I, _f, _I, _f, _I, _f, _I]),
            "orc_zgemm": (_I, [_I, _I, _I, _I, _I, _d, _I, _d, _I, _d, _I]),
            "orc_dgemv": (_I, [_I, _I, _I, _d, _I, _d, _I, _d, _I]),
            "orc_dlu_inverse": (_I, [_I, _d, _I, _i]),
            "orc_slu_inverse": (_I, [_I, _f, _I, _i]),
            "orc_zlu_inverse": (_I, [_I, _d, _I, _i]),
            "orc_dlu_solve": (None, [_I, _d, _I, _i, _I, _d, _I]),
            "orc_dqr_ls": (None, [_I, _I, _d, _I, _d, _d]),
            "orc_sqr_ls": (None, [_I, _I, _f, _I, _f, _f]),
            "orc_zqr_ls": (None, [_I, _I, _d, _I, _d, _d]),
            "orc_dchol_solve_batched": (None, [_L, _i, _l, _d, _l, _d, _i, _I]),
            "orc_dlu_solve_batched": (None, [_L, _i, _l, _d, _l, _i, _l, _d, _I, _i, _I]),
            "orc_schol_solve_batched": (None, [_L, _i, _l, _f, _l, _f, _I, _i, _I]),
            "orc_zchol_solve_batched": (None, [_L, _i, _l, _d, _l, _d, _I, _i, _I]),
            "orc_slu_solve_batched": (None, [_L, _i, _l, _f, _l, _i, _l, _f, _I, _i, _I]),
            "orc_zlu_solve_batched": (None, [_L, _i, _l, _d, _l, _i, _l, _d, _I, _i, _I]),
            "orc_ddot": (ctypes.c_double, [_I, _d, _I, _d, _I]),
            "orc_dnrm2": (ctypes.c_double, [_I, _d, _I]),
            "orc_dger": (None, [_I, _I, _d, _I, _d, _I, _d, _I]),
            "orc_zgemv": (_I, [_I, _I, _I, _d, _I, _d, _I, _d, _I]),
            "orc_sdot": (ctypes.c_float, [_I, _f, _I, _f, _I]),
            "orc_zdot": (None, [_I, _d, _I, _d, _I, _I, _d]),
            "orc_snrm2": (ctypes.c_float, [_I, _f, _I]),
            "orc_dznrm2": (ctypes.c_double, [_I, _d, _I]),
            "orc_sger": (None, [_I, _I, _f, _I, _f, _I, _f, _I]),
            "orc_zger": (None, [_I, _I, _d, _I, _d, _I, _d, _I, _I]),
            "orc_dgevd_front": (_I, [_I, _d, _I, _d, _I, _d]),
            "orc_dgevd_front_batched": (None, [_L, _i, _l, _d, _l, _d, _d, _i, _I]),
            "orc_sgevd_front": (_I, [_I, _f, _I, _f, _I, _f]),
            "orc_zgevd_front": (_I, [_I, _d, _I, _d, _I, _d]),
            "orc_sgevd_front_batched": (None, [_L, _i, _l, _f, _l, _f, _f, _i, _I]),
            "orc_zgevd_front_batched": (None, [_L, _i, _l, _d, _l, _d, _d, _i, _I]),
            "orc_dlu_inverse_batched": (None, [_L, _i, _l, _d, _l, _i, _i, _I]),
            "orc_slu_inverse_batched": (None, [_L, _i, _l, _f, _l, _i, _i, _I]),
            "orc_zlu_inverse_batched": (None, [_L, _i, _l, _d, _l, _i, _i, _I]),
            "orc_dchol_grad": (_I, [_I, _d, _I, _d, _d, _d]),
            "orc_dchol_grad_batched": (None, [_L, _i, _l, _d, _l, _d, _d, _d, _i, _I]),
            "orc_dqr_ls_batched": (None, [_L, _i, _i, _l, _d, _l, _d, _l, _d, _I]),
            "orc_sqr_ls_batched": (None, [_L, _i, _i, _l, _f, _l, _f, _l, _f, _I]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(_lib, name)
            fn.restype = res
            fn.argtypes = args
    return _lib


def _p(arr, ct):
    assert arr.flags["C_CONTIGUOUS"], "oracle arrays must be contiguous"
    return arr.ctypes.data_as(ctypes.POINTER(ct))


def _fp(a):
    if a.dtype == np.float64:
        return _p(a, ctypes.c_double)
    if a.dtype == np.float32:
        return _p(a, ctypes.c_float)
    if a.dtype == np.complex128:
        return _p(a.view(np.float64), ctypes.c_double)
    raise TypeError(a.dtype)


def _pre(a):
    return {np.float64: "d", np.float32: "s", np.complex128: "z"}[a.dtype.type]


def lu(m, n, a, lda, piv):
    """Factorization.Lu (Factorization.Lu.cs:122-161 / LuCore :240-406); returns the sign."""
    return getattr(lib(), "orc_%slu" % _pre(a))(m, n, _fp(a), lda, _p(piv, ctypes.c_int))


def cholesky(n, a, lda):
    """Factorization.Cholesky (Factorization.Cholesky.cs:33-249); returns 0 or failing column+1."""
    return getattr(lib(), "orc_%scholesky" % _pre(a))(n, _fp(a), lda)


def qr(m, n, a, lda, rdiag):
    """Factorization.Qr (Factorization.Qr.cs:32-255)."""
    getattr(lib(), "orc_%sqr" % _pre(a))(m, n, _fp(a), lda, _fp(rdiag))


def qr_q(m, n, a, lda, q, ldq):
    """Factorization.QrOrthogonalFactor (Factorization.Qr.cs:278-492)."""
    getattr(lib(), "orc_%sqr_q" % _pre(a))(m, n, _fp(a), lda, _fp(q), ldq)


def qr_r(m, n, a, lda, r, ldr, rdiag):
    """Factorization.QrUpperTriangularFactor (Factorization.Qr.cs:518-730)."""
    getattr(lib(), "orc_%sqr_r" % _pre(a))(m, n, _fp(a), lda, _fp(r), ldr, _fp(rdiag))


def trsv(uplo, trans, n, a, lda, x, incx):
    """Blas.SolveTriangular (Blas.SolveTriangular.cs:44-395)."""
    return getattr(lib(), "orc_%strsv" % _pre(a))(uplo, trans, n, _fp(a), lda, _fp(x), incx)


def gemm(transa, transb, m, n, k, a, lda, b, ldb, c, ldc):
    """Blas.MulMatMat (Blas.MulMatMat.cs:45-648)."""
    return getattr(lib(), "orc_%sgemm" % _pre(a))(transa, transb, m, n, k, _fp(a), lda, _fp(b), ldb,
                                                  _fp(c), ldc)


def gemv(trans, m, n, a, lda, x, incx, y, incy):
    """Blas.MulMatVec (Blas.MulMatVec.cs:38-336), the overload a's dtype selects."""
    return getattr(lib(), "orc_%sgemv" % _pre(a))(trans, m, n, _fp(a), lda, _fp(x), incx,
                                                  _fp(y), incy)


def dot(n, x, incx, y, incy, conj=False):
    """Blas.Dot / DotConj (Blas.VectorOperations.cs:110-246), the overload x's dtype selects."""
    if x.dtype == np.complex128:
        out = np.zeros(2)
        lib().orc_zdot(n, _fp(x), incx, _fp(y), incy, 1 if conj else 0, _fp(out))
        return complex(out[0], out[1])
    return getattr(lib(), "orc_%sdot" % _pre(x))(n, _fp(x), incx, _fp(y), incy)


def nrm2(n, x, incx):
    """Blas.L2Norm (Blas.VectorOperations.cs:23-108), the overload x's dtype selects."""
    name = {"d": "orc_dnrm2", "s": "orc_snrm2", "z": "orc_dznrm2"}[_pre(x)]
    return getattr(lib(), name)(n, _fp(x), incx)


def ger(m, n, x, incx, y, incy, a, lda, conj=False):
    """Blas.Outer / OuterConj (Blas.VectorOperations.cs:248-420): a(i,j) = y_j * x_i (conj(y_j)
    * x_i), the overload x's dtype selects."""
    if x.dtype == np.complex128:
        lib().orc_zger(m, n, _fp(x), incx, _fp(y), incy, _fp(a), lda, 1 if conj else 0)
    else:
        getattr(lib(), "orc_%sger" % _pre(x))(m, n, _fp(x), incx, _fp(y), incy, _fp(a), lda)


def lu_inverse(n, a, lda, piv):
    """Factorization.LuInverse (Factorization.LuInverse.cs:27-295), the overload a's dtype
    selects; 0 or 1 (singular)."""
    return getattr(lib(), "orc_%slu_inverse" % _pre(a))(n, _fp(a), lda, _p(piv, ctypes.c_int))


def lu_solve(n, lu_, lda, piv, nrhs, b, ldb):
    """P*b, unit-lower solve (LuInverse idiom), upper solve; b has nrhs columns."""
    lib().orc_dlu_solve(n, _fp(lu_), lda, _p(piv, ctypes.c_int), nrhs, _fp(b), ldb)


def qr_ls(m, n, a, lda, b, x):
    """Least squares through Qr, QrOrthogonalFactor, MulMatVec(Trans) (Complex: MulMatMat
    ConjTrans), QrUpperTriangularFactor and SolveTriangular(Upper, NoTrans)."""
    getattr(lib(), "orc_%sqr_ls" % _pre(a))(m, n, _fp(a), lda, _fp(b), _fp(x))


def chol_solve_batched(n, a_off, a, b_off, b, info, nthreads=1, nrhs=1):
    """Batched Cholesky + solve.  float64: one right-hand side per matrix; float32 and
    complex128 (MatFlat's float and Complex overloads): nrhs columns, ldb = n."""
    if a.dtype != np.float64:
        fn = getattr(lib(), "orc_%schol_solve_batched" % _pre(a))
        fn(len(n), _p(n, ctypes.c_int), _p(a_off, ctypes.c_int64), _fp(a),
           _p(b_off, ctypes.c_int64), _fp(b), nrhs, _p(info, ctypes.c_int), nthreads)
        return
    lib().orc_dchol_solve_batched(len(n), _p(n, ctypes.c_int), _p(a_off, ctypes.c_int64), _fp(a),
                                  _p(b_off, ctypes.c_int64), _fp(b), _p(info, ctypes.c_int), nthreads)


def lu_solve_batched(n, a_off, a, piv_off, piv, b_off, b, nrhs, sign, nthreads=1):
    """Batched LU + solve; a (and b) float64, float32 or complex128 select the overload."""
    fn = getattr(lib(), "orc_%slu_solve_batched" % _pre(a))
    fn(len(n), _p(n, ctypes.c_int), _p(a_off, ctypes.c_int64), _fp(a),
       _p(piv_off, ctypes.c_int64), _p(piv, ctypes.c_int), _p(b_off, ctypes.c_int64), _fp(b), nrhs,
       _p(sign, ctypes.c_int), nthreads)


def lu_inverse_batched(n, a_off, a, piv_off, piv, info, nthreads=1):
    """Factorization.LuInverse per matrix (lda = n); info = j+1 for the first zero U(j,j)."""
    getattr(lib(), "orc_%slu_inverse_batched" % _pre(a))(
                                  len(n), _p(n, ctypes.c_int), _p(a_off, ctypes.c_int64), _fp(a),
                                  _p(piv_off, ctypes.c_int64), _p(piv, ctypes.c_int),
                                  _p(info, ctypes.c_int), nthreads)


def gevd_front(n, a, lda, b, ldb, c):
    """Factorization.GevdCore's front half (Factorization.Gevd.cs:330-365 double, :282-318 float,
    :378-422 Complex): B -> L, C = L^-1 A L^-T (L^-H for Complex; leading dimension n); returns 0
    or Cholesky's k+1.  The overload follows a's dtype."""
    return getattr(lib(), "orc_%sgevd_front" % _pre(a))(n, _fp(a), lda, _fp(b), ldb, _fp(c))


def gevd_front_batched(n, a_off, a, b_off, b, c, info, nthreads=1):
    getattr(lib(), "orc_%sgevd_front_batched" % _pre(a))(
        len(n), _p(n, ctypes.c_int), _p(a_off, ctypes.c_int64), _fp(a),
        _p(b_off, ctypes.c_int64), _fp(b), _fp(c), _p(info, ctypes.c_int), nthreads)


def qr_ls_batched(m, n, a_off, a, b_off, b, x_off, x, nthreads=1):
    fn = lib().orc_dqr_ls_batched if a.dtype == np.float64 else lib().orc_sqr_ls_batched
    fn(len(m), _p(m, ctypes.c_int), _p(n, ctypes.c_int), _p(a_off, ctypes.c_int64), _fp(a),
       _p(b_off, ctypes.c_int64), _fp(b), _p(x_off, ctypes.c_int64), _fp(x), nthreads)


def chol_grad(n, k, lda, y, g):
    """loss = y^T K^-1 y + log det K and grad K^-1 - alpha alpha^T from MatFlat's routines;
    k -> L, y -> alpha, g -> grad.  Returns (info, loss)."""
    loss = ctypes.c_double(0.0)
    info = lib().orc_dchol_grad(n, _fp(k), lda, _fp(y), ctypes.byref(loss), _fp(g))
    return info, loss.value


def chol_grad_batched(n, a_off, a, b_off, y, loss, g, info, nthreads=1):
    lib().orc_dchol_grad_batched(len(n), _p(n, ctypes.c_int), _p(a_off, ctypes.c_int64), _fp(a),
                                 _p(b_off, ctypes.c_int64), _fp(y), _fp(loss), _fp(g),
                                 _p(info, ctypes.c_int), nthreads)

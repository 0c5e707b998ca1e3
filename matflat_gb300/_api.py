"""ctypes binding of libmatflat_gpu.so and the MatFlat-shaped facade above it."""
import ctypes
import enum
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_lib", "libmatflat_gpu.so")

_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_dbl_p = ctypes.POINTER(ctypes.c_double)
_c_i64_p = ctypes.POINTER(ctypes.c_int64)
_vp = ctypes.c_void_p
_I = ctypes.c_int

_SIGS = {
    "mfg_version": (ctypes.c_char_p, []),
    "mfg_create": (_I, [ctypes.POINTER(_vp)]),
    "mfg_destroy": (_I, [_vp]),
    "mfg_set_stream": (_I, [_vp, _vp]),
    "mfg_synchronize": (_I, [_vp]),
    "mfg_last_error": (ctypes.c_char_p, [_vp]),
    "mfg_get_device": (_I, [_vp, _c_int_p]),
    "mfg_dpotrf_backward_batched": (_I, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _I]),
    "mfg_dgetrf": (_I, [_vp, _I, _I, _vp, _I, _vp, _c_int_p]),
    "mfg_dpotrf": (_I, [_vp, _I, _vp, _I, _c_int_p]),
    "mfg_dgeqrf": (_I, [_vp, _I, _I, _vp, _I, _vp]),
    "mfg_dorgqr": (_I, [_vp, _I, _I, _vp, _I, _vp, _I]),
    "mfg_dqr_r": (_I, [_vp, _I, _I, _vp, _I, _vp, _I, _vp]),
    "mfg_sgeqrf": (_I, [_vp, _I, _I, _vp, _I, _vp]),
    "mfg_sorgqr": (_I, [_vp, _I, _I, _vp, _I, _vp, _I]),
    "mfg_sqr_r": (_I, [_vp, _I, _I, _vp, _I, _vp, _I, _vp]),
    "mfg_plan_geqrf_batched": (_I, [_vp, ctypes.POINTER(_vp), _I, _vp, _vp, _vp, _vp, _vp, _I,
                                    _vp]),
    "mfg_dgeqrf_batched": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_sgeqrf_batched": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_zgeqrf_batched": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_zgeqrs_batched": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_dtrsv": (_I, [_vp, _I, _I, _I, _vp, _I, _vp, _I]),
    "mfg_sgetrf": (_I, [_vp, _I, _I, _vp, _I, _vp, _c_int_p]),
    "mfg_zgetrf": (_I, [_vp, _I, _I, _vp, _I, _vp, _c_int_p]),
    "mfg_spotrf": (_I, [_vp, _I, _vp, _I, _c_int_p]),
    "mfg_zpotrf": (_I, [_vp, _I, _vp, _I, _c_int_p]),
    "mfg_zgeqrf": (_I, [_vp, _I, _I, _vp, _I, _vp]),
    "mfg_zorgqr": (_I, [_vp, _I, _I, _vp, _I, _vp, _I]),
    "mfg_zqr_r": (_I, [_vp, _I, _I, _vp, _I, _vp, _I, _vp]),
    "mfg_strsv": (_I, [_vp, _I, _I, _I, _vp, _I, _vp, _I]),
    "mfg_ztrsv": (_I, [_vp, _I, _I, _I, _vp, _I, _vp, _I]),
    "mfg_sgemm": (_I, [_vp, _I, _I, _I, _I, _I, _vp, _I, _vp, _I, _vp, _I]),
    "mfg_zgemm": (_I, [_vp, _I, _I, _I, _I, _I, _vp, _I, _vp, _I, _vp, _I]),
    "mfg_dgemm": (_I, [_vp, _I, _I, _I, _I, _I, _vp, _I, _vp, _I, _vp, _I]),
    "mfg_dgetri": (_I, [_vp, _I, _vp, _I, _vp, _c_int_p]),
    "mfg_sgetri": (_I, [_vp, _I, _vp, _I, _vp, _c_int_p]),
    "mfg_sgetri_batched": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_zgetri_batched": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_zgetri": (_I, [_vp, _I, _vp, _I, _vp, _c_int_p]),
    "mfg_plan_getrf_batched": (_I, [_vp, ctypes.POINTER(_vp), _I, _vp, _vp, _vp, _vp, _I, _vp]),
    "mfg_plan_potrf_batched": (_I, [_vp, ctypes.POINTER(_vp), _I, _vp, _vp, _vp, _I, _vp]),
    "mfg_plan_destroy": (_I, [_vp]),
    "mfg_plan_status": (_I, [_vp]),
    "mfg_dgetrf_batched": (_I, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "mfg_dpotrf_batched": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_plan_autotune": (_I, [_vp, _c_int_p]),
    "mfg_plan_set_form": (_I, [_vp, ctypes.c_int]),
    "mfg_plan_form_fallbacks": (_I, [_vp, _vp]),
    **{"mfg_%sgemv_strided_batched" % _p: (_I, [_vp, _I, _I, _I, _vp, _I, ctypes.c_int64, _vp,
                                                 _I, ctypes.c_int64, _vp, _I, ctypes.c_int64, _I])
       for _p in "sz"},
    **{_f: (_I, [_vp, _I, _vp, _I, ctypes.c_int64, _vp, _I, ctypes.c_int64, _vp, _I])
       for _f in ("mfg_sdot_strided_batched", "mfg_zdot_strided_batched",
                  "mfg_zdotc_strided_batched")},
    **{_f: (_I, [_vp, _I, _vp, _I, ctypes.c_int64, _vp, _I])
       for _f in ("mfg_snrm2_strided_batched", "mfg_dznrm2_strided_batched")},
    **{_f: (_I, [_vp, _I, _I, _vp, _I, ctypes.c_int64, _vp, _I, ctypes.c_int64, _vp, _I,
                 ctypes.c_int64, _I])
       for _f in ("mfg_sger_strided_batched", "mfg_zger_strided_batched",
                  "mfg_zgerc_strided_batched")},
    "mfg_dgemv_strided_batched": (_I, [_vp, _I, _I, _I, _vp, _I, ctypes.c_int64, _vp, _I,
                                       ctypes.c_int64, _vp, _I, ctypes.c_int64, _I]),
    "mfg_ddot_strided_batched": (_I, [_vp, _I, _vp, _I, ctypes.c_int64, _vp, _I, ctypes.c_int64,
                                      _vp, _I]),
    "mfg_dnrm2_strided_batched": (_I, [_vp, _I, _vp, _I, ctypes.c_int64, _vp, _I]),
    "mfg_dger_strided_batched": (_I, [_vp, _I, _I, _vp, _I, ctypes.c_int64, _vp, _I,
                                      ctypes.c_int64, _vp, _I, ctypes.c_int64, _I]),
    "mfg_plan_gevd_front_batched": (_I, [_vp, ctypes.POINTER(_vp), _I, _vp, _vp, _vp, _vp, _vp,
                                         _vp]),
    "mfg_dgevd_front_batched": (_I, [_vp, _vp, _vp, _vp, _vp]),
    "mfg_sgevd_front_batched": (_I, [_vp, _vp, _vp, _vp, _vp]),
    "mfg_zgevd_front_batched": (_I, [_vp, _vp, _vp, _vp, _vp]),
    "mfg_dgetrf_batched_host": (_I, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "mfg_dpotrf_batched_host": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_dgetri_batched_host": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_dgeqrf_batched_host": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_sgeqrf_batched_host": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_zgeqrf_batched_host": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_sgetrf_batched_host": (_I, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "mfg_zgetrf_batched_host": (_I, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "mfg_spotrf_batched_host": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_zpotrf_batched_host": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_dgevd_front_batched_host": (_I, [_vp, _vp, _vp, _vp, _vp]),
    "mfg_sgevd_front_batched_host": (_I, [_vp, _vp, _vp, _vp, _vp]),
    "mfg_zgevd_front_batched_host": (_I, [_vp, _vp, _vp, _vp, _vp]),
    "mfg_dpotrf_logdet_solve_grad_batched_host": (_I, [_vp, _vp, _vp, _vp, _vp, _vp, _I]),
    "mfg_dgetrs_batched": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_sgetrf_batched": (_I, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "mfg_spotrf_batched": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_zpotrf_batched": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_spotrs_batched": (_I, [_vp, _vp, _vp]),
    "mfg_zpotrs_batched": (_I, [_vp, _vp, _vp]),
    "mfg_zgetrf_batched": (_I, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "mfg_sgetrs_batched": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_zgetrs_batched": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_dpotrs_batched": (_I, [_vp, _vp, _vp]),
    "mfg_dgeqrs_batched": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_sgeqrs_batched": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_plan_getri_batched": (_I, [_vp, ctypes.POINTER(_vp), _I, _vp, _vp, _vp, _vp]),
    "mfg_dgetri_batched": (_I, [_vp, _vp, _vp, _vp]),
    "mfg_selftest_dmul": (_I, [_vp, _vp, _vp, _vp, ctypes.c_int64]),
    "mfg_selftest_ddiv": (_I, [_vp, _vp, _vp, _vp, ctypes.c_int64]),
    "mfg_plan_gesv_mixed_batched": (_I, [_vp, ctypes.POINTER(_vp), _I, _I]),
    "mfg_dgesv_mixed_batched": (_I, [_vp, _vp, _vp, _vp, _I, _I, ctypes.c_double, _vp, _vp,
                                     _vp]),
    "mfg_dpotrf_logdet_solve_grad_batched": (_I, [_vp, _vp, _vp, _vp, _vp, _vp, _I]),
    "mfg_dgetrf_strided_batched_noalloc": (_I, [_vp, _I, _I, _vp, _I, ctypes.c_int64, _vp,
                                                ctypes.c_int64, _I, _vp, ctypes.c_int64, _vp,
                                                _vp]),
}

_lib = None
_lib_lock = threading.Lock()


def library_path():
    return _LIB_PATH


def library():
    """Loads libmatflat_gpu.so (raises if it has not been built)."""
    global _lib
    with _lib_lock:
        if _lib is None:
            if not os.path.exists(_LIB_PATH):
                raise RuntimeError(
                    "libmatflat_gpu.so is not built (run `python -c \"import __graft_entry__ as g; "
                    "g.build()\"` or `python matflat_gb300/build.py`)")
            lib = ctypes.CDLL(_LIB_PATH)
            for name, (res, args) in _SIGS.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


# ---------------------------------------------------------------------------------------------
# MatFlat's exception hierarchy (MatFlat/MatFlatException.cs, MatrixFactorizationException.cs)
# and the .NET argument exceptions it throws.

class MatFlatException(Exception):
    """MatFlat.MatFlatException."""


class MatrixFactorizationException(MatFlatException):
    """MatFlat.MatrixFactorizationException: thrown when a factorization fails."""


class ArgumentException(ValueError):
    """System.ArgumentException."""

    def __init__(self, message, param=None):
        super().__init__(message if param is None else "%s (Parameter '%s')" % (message, param))
        self.param = param


class ArgumentNullException(ArgumentException):
    """System.ArgumentNullException."""

    def __init__(self, param):
        super().__init__("Value cannot be null.", param)


class Uplo(enum.IntEnum):
    """MatFlat.Uplo (MatFlat/Uplo.cs:13,18)."""
    Upper = 121
    Lower = 122


class Transpose(enum.IntEnum):
    """MatFlat.Transpose (MatFlat/Transpose.cs:13-28)."""
    NoTrans = 111
    Trans = 112
    ConjTrans = 113
    ConjNoTrans = 114


class _Context:
    def __init__(self):
        lib = library()
        h = _vp()
        rc = lib.mfg_create(ctypes.byref(h))
        if rc != 0:
            raise RuntimeError("mfg_create failed (%d): no usable CUDA device" % rc)
        self.h = h
        self.lib = lib

    def set_stream(self, stream_handle):
        self.lib.mfg_set_stream(self.h, _vp(stream_handle or 0))

    def synchronize(self):
        self.check(self.lib.mfg_synchronize(self.h))

    def device(self):
        """The CUDA device the context runs on (current at its creation)."""
        d = ctypes.c_int(-1)
        self.check(self.lib.mfg_get_device(self.h, ctypes.byref(d)), "mfg_get_device")
        return d.value

    def last_error(self):
        msg = self.lib.mfg_last_error(self.h)
        return msg.decode() if msg else ""

    def check(self, rc, what="call"):
        if rc != 0:
            raise RuntimeError("%s failed with status %d: %s" % (what, rc, self.last_error()))


_ctx = None
_ctx_lock = threading.Lock()


def context():
    """The process-wide default context (created on first use).

    Batched calls on device buffers are asynchronous on the context's own stream, which does not
    wait for other streams: finish (or synchronize) the work that fills their inputs on torch's
    stream before the call, keep every tensor passed to them alive (and do not let another
    stream reuse its memory) until context().synchronize(), or point the context at torch's
    stream with set_stream."""
    global _ctx
    with _ctx_lock:
        if _ctx is None:
            _ctx = _Context()
    return _ctx


def _need(arr, count, name, dtype=np.float64):
    if arr is None:
        raise ArgumentNullException(name)
    if not isinstance(arr, np.ndarray) or arr.dtype != dtype or arr.ndim != 1 or not \
            arr.flags["C_CONTIGUOUS"]:
        raise TypeError("%s must be a contiguous 1-D numpy array of %s" % (name, np.dtype(dtype)))
    if arr.size < count:
        raise ArgumentException("The array is too small (%d < %d elements)." % (arr.size, count),
                                name)


def _dt(a):
    if isinstance(a, np.ndarray) and a.dtype in (np.float32, np.complex128):
        return a.dtype.type
    return np.float64


def _pfx(dt):
    return {np.float64: "d", np.float32: "s", np.complex128: "z"}[dt]


_RDIAG_DT = {np.float64: np.float64, np.float32: np.float32, np.complex128: np.float64}


def _span(rows, cols, ld):
    return 0 if rows <= 0 or cols <= 0 else ld * (cols - 1) + rows


def _ptr(arr):
    return _vp(arr.ctypes.data)


def _raise_status(rc, names, ctx):
    """Maps a negative argument status to the .NET exception MatFlat throws."""
    msg = ctx.last_error()
    if rc == -1003:
        raise ArgumentException("In-place operation is not supported.")
    if rc < 0 and -rc - 2 < len(names):
        name = names[-rc - 2]
        if msg.endswith("is null"):
            raise ArgumentNullException(name)
        raise ArgumentException(msg, name)
    raise RuntimeError("status %d: %s" % (rc, msg))


class Factorization:
    """Mirror of MatFlat.Factorization: float32, float64 and complex128 arrays select MatFlat's
    float, double and Complex overloads."""

    @staticmethod
    def Lu(m, n, a, lda, piv):
        """Factorization.Lu (MatFlat/Factorization.Lu.cs:122-161); returns the pivot sign."""
        ctx = context()
        dt = _dt(a)
        if m > 0 and n > 0 and lda >= m:
            _need(a, _span(m, n, lda), "a", dt)
            _need(piv, m, "piv", np.int32)
        sign = ctypes.c_int(0)
        rc = getattr(ctx.lib, "mfg_%sgetrf" % _pfx(dt))(ctx.h, m, n, None if a is None else _ptr(a), lda,
                                None if piv is None else _ptr(piv), ctypes.byref(sign))
        if rc != 0:
            _raise_status(rc, ["m", "n", "a", "lda", "piv"], ctx)
        return sign.value

    @staticmethod
    def Cholesky(n, a, lda):
        """Factorization.Cholesky (MatFlat/Factorization.Cholesky.cs:114-168)."""
        ctx = context()
        dt = _dt(a)
        if n > 0 and lda >= n:
            _need(a, _span(n, n, lda), "a", dt)
        info = ctypes.c_int(0)
        rc = getattr(ctx.lib, "mfg_%spotrf" % _pfx(dt))(ctx.h, n, None if a is None else _ptr(a), lda, ctypes.byref(info))
        if rc != 0:
            _raise_status(rc, ["n", "a", "lda"], ctx)
        if info.value != 0:
            raise MatrixFactorizationException(
                "Cholesky decomposition failed. The matrix must be positive definite.")

    @staticmethod
    def Qr(m, n, a, lda, rdiag):
        """Factorization.Qr (MatFlat/Factorization.Qr.cs:115-172 double, :32-89 float)."""
        ctx = context()
        dt = _dt(a)
        if m > 0 and n > 0 and lda >= m and n <= m:
            _need(a, _span(m, n, lda), "a", dt)
            _need(rdiag, n, "rdiag", _RDIAG_DT[dt])
        fn = getattr(ctx.lib, "mfg_%sgeqrf" % _pfx(dt))
        rc = fn(ctx.h, m, n, None if a is None else _ptr(a), lda,
                                None if rdiag is None else _ptr(rdiag))
        if rc != 0:
            _raise_status(rc, ["m", "n", "a", "lda", "rdiag"], ctx)

    @staticmethod
    def QrOrthogonalFactor(m, n, a, lda, q, ldq):
        """Factorization.QrOrthogonalFactor (MatFlat/Factorization.Qr.cs:357-413, :278-334)."""
        ctx = context()
        dt = _dt(a)
        if m > 0 and n > 0 and lda >= m and ldq >= m and n <= m:
            _need(a, _span(m, n, lda), "a", dt)
            _need(q, _span(m, n, ldq), "q", dt)
        fn = getattr(ctx.lib, "mfg_%sorgqr" % _pfx(dt))
        rc = fn(ctx.h, m, n, None if a is None else _ptr(a), lda,
                                None if q is None else _ptr(q), ldq)
        if rc != 0:
            _raise_status(rc, ["m", "n", "a", "lda", "q", "ldq"], ctx)

    @staticmethod
    def QrUpperTriangularFactor(m, n, a, lda, r, ldr, rdiag):
        """Factorization.QrUpperTriangularFactor (MatFlat/Factorization.Qr.cs:597-650, :518-571)."""
        ctx = context()
        dt = _dt(a)
        if m > 0 and n > 0 and lda >= m and ldr >= n and n <= m:
            _need(a, _span(m, n, lda), "a", dt)
            _need(r, _span(n, n, ldr), "r", dt)
            _need(rdiag, n, "rdiag", _RDIAG_DT[dt])
        fn = getattr(ctx.lib, "mfg_%sqr_r" % _pfx(dt))
        rc = fn(ctx.h, m, n, None if a is None else _ptr(a), lda,
                               None if r is None else _ptr(r), ldr,
                               None if rdiag is None else _ptr(rdiag))
        if rc != 0:
            _raise_status(rc, ["m", "n", "a", "lda", "r", "ldr", "rdiag"], ctx)

    @staticmethod
    def LuInverse(n, a, lda, piv):
        """Factorization.LuInverse (MatFlat/Factorization.LuInverse.cs:27-295): float32,
        float64 and complex128 overloads."""
        ctx = context()
        dt = _dt(a)
        if n > 0 and lda >= n:
            _need(a, _span(n, n, lda), "a", dt)
            _need(piv, n, "piv", np.int32)
        info = ctypes.c_int(0)
        fn = getattr(ctx.lib, "mfg_%sgetri" % _pfx(dt))
        rc = fn(ctx.h, n, None if a is None else _ptr(a), lda,
                None if piv is None else _ptr(piv), ctypes.byref(info))
        if rc != 0:
            _raise_status(rc, ["n", "a", "lda", "piv"], ctx)
        if info.value != 0:
            raise MatrixFactorizationException("The matrix is not invertible.")


class Blas:
    """Mirror of MatFlat.Blas: float32, float64 and complex128 overloads."""

    @staticmethod
    def SolveTriangular(uplo, transa, n, a, lda, x, incx):
        """Blas.SolveTriangular (MatFlat/Blas.SolveTriangular.cs:162-242)."""
        ctx = context()
        dt = _dt(a)
        if n > 0 and lda >= n and incx > 0:
            _need(a, _span(n, n, lda), "a", dt)
            _need(x, (n - 1) * incx + 1, "x", dt)
        rc = getattr(ctx.lib, "mfg_%strsv" % _pfx(dt))(ctx.h, int(uplo), int(transa), n, None if a is None else _ptr(a),
                               lda, None if x is None else _ptr(x), incx)
        if rc != 0:
            _raise_status(rc, ["uplo", "transa", "n", "a", "lda", "x", "incx"], ctx)

    @staticmethod
    def MulMatMat(transa, transb, m, n, k, a, lda, b, ldb, c, ldc):
        """Blas.MulMatMat (MatFlat/Blas.MulMatMat.cs:226-368)."""
        ctx = context()
        dt = _dt(a)
        ok = m > 0 and n > 0 and k > 0 and ldc >= m
        ta, tb = int(transa), int(transb)
        modes = (111, 112, 113, 114) if dt == np.complex128 else (111, 112)
        if ok and ta in modes and tb in modes:
            ar, ac = (m, k) if ta in (111, 114) else (k, m)
            br, bc = (k, n) if tb in (111, 114) else (n, k)
            if lda >= ar and ldb >= br:
                _need(a, _span(ar, ac, lda), "a", dt)
                _need(b, _span(br, bc, ldb), "b", dt)
                _need(c, _span(m, n, ldc), "c", dt)
                if a is not None and c is not None and (np.shares_memory(a, c) or
                                                        np.shares_memory(b, c)):
                    raise ArgumentException("In-place operation is not supported.")
        rc = getattr(ctx.lib, "mfg_%sgemm" % _pfx(dt))(ctx.h, ta, tb, m, n, k, None if a is None else _ptr(a), lda,
                               None if b is None else _ptr(b), ldb,
                               None if c is None else _ptr(c), ldc)
        if rc != 0:
            _raise_status(rc, ["transa", "transb", "m", "n", "k", "a", "lda", "b", "ldb", "c",
                               "ldc"], ctx)


# ---------------------------------------------------------------------------------------------
# Batched overloads.  Arrays are device memory: pass torch CUDA tensors or raw device pointers.

def _hptr(x):
    """Pointer of a host array: numpy array or CPU tensor."""
    if x is None:
        return None
    if isinstance(x, np.ndarray):
        return _ptr(x)
    return _vp(x.data_ptr())


def _dptr(x):
    if x is None:
        return None
    if isinstance(x, int):
        return _vp(x)
    return _vp(x.data_ptr())


def _elem(a, dtype=None):
    """BLAS prefix of a batched call: "d", "s" or "z" from `dtype` or from a's element type."""
    if dtype is not None:
        if dtype not in ("d", "s", "z"):
            raise ValueError("dtype must be 'd', 's' or 'z'")
        return dtype
    name = str(getattr(a, "dtype", "float64")).replace("torch.", "")
    if name == "float32":
        return "s"
    if name == "complex128":
        return "z"
    if name == "float64":
        return "d"
    raise TypeError("unsupported element type %s (float64, float32 or complex128)" % name)


class _Batch:
    def __init__(self, ctx, handle):
        self.ctx = ctx
        self.h = handle

    def close(self):
        if self.h is not None and self.h.value:
            self.ctx.lib.mfg_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def status(self):
        self.ctx.check(self.ctx.lib.mfg_plan_status(self.h), "mfg_plan_status")

    def autotune(self):
        """Times candidate launch shapes on a synthetic batch with this plan's size mix and keeps
        the fastest (getrf, potrf and geqrf plans); returns (warps per CTA, warps per SM, lanes
        per matrix (getrf: the lanes table of its size buckets), multiply mode, dot pairs per
        block)."""
        cfg = (ctypes.c_int * 5)()
        rc = self.ctx.lib.mfg_plan_autotune(self.h, cfg)
        self.ctx.check(rc, "mfg_plan_autotune")
        return tuple(cfg)


def _i32(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.int32))


def _i64(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.int64))


class LuBatch(_Batch):
    """Batched Factorization.Lu (+ solve of nrhs right-hand sides) over matrices of uneven n.

    n, a_off, piv_off, b_off are host arrays describing the layout (element offsets into the
    device buffers passed to `run`); lda defaults to n.
    """

    def __init__(self, n, a_off, piv_off, nrhs=0, b_off=None, lda=None, ctx=None):
        ctx = ctx or context()
        self._n = _i32(n)
        self._lda = None if lda is None else _i32(lda)
        self._a_off = _i64(a_off)
        self._piv_off = _i64(piv_off)
        self._b_off = None if b_off is None else _i64(b_off)
        h = _vp()
        rc = ctx.lib.mfg_plan_getrf_batched(
            ctx.h, ctypes.byref(h), len(self._n), _ptr(self._n),
            None if self._lda is None else _ptr(self._lda), _ptr(self._a_off),
            _ptr(self._piv_off), nrhs, None if self._b_off is None else _ptr(self._b_off))
        ctx.check(rc, "mfg_plan_getrf_batched")
        super().__init__(ctx, h)
        self.count = len(self._n)
        self.nrhs = nrhs

    def set_form(self, form):
        """Arithmetic form of the double factorization: "exact" (MatFlat's bits, the default) or
        "fma" (fused multiply-adds with MatFlat's pivots kept by a screen and an exact redo of
        the matrices it rejects; backward-stable factors, not MatFlat's bits)."""
        code = FORMS[form]
        self.ctx.check(self.ctx.lib.mfg_plan_set_form(self.h, code), "mfg_plan_set_form")

    def form_fallbacks(self):
        """Matrices of the last execution that the FMA form redid in MatFlat's arithmetic."""
        v = ctypes.c_longlong(0)
        self.ctx.check(self.ctx.lib.mfg_plan_form_fallbacks(self.h, ctypes.byref(v)),
                       "mfg_plan_form_fallbacks")
        return v.value

    def run(self, a, piv, b, sign, info, dtype=None):
        """Factor (+ solve) device buffers.  The element type follows a's dtype (float64,
        float32 or complex128 tensors: MatFlat's double, float and Complex overloads); pass
        dtype="z" for Complex data held as interleaved float64."""
        name = "mfg_%sgetrf_batched" % _elem(a, dtype)
        rc = getattr(self.ctx.lib, name)(self.h, _dptr(a), _dptr(piv), _dptr(b), _dptr(sign),
                                         _dptr(info))
        self.ctx.check(rc, name)

    def run_host(self, a, piv, b, sign, info, dtype=None):
        """Factor + solve on host buffers (numpy arrays or CPU tensors, page-locked for full
        speed); copies and compute are pipelined over chunks of the batch.  Synchronous.
        Element type as in `run`."""
        name = "mfg_%sgetrf_batched_host" % _elem(a, dtype)
        rc = getattr(self.ctx.lib, name)(self.h, _hptr(a), _hptr(piv), _hptr(b), _hptr(sign),
                                         _hptr(info))
        self.ctx.check(rc, name)

    def solve(self, a, piv, b, dtype=None):
        """Solves with factors and pivots already in a and piv (the plan's nrhs columns of b);
        element type as in `run`."""
        name = "mfg_%sgetrs_batched" % _elem(a, dtype)
        rc = getattr(self.ctx.lib, name)(self.h, _dptr(a), _dptr(piv), _dptr(b))
        self.ctx.check(rc, name)


class StridedBlas:
    """Strided batches of Blas.MulMatVec / Dot / DotConj / L2Norm / Outer / OuterConj on device
    buffers (torch CUDA tensors or device pointers); item b of each operand starts at base +
    b * stride (elements).  The overload follows the operand's dtype (float64, float32,
    complex128), or `dtype` ("d", "s", "z") for raw pointers or interleaved float64."""

    @staticmethod
    def MulMatVec(trans, m, n, a, lda, stride_a, x, incx, stride_x, y, incy, stride_y, count,
                  ctx=None, dtype=None):
        ctx = ctx or context()
        name = "mfg_%sgemv_strided_batched" % _elem(a, dtype)
        rc = getattr(ctx.lib, name)(ctx.h, trans, m, n, _dptr(a), lda, stride_a, _dptr(x), incx,
                                    stride_x, _dptr(y), incy, stride_y, count)
        if rc != 0:
            _raise_status(rc, ["trans", "m", "n", "a", "lda", "stride_a", "x", "incx",
                               "stride_x", "y", "incy", "stride_y", "count"], ctx)

    @staticmethod
    def _dot(name, n, x, incx, stride_x, y, incy, stride_y, result, count, ctx):
        ctx = ctx or context()
        rc = getattr(ctx.lib, name)(ctx.h, n, _dptr(x), incx, stride_x, _dptr(y), incy, stride_y,
                                    _dptr(result), count)
        if rc != 0:
            _raise_status(rc, ["n", "x", "incx", "stride_x", "y", "incy", "stride_y", "result",
                               "count"], ctx)

    @staticmethod
    def Dot(n, x, incx, stride_x, y, incy, stride_y, result, count, ctx=None, dtype=None):
        StridedBlas._dot("mfg_%sdot_strided_batched" % _elem(x, dtype), n, x, incx, stride_x, y,
                         incy, stride_y, result, count, ctx)

    @staticmethod
    def DotConj(n, x, incx, stride_x, y, incy, stride_y, result, count, ctx=None):
        """Complex only: sum of conj(x_i) * y_i (Blas.DotConj)."""
        StridedBlas._dot("mfg_zdotc_strided_batched", n, x, incx, stride_x, y, incy, stride_y,
                         result, count, ctx)

    @staticmethod
    def L2Norm(n, x, incx, stride_x, result, count, ctx=None, dtype=None):
        """Result dtype: float32 for float32 input, float64 otherwise (Complex norms are real)."""
        ctx = ctx or context()
        name = {"d": "mfg_dnrm2_strided_batched", "s": "mfg_snrm2_strided_batched",
                "z": "mfg_dznrm2_strided_batched"}[_elem(x, dtype)]
        rc = getattr(ctx.lib, name)(ctx.h, n, _dptr(x), incx, stride_x, _dptr(result), count)
        if rc != 0:
            _raise_status(rc, ["n", "x", "incx", "stride_x", "result", "count"], ctx)

    @staticmethod
    def _outer(name, m, n, x, incx, stride_x, y, incy, stride_y, a, lda, stride_a, count, ctx):
        ctx = ctx or context()
        rc = getattr(ctx.lib, name)(ctx.h, m, n, _dptr(x), incx, stride_x, _dptr(y), incy,
                                    stride_y, _dptr(a), lda, stride_a, count)
        if rc != 0:
            _raise_status(rc, ["m", "n", "x", "incx", "stride_x", "y", "incy", "stride_y", "a",
                               "lda", "stride_a", "count"], ctx)

    @staticmethod
    def Outer(m, n, x, incx, stride_x, y, incy, stride_y, a, lda, stride_a, count, ctx=None,
              dtype=None):
        StridedBlas._outer("mfg_%sger_strided_batched" % _elem(x, dtype), m, n, x, incx,
                           stride_x, y, incy, stride_y, a, lda, stride_a, count, ctx)

    @staticmethod
    def OuterConj(m, n, x, incx, stride_x, y, incy, stride_y, a, lda, stride_a, count,
                  ctx=None):
        """Complex only: a(i,j) = conj(y_j) * x_i (Blas.OuterConj)."""
        StridedBlas._outer("mfg_zgerc_strided_batched", m, n, x, incx, stride_x, y, incy,
                           stride_y, a, lda, stride_a, count, ctx)


class LuInverseBatch(_Batch):
    """Batched Factorization.LuInverse: every matrix's LU factors (from LuBatch) become A^-1.

    info per matrix: 0, j+1 when U(j,j) == 0 (MatFlat's "The matrix is not invertible."), or -1
    when its pivot vector is not a permutation; such matrices are left unchanged.
    """

    def __init__(self, n, a_off, piv_off, lda=None, ctx=None):
        ctx = ctx or context()
        self._n = _i32(n)
        self._lda = None if lda is None else _i32(lda)
        self._a_off = _i64(a_off)
        self._piv_off = _i64(piv_off)
        h = _vp()
        rc = ctx.lib.mfg_plan_getri_batched(
            ctx.h, ctypes.byref(h), len(self._n), _ptr(self._n),
            None if self._lda is None else _ptr(self._lda), _ptr(self._a_off),
            _ptr(self._piv_off))
        if rc != 0:
            _raise_status(rc, ["plan", "count", "n", "lda", "a_off", "piv_off"], ctx)
        super().__init__(ctx, h)
        self.count = len(self._n)

    def run(self, a, piv, info, dtype=None):
        """Element type as in LuBatch.run (float64, float32 or complex128)."""
        name = "mfg_%sgetri_batched" % _elem(a, dtype)
        rc = getattr(self.ctx.lib, name)(self.h, _dptr(a), _dptr(piv), _dptr(info))
        self.ctx.check(rc, name)

    def run_host(self, a, piv, info):
        """The inverse on host arrays, copies pipelined with compute.  Synchronous."""
        rc = self.ctx.lib.mfg_dgetri_batched_host(self.h, _hptr(a), _hptr(piv), _hptr(info))
        self.ctx.check(rc, "mfg_dgetri_batched_host")


class GevdFrontBatch(_Batch):
    """Front half of Factorization.Gevd over a batch of pairs (A, B): B becomes its Cholesky factor
    L and C = L^-1 A L^-T (L^-1 A L^-H for Complex; leading dimension n) is written at c_off.  info
    per pair: 0, or k+1 when B is not positive definite ("The right-hand side matrix is not
    positive definite.").  The double, float and Complex overloads share the plan; the overload
    follows the arrays' element type, or `dtype` ("d", "s", "z") for Complex held as doubles."""

    def __init__(self, n, a_off, b_off, c_off, lda=None, ldb=None, ctx=None):
        ctx = ctx or context()
        self._n = _i32(n)
        self._lda = None if lda is None else _i32(lda)
        self._ldb = None if ldb is None else _i32(ldb)
        self._a_off, self._b_off, self._c_off = _i64(a_off), _i64(b_off), _i64(c_off)
        h = _vp()
        rc = ctx.lib.mfg_plan_gevd_front_batched(
            ctx.h, ctypes.byref(h), len(self._n), _ptr(self._n),
            None if self._lda is None else _ptr(self._lda), _ptr(self._a_off),
            None if self._ldb is None else _ptr(self._ldb), _ptr(self._b_off), _ptr(self._c_off))
        if rc != 0:
            _raise_status(rc, ["plan", "count", "n", "lda", "a_off", "ldb", "b_off", "c_off"], ctx)
        super().__init__(ctx, h)
        self.count = len(self._n)

    def run(self, a, b, c, info, dtype=None):
        name = "mfg_%sgevd_front_batched" % _elem(a, dtype)
        rc = getattr(self.ctx.lib, name)(self.h, _dptr(a), _dptr(b), _dptr(c), _dptr(info))
        self.ctx.check(rc, name)

    def run_host(self, a, b, c, info, dtype=None):
        """The front half on host arrays, copies pipelined with compute.  Synchronous."""
        name = "mfg_%sgevd_front_batched_host" % _elem(a, dtype)
        rc = getattr(self.ctx.lib, name)(self.h, _hptr(a), _hptr(b), _hptr(c), _hptr(info))
        self.ctx.check(rc, name)


class CholeskyBatch(_Batch):
    """Batched Factorization.Cholesky (+ L y = b, L^T x = y) over matrices of uneven n."""

    def __init__(self, n, a_off, nrhs=0, b_off=None, lda=None, ctx=None):
        ctx = ctx or context()
        self._n = _i32(n)
        self._lda = None if lda is None else _i32(lda)
        self._a_off = _i64(a_off)
        self._b_off = None if b_off is None else _i64(b_off)
        h = _vp()
        rc = ctx.lib.mfg_plan_potrf_batched(
            ctx.h, ctypes.byref(h), len(self._n), _ptr(self._n),
            None if self._lda is None else _ptr(self._lda), _ptr(self._a_off), nrhs,
            None if self._b_off is None else _ptr(self._b_off))
        ctx.check(rc, "mfg_plan_potrf_batched")
        super().__init__(ctx, h)
        self.count = len(self._n)
        self.nrhs = nrhs

    def set_form(self, form):
        """Arithmetic form of the double factorization: "exact" (MatFlat's bits, the default) or
        "fma" (fused multiply-adds in any order: backward-stable factors, not MatFlat's bits)."""
        code = FORMS[form]
        self.ctx.check(self.ctx.lib.mfg_plan_set_form(self.h, code), "mfg_plan_set_form")

    def run(self, a, b, info, dtype=None):
        """Factor (+ solve) device buffers; the element type follows a's dtype (float64,
        float32, complex128; dtype="z" for Complex held as interleaved float64).  Complex
        solves L y = b, then L^H x = y."""
        name = "mfg_%spotrf_batched" % _elem(a, dtype)
        rc = getattr(self.ctx.lib, name)(self.h, _dptr(a), _dptr(b), _dptr(info))
        self.ctx.check(rc, name)

    def run_host(self, a, b, info, dtype=None):
        """Factor + solve on host arrays, copies pipelined with compute.  Synchronous.  Element
        type as in `run`."""
        name = "mfg_%spotrf_batched_host" % _elem(a, dtype)
        rc = getattr(self.ctx.lib, name)(self.h, _hptr(a), _hptr(b), _hptr(info))
        self.ctx.check(rc, name)

    def backward(self, a, abar, info, lbar=None, logdet_bar=None, x=None, xbar=None, bbar=None,
                 recompute=True):
        """Vector-Jacobian product of (L = Cholesky(A), log det A, x = A^-1 b): writes the
        symmetric gradient to abar (and A^-1 xbar to bbar).  recompute=True: a holds A and is
        overwritten with L; False: a holds L already.  Device buffers; asynchronous."""
        rc = self.ctx.lib.mfg_dpotrf_backward_batched(
            self.h, _dptr(a), _dptr(lbar), _dptr(logdet_bar), _dptr(x), _dptr(xbar),
            _dptr(abar), _dptr(bbar), _dptr(info), 1 if recompute else 0)
        self.ctx.check(rc, "mfg_dpotrf_backward_batched")

    def loss_and_grad_host(self, k, y, loss, grad, info, keep_factor=True):
        """loss_and_grad on host arrays, copies pipelined with compute.  Synchronous."""
        rc = self.ctx.lib.mfg_dpotrf_logdet_solve_grad_batched_host(
            self.h, _hptr(k), _hptr(y), _hptr(loss), _hptr(grad), _hptr(info),
            1 if keep_factor else 0)
        self.ctx.check(rc, "mfg_dpotrf_logdet_solve_grad_batched_host")

    def solve(self, a, b, dtype=None):
        """Solves with Cholesky factors already in a (the plan's nrhs columns of b); element
        type as in `run`."""
        name = "mfg_%spotrs_batched" % _elem(a, dtype)
        rc = getattr(self.ctx.lib, name)(self.h, _dptr(a), _dptr(b))
        self.ctx.check(rc, name)

    def loss_and_grad(self, k, y, loss, grad, info, keep_factor=True):
        """loss = y^T K^-1 y + log det K and grad = K^-1 - alpha alpha^T per matrix; y becomes
        alpha = K^-1 y; with keep_factor, k becomes the Cholesky factor L."""
        rc = self.ctx.lib.mfg_dpotrf_logdet_solve_grad_batched(
            self.h, _dptr(k), _dptr(y), _dptr(loss), _dptr(grad), _dptr(info),
            1 if keep_factor else 0)
        self.ctx.check(rc, "mfg_dpotrf_logdet_solve_grad_batched")


class QrBatch(_Batch):
    """Batched Factorization.Qr of tall matrices (+ least squares of nrhs right-hand sides).

    m, n, a_off, rdiag_off, b_off are host arrays; lda defaults to m; b has nrhs columns of m
    entries per matrix.  `run` takes float64 or float32 device buffers (MatFlat's two overloads).
    """

    def __init__(self, m, n, a_off, rdiag_off, nrhs=0, b_off=None, lda=None, ctx=None):
        ctx = ctx or context()
        self._m = _i32(m)
        self._n = _i32(n)
        self._lda = None if lda is None else _i32(lda)
        self._a_off = _i64(a_off)
        self._rdiag_off = _i64(rdiag_off)
        self._b_off = None if b_off is None else _i64(b_off)
        h = _vp()
        rc = ctx.lib.mfg_plan_geqrf_batched(
            ctx.h, ctypes.byref(h), len(self._m), _ptr(self._m), _ptr(self._n),
            None if self._lda is None else _ptr(self._lda), _ptr(self._a_off),
            _ptr(self._rdiag_off), nrhs, None if self._b_off is None else _ptr(self._b_off))
        ctx.check(rc, "mfg_plan_geqrf_batched")
        super().__init__(ctx, h)
        self.count = len(self._m)
        self.nrhs = nrhs

    def set_form(self, form):
        """Arithmetic form of the double factorization: "exact" (MatFlat's bits, the default) or
        "fma" (fused multiply-adds, backward-stable factors, not MatFlat's bits)."""
        code = FORMS[form]
        self.ctx.check(self.ctx.lib.mfg_plan_set_form(self.h, code), "mfg_plan_set_form")

    def run(self, a, rdiag, b=None, single=False, dtype=None):
        """QR (+ least squares) of device buffers: float64 (default), float32 (single=True or a
        float32 tensor) or Complex (a complex128 tensor, or dtype="z" for interleaved float64;
        rdiag is then float64)."""
        name = "mfg_%sgeqrf_batched" % ("s" if single else _elem(a, dtype))
        rc = getattr(self.ctx.lib, name)(self.h, _dptr(a), _dptr(rdiag), _dptr(b))
        self.ctx.check(rc, name)

    def run_host(self, a, rdiag, b=None, single=False, dtype=None):
        """QR (+ least squares) on host arrays, copies pipelined with compute.  Synchronous.
        Element type as in `run`."""
        name = "mfg_%sgeqrf_batched_host" % ("s" if single else _elem(a, dtype))
        rc = getattr(self.ctx.lib, name)(self.h, _hptr(a), _hptr(rdiag), _hptr(b))
        self.ctx.check(rc, name)

    def solve(self, a, rdiag, b, single=False, dtype=None):
        """Least squares with the factorization already in a and rdiag (nrhs columns of b);
        element type as in `run`."""
        name = "mfg_%sgeqrs_batched" % ("s" if single else _elem(a, dtype))
        rc = getattr(self.ctx.lib, name)(self.h, _dptr(a), _dptr(rdiag), _dptr(b))
        self.ctx.check(rc, name)


def selftest_dmul(a, b, out):
    """out = a * b through the integer-pipe product (device tensors of float64)."""
    ctx = context()
    ctx.check(ctx.lib.mfg_selftest_dmul(ctx.h, _dptr(a), _dptr(b), _dptr(out), a.numel()),
              "mfg_selftest_dmul")


def selftest_ddiv(a, b, out):
    """out = a / b through the integer-pipe quotient (device tensors of float64)."""
    ctx = context()
    ctx.check(ctx.lib.mfg_selftest_ddiv(ctx.h, _dptr(a), _dptr(b), _dptr(out), a.numel()),
              "mfg_selftest_ddiv")


LOWP = {"fp32": 0, "tf32": 1, "bf16": 2, "tf32x3": 3}
FORMS = {"exact": 0, "fma": 1}


class MixedSolveBatch(_Batch):
    """Mixed-precision LU solve with FP64 iterative refinement for `count` systems of order n
    (device buffers: a count*n*n, b and x count*n, berr/iters/info count)."""

    def __init__(self, count, n, ctx=None):
        ctx = ctx or context()
        h = _vp()
        ctx.check(ctx.lib.mfg_plan_gesv_mixed_batched(ctx.h, ctypes.byref(h), count, n),
                  "mfg_plan_gesv_mixed_batched")
        super().__init__(ctx, h)
        self.count = count
        self.n = n

    def run(self, a, b, x, berr, iters, info, lowp="tf32", max_iter=10, tol=1e-12, sync=True):
        """Solves on the context's stream.  With sync (the default) the call waits for the
        results and raises if a bounded device-side wait of the tensor-core update gave up
        (mfg_plan_status); with sync=False it returns at once and status() checks later."""
        rc = self.ctx.lib.mfg_dgesv_mixed_batched(self.h, _dptr(a), _dptr(b), _dptr(x),
                                                  LOWP[lowp], max_iter, tol, _dptr(berr),
                                                  _dptr(iters), _dptr(info))
        self.ctx.check(rc, "mfg_dgesv_mixed_batched")
        if sync:
            self.status()

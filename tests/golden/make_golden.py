"""Generates tests/golden/matflat_cases.npz — golden vectors for the oracle pin and GPU parity.

For every shape the reference test suite uses (MatFlatTest/*.cs, cited per family below) this
script draws a seeded input the way the reference's helpers do (Matrix.RandomDouble /
Vector.RandomDouble fill every slot, padding included, with values in [-1, 1):
MatFlatTest/Matrix.cs:16-21, MatFlatTest/Vector.cs:16-21; the reference uses .NET's
System.Random, which cannot run here, so a numpy PCG64 stream with the same seeds stands in),
and stores:
  * `<case>/in...`     the inputs,
  * `<case>/lapack...` what the reference suite's own oracle (OpenBLAS LAPACK/BLAS, here through
                       scipy, which bundles OpenBLAS) returns for them,
  * `<case>/oracle...` what the CPU restatement of MatFlat (oracle/) returns.
The tests check oracle == oracle fixture bit for bit, oracle ~ LAPACK at the reference's
tolerances, and GPU == oracle fixture bit for bit.  The literal fixtures of the reference
(LuTests.cs:146-192, QrTests.cs:133, :314-386) are included verbatim as inputs.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np
import scipy.linalg.blas as sblas
import scipy.linalg.lapack as slapack

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "matflat_cases.npz")

# MatFlatTest/LuTests.cs:103-122 (m, n, lda)
LU_SHAPES = [(1, 1, 1), (1, 1, 3), (2, 2, 2), (2, 2, 3), (3, 3, 3), (3, 3, 5), (3, 1, 3),
             (3, 1, 5), (1, 3, 1), (1, 3, 3), (3, 4, 3), (3, 4, 5), (4, 3, 4), (4, 3, 5),
             (11, 23, 11), (11, 23, 17), (16, 8, 16), (16, 8, 32), (23, 11, 23), (23, 11, 31)]
# MatFlatTest/CholeskyTests.cs:95-106 and :127-138 (n, lda)
CHOL_SHAPES = [(1, 1), (1, 3), (2, 2), (2, 3), (3, 3), (3, 5), (11, 11), (11, 17), (16, 16),
               (16, 32), (23, 23), (23, 31)]
# MatFlatTest/QrTests.cs:200-213 (m, n, lda, ldq, ldr)
QR_SHAPES = [(1, 1, 1, 1, 1), (1, 1, 3, 2, 4), (2, 2, 2, 2, 2), (2, 2, 3, 4, 5), (3, 3, 3, 3, 3),
             (3, 3, 5, 4, 6), (3, 1, 3, 3, 1), (3, 1, 5, 4, 6), (4, 3, 4, 4, 3), (4, 3, 5, 7, 6),
             (16, 8, 16, 16, 8), (16, 8, 32, 24, 20), (23, 11, 23, 23, 11), (23, 11, 31, 29, 37)]
# MatFlatTest/BlasTests.SolveTriangularDouble.cs:10-19 (n, lda, incx), four uplo/trans modes
TRSV_SHAPES = [(1, 1, 1), (1, 2, 3), (2, 2, 1), (2, 3, 4), (3, 3, 1), (3, 5, 2), (5, 5, 1),
               (5, 7, 3), (10, 10, 1), (10, 17, 5)]
# MatFlatTest/BlasTests.MulMatMatDouble.cs:9-20, :54-62, :96-104, :138-146 (m, n, k, lda, ldb, ldc)
GEMM_SHAPES = {
    "NN": [(1, 1, 1, 1, 1, 1), (1, 1, 1, 2, 3, 4), (2, 2, 2, 2, 2, 2), (2, 2, 2, 3, 4, 5),
           (3, 3, 3, 3, 3, 3), (3, 3, 3, 4, 5, 6), (2, 3, 4, 2, 4, 2), (2, 3, 4, 3, 5, 3),
           (1, 5, 2, 1, 2, 1), (1, 5, 2, 3, 4, 3), (5, 3, 2, 5, 2, 5), (5, 3, 2, 7, 4, 7)],
    "TN": [(1, 1, 1, 1, 1, 1), (2, 2, 2, 2, 2, 2), (3, 3, 3, 3, 3, 3), (2, 3, 4, 4, 4, 2),
           (2, 3, 4, 5, 6, 3), (5, 4, 3, 3, 3, 5), (5, 4, 3, 4, 5, 6), (3, 7, 5, 5, 5, 3),
           (3, 7, 5, 8, 9, 7)],
    "NT": [(1, 1, 1, 1, 1, 1), (2, 2, 2, 2, 2, 2), (3, 3, 3, 3, 3, 3), (2, 3, 4, 2, 3, 2),
           (2, 3, 4, 5, 6, 3), (5, 4, 3, 5, 4, 5), (5, 4, 3, 6, 6, 7), (3, 7, 5, 3, 7, 3),
           (3, 7, 5, 5, 9, 6)],
    "TT": [(1, 1, 1, 1, 1, 1), (2, 2, 2, 2, 2, 2), (3, 3, 3, 3, 3, 3), (2, 3, 4, 4, 3, 2),
           (2, 3, 4, 5, 5, 5), (5, 4, 3, 3, 4, 5), (5, 4, 3, 7, 5, 6), (3, 7, 5, 5, 7, 3),
           (3, 7, 5, 6, 8, 4)],
}
# MatFlatTest/LuInverseTests.cs:75-84 (n, lda)
LUINV_SHAPES = [(1, 1), (1, 3), (2, 2), (2, 3), (3, 3), (3, 5), (5, 5), (5, 8), (10, 10), (10, 17)]
# MatFlatTest/GevdTests.cs:12-21, :96-105, :180-189 (n, lda, ldb)
GEVD_SHAPES = [(1, 1, 1), (1, 3, 2), (2, 2, 2), (2, 4, 3), (3, 3, 3), (3, 4, 5), (5, 5, 5),
               (5, 7, 8), (10, 10, 10), (10, 17, 11)]

U, L = 121, 122
NT, T = 111, 112


def random_double(seed, count):
    """[-1, 1) fill of every slot, as Matrix.RandomDouble does."""
    return 2.0 * np.random.default_rng(seed).random(count) - 1.0


def random_single(seed, count):
    return (2.0 * np.random.default_rng(seed).random(count, dtype=np.float32) - 1.0).astype(
        np.float32)


def random_complex(seed, count):
    """Matrix.RandomComplex (MatFlatTest/Matrix.cs:23-28): re and im in [-1, 1) from one stream."""
    v = 2.0 * np.random.default_rng(seed).random(2 * count) - 1.0
    return v[0::2] + 1j * v[1::2]


def fmat(flat, m, n, ld):
    """m-by-n Fortran view (copy) of a column-major flat array with leading dimension ld."""
    return np.array(flat[:ld * n].reshape(n, ld).T[:m, :], order="F")


def put(flat, mat, ld):
    m, n = mat.shape
    out = flat.copy()
    for j in range(n):
        out[j * ld:j * ld + m] = mat[:, j]
    return out


def main():
    g = {}

    # ---- LU (double and single) --------------------------------------------------------
    for (m, n, lda) in LU_SHAPES:
        for prec in ("d", "s"):
            a = (random_double if prec == "d" else random_single)(42, n * lda)
            key = "lu_%s/%d_%d_%d" % (prec, m, n, lda)
            g[key + "/in"] = a
            lu_ = a.copy()
            piv = np.zeros(m, np.int32)
            sign = oracle.lu(m, n, lu_, lda, piv)
            g[key + "/oracle"] = lu_
            g[key + "/oracle_piv"] = piv
            g[key + "/oracle_sign"] = np.array([sign], np.int32)
            f = slapack.dgetrf if prec == "d" else slapack.sgetrf
            lu_l, ipiv, info = f(fmat(a, m, n, lda))
            g[key + "/lapack"] = put(a, lu_l, lda)
    for name, a in (("zero", np.zeros(9)), ("singular", np.arange(1, 10, dtype=np.float64))):
        key = "lu_d/lit_" + name
        g[key + "/in"] = a
        lu_ = a.copy()
        piv = np.zeros(3, np.int32)
        sign = oracle.lu(3, 3, lu_, 3, piv)
        g[key + "/oracle"] = lu_
        g[key + "/oracle_piv"] = piv
        g[key + "/oracle_sign"] = np.array([sign], np.int32)
        lu_l, ipiv, info = slapack.dgetrf(fmat(a, 3, 3, 3))
        g[key + "/lapack"] = put(a, lu_l, 3)

    # ---- Cholesky ------------------------------------------------------------------------
    for (n, lda) in CHOL_SHAPES:
        for kind in ("general", "maybe"):
            a = random_double(42, n * lda)
            if kind == "general":
                # CholeskyTests.cs:302-339: A*A^T in the upper triangle, NaN below.
                am = fmat(a, n, n, lda)
                s = am @ am.T
                for j in range(n):
                    for i in range(n):
                        a[j * lda + i] = s[i, j] if j >= i else np.nan
            else:
                # CholeskyTests.cs:400-416: raw random upper triangle, NaN below.
                for j in range(n):
                    for i in range(j + 1, n):
                        a[j * lda + i] = np.nan
            key = "chol_d/%s_%d_%d" % (kind, n, lda)
            g[key + "/in"] = a
            c = a.copy()
            info = oracle.cholesky(n, c, lda)
            g[key + "/oracle"] = c
            g[key + "/oracle_info"] = np.array([info], np.int32)
            up = np.triu(np.nan_to_num(fmat(a, n, n, lda)))
            r, linfo = slapack.dpotrf(up, lower=0)
            g[key + "/lapack_info"] = np.array([linfo], np.int32)
            exp = a.copy()
            lmat = np.tril(r.T)
            g[key + "/lapack"] = put(exp, lmat, lda)

    # ---- QR (double and single) ----------------------------------------------------------
    for (m, n, lda, ldq, ldr) in QR_SHAPES:
        for prec in ("d", "s"):
            rnd = random_double if prec == "d" else random_single
            a = rnd(42, n * lda)
            key = "qr_%s/%d_%d_%d_%d_%d" % (prec, m, n, lda, ldq, ldr)
            g[key + "/in"] = a
            g[key + "/q_in"] = rnd(57, n * ldq)
            g[key + "/r_in"] = rnd(58, n * ldr)
            qa = a.copy()
            rd = np.zeros(n, a.dtype)
            oracle.qr(m, n, qa, lda, rd)
            q = g[key + "/q_in"].copy()
            oracle.qr_q(m, n, qa, lda, q, ldq)
            r = g[key + "/r_in"].copy()
            oracle.qr_r(m, n, qa, lda, r, ldr, rd)
            g[key + "/oracle"] = qa
            g[key + "/oracle_rdiag"] = rd
            g[key + "/oracle_q"] = q
            g[key + "/oracle_r"] = r
    a = np.array([1, 2, 3, 2, 4, 6, 0, 0, 0], np.float64)  # QrTests.cs:133 (singular)
    key = "qr_d/lit_singular"
    g[key + "/in"] = a
    qa = a.copy()
    rd = np.zeros(3)
    oracle.qr(3, 3, qa, 3, rd)
    q = np.zeros(9)
    oracle.qr_q(3, 3, qa, 3, q, 3)
    r = np.zeros(9)
    oracle.qr_r(3, 3, qa, 3, r, 3, rd)
    g[key + "/oracle"], g[key + "/oracle_rdiag"], g[key + "/oracle_q"], g[key + "/oracle_r"] = \
        qa, rd, q, r

    # ---- Triangular solve ------------------------------------------------------------------
    for (n, lda, incx) in TRSV_SHAPES:
        for uplo, trans in ((U, NT), (L, NT), (U, T), (L, T)):
            a = random_double(42, n * lda)
            for j in range(n):
                for i in range(n):
                    if (uplo == U and i > j) or (uplo == L and i < j):
                        a[j * lda + i] = 0.0
            x = random_double(57, (n - 1) * incx + 1)
            key = "trsv_d/%d_%d_%d_%d_%d" % (uplo, trans, n, lda, incx)
            g[key + "/a"] = a
            g[key + "/x"] = x
            xo = x.copy()
            oracle.trsv(uplo, trans, n, a, lda, xo, incx)
            g[key + "/oracle"] = xo
            xe = x.copy()
            res = sblas.dtrsv(fmat(a, n, n, lda), x[::incx][:n].copy(), trans=int(trans == T),
                              lower=int(uplo == L), diag=0)
            xe[::incx][:n] = res
            g[key + "/lapack"] = xe

    # ---- MulMatMat -------------------------------------------------------------------------
    for mode, shapes in GEMM_SHAPES.items():
        ta = NT if mode[0] == "N" else T
        tb = NT if mode[1] == "N" else T
        for (m, n, k, lda, ldb, ldc) in shapes:
            ar, ac = (m, k) if ta == NT else (k, m)
            br, bc = (k, n) if tb == NT else (n, k)
            a = random_double(42, ac * lda)
            b = random_double(57, bc * ldb)
            c = random_double(0, n * ldc)
            key = "gemm_d/%s_%d_%d_%d_%d_%d_%d" % (mode, m, n, k, lda, ldb, ldc)
            g[key + "/a"], g[key + "/b"], g[key + "/c"] = a, b, c
            co = c.copy()
            oracle.gemm(ta, tb, m, n, k, a, lda, b, ldb, co, ldc)
            g[key + "/oracle"] = co
            am = fmat(a, ar, ac, lda)
            bm = fmat(b, br, bc, ldb)
            am = am if ta == NT else am.T
            bm = bm if tb == NT else bm.T
            g[key + "/lapack"] = put(c, am @ bm, ldc)

    # ---- LuInverse -------------------------------------------------------------------------
    for (n, lda) in LUINV_SHAPES:
        a = random_double(42, n * lda)
        key = "luinv_d/%d_%d" % (n, lda)
        g[key + "/in"] = a
        lu_ = a.copy()
        piv = np.zeros(n, np.int32)
        oracle.lu(n, n, lu_, lda, piv)
        g[key + "/lu"] = lu_
        g[key + "/piv"] = piv
        inv = lu_.copy()
        rc = oracle.lu_inverse(n, inv, lda, piv)
        assert rc == 0
        g[key + "/oracle"] = inv

    # ---- Complex LU (LuTests.cs:194-286; LAPACK pivots by |re| + |im| too) -----------------
    for (m, n, lda) in LU_SHAPES:
        a = random_complex(42, n * lda)
        key = "lu_z/%d_%d_%d" % (m, n, lda)
        g[key + "/in"] = a
        lu_ = a.copy()
        piv = np.zeros(m, np.int32)
        sign = oracle.lu(m, n, lu_, lda, piv)
        g[key + "/oracle"] = lu_
        g[key + "/oracle_piv"] = piv
        g[key + "/oracle_sign"] = np.array([sign], np.int32)
        lu_l, ipiv, info = slapack.zgetrf(fmat(a, m, n, lda))
        g[key + "/lapack"] = put(a, lu_l, lda)

    # ---- float and Complex Cholesky (CholeskyTests.cs:12-92, :178-260) ----------------------
    for (n, lda) in CHOL_SHAPES:
        for prec in ("s", "z"):
            for kind in ("general", "maybe"):
                if prec == "s":
                    a = random_single(42, n * lda)
                else:
                    a = random_complex(42, n * lda)
                if kind == "general":
                    am = fmat(a, n, n, lda)
                    sm = am @ am.conj().T
                    for j in range(n):
                        for i in range(n):
                            a[j * lda + i] = sm[i, j] if j >= i else np.nan
                else:
                    for j in range(n):
                        for i in range(j + 1, n):
                            a[j * lda + i] = np.nan
                key = "chol_%s/%s_%d_%d" % (prec, kind, n, lda)
                g[key + "/in"] = a
                c = a.copy()
                g[key + "/oracle_info"] = np.array([oracle.cholesky(n, c, lda)], np.int32)
                g[key + "/oracle"] = c
                up = np.triu(np.nan_to_num(fmat(a, n, n, lda)))
                f = slapack.spotrf if prec == "s" else slapack.zpotrf
                r, linfo = f(up, lower=0)
                g[key + "/lapack_info"] = np.array([linfo], np.int32)
                g[key + "/lapack"] = put(a.copy(), np.tril(r.conj().T), lda)

    # ---- Complex QR ------------------------------------------------------------------------
    for (m, n, lda, ldq, ldr) in QR_SHAPES:
        a = random_complex(42, n * lda)
        key = "qr_z/%d_%d_%d_%d_%d" % (m, n, lda, ldq, ldr)
        g[key + "/in"] = a
        g[key + "/q_in"] = random_complex(57, n * ldq)
        g[key + "/r_in"] = random_complex(58, n * ldr)
        qa = a.copy()
        rd = np.zeros(n)
        oracle.qr(m, n, qa, lda, rd)
        q = g[key + "/q_in"].copy()
        oracle.qr_q(m, n, qa, lda, q, ldq)
        r = g[key + "/r_in"].copy()
        oracle.qr_r(m, n, qa, lda, r, ldr, rd)
        g[key + "/oracle"], g[key + "/oracle_rdiag"] = qa, rd
        g[key + "/oracle_q"], g[key + "/oracle_r"] = q, r

    # ---- float and Complex triangular solves (SolveTriangularSingle/Complex.cs) --------------
    CT, CN = 113, 114
    for (n, lda, incx) in TRSV_SHAPES:
        for prec, modes in (("s", (NT, T)), ("z", (NT, T, CT, CN))):
            for uplo in (U, L):
                for trans in modes:
                    if prec == "s":
                        a = random_single(42, n * lda)
                        x = random_single(57, (n - 1) * incx + 1)
                    else:
                        a = random_complex(42, n * lda)
                        x = random_complex(57, (n - 1) * incx + 1)
                    for j in range(n):
                        for i in range(n):
                            if (uplo == U and i > j) or (uplo == L and i < j):
                                a[j * lda + i] = 0.0
                    key = "trsv_%s/%d_%d_%d_%d_%d" % (prec, uplo, trans, n, lda, incx)
                    g[key + "/a"], g[key + "/x"] = a, x
                    xo = x.copy()
                    oracle.trsv(uplo, trans, n, a, lda, xo, incx)
                    g[key + "/oracle"] = xo
                    am = fmat(a, n, n, lda).astype(np.complex128 if prec == "z" else np.float64)
                    op = {NT: am, T: am.T, CT: am.conj().T, CN: am.conj()}[trans]
                    xe = x.astype(np.complex128 if prec == "z" else np.float64)
                    sol = np.linalg.solve(op, xe[::incx][:n])
                    xe[::incx][:n] = sol
                    g[key + "/lapack"] = xe

    # ---- float and Complex MulMatMat (MulMatMatSingle/Complex.cs, four conj conditions) ------
    for mode, shapes in GEMM_SHAPES.items():
        for prec in ("s", "z"):
            conds = [(False, False)] if prec == "s" else [(False, False), (True, False),
                                                         (False, True), (True, True)]
            for (ca, cb) in conds:
                ta = (CN if ca else NT) if mode[0] == "N" else (CT if ca else T)
                tb = (CN if cb else NT) if mode[1] == "N" else (CT if cb else T)
                for (m, n, k, lda, ldb, ldc) in shapes:
                    ar, ac = (m, k) if mode[0] == "N" else (k, m)
                    br, bc = (k, n) if mode[1] == "N" else (n, k)
                    rnd = random_single if prec == "s" else random_complex
                    a, b, c = rnd(42, ac * lda), rnd(57, bc * ldb), rnd(0, n * ldc)
                    key = "gemm_%s/%d_%d_%d_%d_%d_%d_%d_%d" % (prec, ta, tb, m, n, k, lda, ldb, ldc)
                    g[key + "/a"], g[key + "/b"], g[key + "/c"] = a, b, c
                    co = c.copy()
                    oracle.gemm(ta, tb, m, n, k, a, lda, b, ldb, co, ldc)
                    g[key + "/oracle"] = co
                    am = fmat(a, ar, ac, lda).astype(np.complex128 if prec == "z" else np.float64)
                    bm = fmat(b, br, bc, ldb).astype(np.complex128 if prec == "z" else np.float64)
                    am = am if mode[0] == "N" else am.T
                    bm = bm if mode[1] == "N" else bm.T
                    am = am.conj() if ca else am
                    bm = bm.conj() if cb else bm
                    g[key + "/lapack"] = put(c.astype(am.dtype), am @ bm, ldc)

    # ---- float and Complex LuInverse (LuInverseTests.cs:12-72, :138-204) ---------------------
    for (n, lda) in LUINV_SHAPES:
        for prec, rnd in (("s", random_single), ("z", random_complex)):
            a = rnd(42, n * lda)
            key = "luinv_%s/%d_%d" % (prec, n, lda)
            g[key + "/in"] = a
            lu_ = a.copy()
            piv = np.zeros(n, np.int32)
            oracle.lu(n, n, lu_, lda, piv)
            g[key + "/lu"] = lu_
            g[key + "/piv"] = piv
            inv = lu_.copy()
            assert oracle.lu_inverse(n, inv, lda, piv) == 0
            g[key + "/oracle"] = inv
            wide = np.complex128 if prec == "z" else np.float64
            g[key + "/lapack"] = put(a.astype(wide), np.linalg.inv(fmat(a, n, n, lda).astype(wide)),
                                     lda)

    # ---- GEVD front half (GevdTests.cs:12-94 float, :96-178 double, :180-262 Complex) --------
    # A and B as the reference's GetDecomposable* helpers build them (X X^T, or X X^H, from a
    # random X, written over X's leading n-by-n block; :271-364), then the strict lower parts set
    # to NaN (NanLowerPart, :366-406), as the reference passes them to Factorization.Gevd.  The
    # LAPACK side: potrf of B and C = L^-1 A L^-T (L^-H) from numpy's LAPACK solves.
    for (n, lda, ldb) in GEVD_SHAPES:
        for prec, rnd in (("d", random_double), ("s", random_single), ("z", random_complex)):
            def decomposable(seed, ld):
                x = rnd(seed, n * ld)
                xm = fmat(x, n, n, ld).astype(np.complex128 if prec == "z" else np.float64)
                sym = xm @ xm.conj().T
                return put(x, sym.astype(x.dtype), ld)
            a, b = decomposable(42, lda), decomposable(57, ldb)
            full_a, full_b = a.copy(), b.copy()
            for j in range(n):
                a[j * lda + j + 1:j * lda + n] = np.nan
                b[j * ldb + j + 1:j * ldb + n] = np.nan
            key = "gevd_%s/%d_%d_%d" % (prec, n, lda, ldb)
            g[key + "/a"], g[key + "/b"] = a, b
            ob, oc = b.copy(), np.zeros(n * n, a.dtype)
            assert oracle.gevd_front(n, a, lda, ob, ldb, oc) == 0
            g[key + "/oracle_b"], g[key + "/oracle_c"] = ob, oc
            wide = np.complex128 if prec == "z" else np.float64
            Am = fmat(full_a, n, n, lda).astype(wide)
            Bm = fmat(full_b, n, n, ldb).astype(wide)
            Lm = np.linalg.cholesky(Bm)
            Cm = np.linalg.solve(Lm, np.linalg.solve(Lm, Am).conj().T).conj().T
            g[key + "/lapack_l"] = put(full_b.astype(wide), Lm, ldb)
            g[key + "/lapack_c"] = Cm.flatten(order="F")

    np.savez_compressed(OUT, **g)
    print("wrote %s (%d arrays, %.1f KB)" % (OUT, len(g), os.path.getsize(OUT) / 1024))


if __name__ == "__main__":
    main()

"""Pins the CPU oracle (test infrastructure) before anything is compared against it.

1. Regression: the oracle rebuilt on this machine reproduces the committed golden outputs bit
   for bit (so the x86 container and the Arm GPU host agree, -ffp-contract=off honoured).
2. Agreement with the reference test suite's own oracle — OpenBLAS LAPACK/BLAS — at the
   reference's tolerances, on the reference's shapes (MatFlatTest/*.cs) and literal fixtures.
"""
import numpy as np
import pytest

from oracle import oracle
from tests.conftest import cases

U, L, NT, T = 121, 122, 111, 112


def _lu_case(golden, key, prec):
    _, dims = key.split("/")
    if dims.startswith("lit_"):
        m = n = lda = 3
    else:
        m, n, lda = map(int, dims.split("_"))
    return m, n, lda


@pytest.mark.parametrize("prec", ["d", "s"])
def test_lu_oracle_pin(golden, prec):
    keys = cases(golden, "lu_%s/" % prec)
    assert keys
    tol = 1e-12 if prec == "d" else 1e-5   # LuTests.cs:143 (double), :52 (single)
    for key in keys:
        m, n, lda = _lu_case(golden, key, prec)
        a = golden[key + "/in"].copy()
        piv = np.zeros(m, np.int32)
        sign = oracle.lu(m, n, a, lda, piv)
        np.testing.assert_array_equal(a.view(np.uint8), golden[key + "/oracle"].view(np.uint8),
                                      err_msg=key)
        np.testing.assert_array_equal(piv, golden[key + "/oracle_piv"], err_msg=key)
        assert sign == golden[key + "/oracle_sign"][0]
        exp = golden[key + "/lapack"]
        assert np.max(np.abs(a - exp)) <= tol, key
        # piv is a permutation vector and sign its parity.
        assert sorted(piv.tolist()) == list(range(m))
        perm_sign = np.linalg.det(np.eye(m)[piv]) if m <= 32 else sign
        assert round(perm_sign) == sign


def test_lu_literal_fixtures(golden):
    # LuTests.cs:146-168: the all-zero 3x3 stays zero; :170-192 the singular 1..9 matrix.
    a = np.zeros(9)
    piv = np.zeros(3, np.int32)
    assert oracle.lu(3, 3, a, 3, piv) == 1
    assert np.all(a == 0) and list(piv) == [0, 1, 2]
    key = "lu_d/lit_singular"
    a = golden[key + "/in"].copy()
    oracle.lu(3, 3, a, 3, piv)
    assert np.max(np.abs(a - golden[key + "/lapack"])) <= 1e-12


def test_cholesky_oracle_pin(golden):
    keys = cases(golden, "chol_d/")
    assert keys
    for key in keys:
        kind, n, lda = key.split("/")[1].split("_")
        n, lda = int(n), int(lda)
        a = golden[key + "/in"].copy()
        info = oracle.cholesky(n, a, lda)
        assert info == golden[key + "/oracle_info"][0]
        lapack_ok = golden[key + "/lapack_info"][0] == 0
        # CholeskyTests.cs:139-176: MatFlat fails exactly when LAPACK reports info != 0.
        assert (info == 0) == lapack_ok, key
        if info == 0:
            np.testing.assert_array_equal(a.view(np.uint8),
                                          golden[key + "/oracle"].view(np.uint8), err_msg=key)
            exp = golden[key + "/lapack"]
            for j in range(n):
                col = slice(j * lda, j * lda + n)
                assert np.max(np.abs(a[col] - exp[col])) <= 1e-12, key   # CholeskyTests.cs:124
                # padding rows (lower part NaN by construction) untouched
                np.testing.assert_array_equal(a[j * lda + n:(j + 1) * lda],
                                              golden[key + "/in"][j * lda + n:(j + 1) * lda])
    assert any(golden[k + "/oracle_info"][0] != 0 for k in keys), "no failing case exercised"


@pytest.mark.parametrize("prec", ["d", "s"])
def test_qr_oracle_pin(golden, prec):
    keys = [k for k in cases(golden, "qr_%s/" % prec) if "lit_" not in k]
    assert keys
    tol = 1e-12 if prec == "d" else 1e-4   # QrTests.cs:262-277 (double), :74-89 (single)
    for key in keys:
        m, n, lda, ldq, ldr = map(int, key.split("/")[1].split("_"))
        a = golden[key + "/in"].copy()
        rd = np.zeros(n, a.dtype)
        oracle.qr(m, n, a, lda, rd)
        q = golden[key + "/q_in"].copy()
        oracle.qr_q(m, n, a, lda, q, ldq)
        r = golden[key + "/r_in"].copy()
        oracle.qr_r(m, n, a, lda, r, ldr, rd)
        for got, name in ((a, "oracle"), (rd, "oracle_rdiag"), (q, "oracle_q"), (r, "oracle_r")):
            np.testing.assert_array_equal(got.view(np.uint8),
                                          golden[key + "/" + name].view(np.uint8), err_msg=key)
        a0 = golden[key + "/in"]
        A = np.array(a0[:n * lda].reshape(n, lda).T[:m], dtype=np.float64)
        Q = np.array(q[:n * ldq].reshape(n, ldq).T[:m], dtype=np.float64)
        R = np.array(r[:n * ldr].reshape(n, ldr).T[:n], dtype=np.float64)
        assert np.max(np.abs(Q @ R - A)) <= tol, key
        assert np.max(np.abs(Q.T @ Q - np.eye(n))) <= tol, key
        # Padding rows of a, q, r are bit-unchanged (QrTests.cs:284-310).
        for arr, ld, rows, src in ((a, lda, m, a0), (q, ldq, m, golden[key + "/q_in"]),
                                   (r, ldr, n, golden[key + "/r_in"])):
            for j in range(n):
                np.testing.assert_array_equal(arr[j * ld + rows:(j + 1) * ld],
                                              src[j * ld + rows:(j + 1) * ld])


def test_qr_singular_literal(golden):
    # QrTests.cs:314-386: the singular {1,2,3,2,4,6,0,0,0} still gives Q R = A, Q^T Q = I.
    key = "qr_d/lit_singular"
    A = golden[key + "/in"].reshape(3, 3).T
    Q = golden[key + "/oracle_q"].reshape(3, 3).T
    R = golden[key + "/oracle_r"].reshape(3, 3).T
    assert np.max(np.abs(Q @ R - A)) <= 1e-12
    assert np.max(np.abs(Q.T @ Q - np.eye(3))) <= 1e-12


def test_trsv_oracle_pin(golden):
    keys = cases(golden, "trsv_d/")
    assert len(keys) == 40
    for key in keys:
        uplo, trans, n, lda, incx = map(int, key.split("/")[1].split("_"))
        x = golden[key + "/x"].copy()
        assert oracle.trsv(uplo, trans, n, golden[key + "/a"], lda, x, incx) == 0
        np.testing.assert_array_equal(x.view(np.uint8), golden[key + "/oracle"].view(np.uint8))
        exp = golden[key + "/lapack"]
        scale = max(1.0, np.max(np.abs(exp)))
        # BlasTests.SolveTriangularDouble.cs:54 uses 1e-11 absolute on its (well-scaled) inputs;
        # the seeded stand-in inputs are scaled here by the solution's magnitude.
        assert np.max(np.abs(x - exp)) <= 1e-11 * scale, key


def test_gemm_oracle_pin(golden):
    keys = cases(golden, "gemm_d/")
    assert len(keys) == 39
    for key in keys:
        f = key.split("/")[1].split("_")
        mode = f[0]
        m, n, k, lda, ldb, ldc = map(int, f[1:])
        c = golden[key + "/c"].copy()
        ta = NT if mode[0] == "N" else T
        tb = NT if mode[1] == "N" else T
        assert oracle.gemm(ta, tb, m, n, k, golden[key + "/a"], lda, golden[key + "/b"], ldb,
                           c, ldc) == 0
        np.testing.assert_array_equal(c.view(np.uint8), golden[key + "/oracle"].view(np.uint8))
        assert np.max(np.abs(c - golden[key + "/lapack"])) <= 1e-12, key  # MulMatMatDouble.cs:51


def test_lu_inverse_oracle_pin(golden):
    for key in cases(golden, "luinv_d/"):
        n, lda = map(int, key.split("/")[1].split("_"))
        a0 = golden[key + "/in"]
        inv = golden[key + "/lu"].copy()
        assert oracle.lu_inverse(n, inv, lda, golden[key + "/piv"]) == 0
        np.testing.assert_array_equal(inv.view(np.uint8), golden[key + "/oracle"].view(np.uint8))
        A = a0[:n * lda].reshape(n, lda).T[:n]
        X = inv[:n * lda].reshape(n, lda).T[:n]
        assert np.max(np.abs(A @ X - np.eye(n))) <= 1e-12, key   # LuInverseTests.cs:118-122
        for j in range(n):   # padding rows unchanged (LuInverseTests.cs:127-134)
            np.testing.assert_array_equal(inv[j * lda + n:(j + 1) * lda], a0[j * lda + n:(j + 1) * lda])


@pytest.mark.parametrize("prec", ["s", "z"])
def test_lu_inverse_types_oracle_pin(golden, prec):
    """Float and Complex LuInverse on the reference's shapes (LuInverseTests.cs:12-72,
    :138-204): bits against the fixture, A X = I at the reference's tolerance (float: 1e-5,
    :55-59, widened by the first-order bound n eps cond(A) for the one ill-conditioned draw;
    Complex: 1e-12, :184-190), padding rows unchanged."""
    keys = cases(golden, "luinv_%s/" % prec)
    assert keys
    for key in keys:
        n, lda = map(int, key.split("/")[1].split("_"))
        a0 = golden[key + "/in"]
        inv = golden[key + "/lu"].copy()
        assert oracle.lu_inverse(n, inv, lda, golden[key + "/piv"]) == 0
        np.testing.assert_array_equal(inv.view(np.uint8), golden[key + "/oracle"].view(np.uint8),
                                      err_msg=key)
        wide = np.complex128 if prec == "z" else np.float64
        A = a0[:n * lda].reshape(n, lda).T[:n].astype(wide)
        X = inv[:n * lda].reshape(n, lda).T[:n].astype(wide)
        if prec == "s":
            tol = max(1e-5, n * 2.0 ** -24 * np.linalg.cond(A))
        else:
            tol = 1e-12
        assert np.max(np.abs(A @ X - np.eye(n))) <= tol, key
        for j in range(n):
            np.testing.assert_array_equal(inv[j * lda + n:(j + 1) * lda],
                                          a0[j * lda + n:(j + 1) * lda])


@pytest.mark.parametrize("prec", ["d", "s", "z"])
def test_gevd_front_oracle_pin(golden, prec):
    """The GEVD front half on the reference's shapes (GevdTests.cs:12-21, :96-105, :180-189) with
    A and B's strict lower parts NaN, as the reference passes them: bits against the fixture,
    only the upper triangles read (C finite), padding rows of B unchanged, L and
    C = L^-1 A L^-T (L^-H) against LAPACK to a first-order bound, 10 n eps cond(B), relative to
    the largest entry."""
    keys = cases(golden, "gevd_%s/" % prec)
    assert keys
    eps = 2.0 ** -24 if prec == "s" else 2.0 ** -53
    for key in keys:
        n, lda, ldb = map(int, key.split("/")[1].split("_"))
        a, b0 = golden[key + "/a"], golden[key + "/b"]
        b, c = b0.copy(), np.zeros(n * n, a.dtype)
        assert oracle.gevd_front(n, a, lda, b, ldb, c) == 0
        np.testing.assert_array_equal(b.view(np.uint8), golden[key + "/oracle_b"].view(np.uint8),
                                      err_msg=key)
        np.testing.assert_array_equal(c.view(np.uint8), golden[key + "/oracle_c"].view(np.uint8),
                                      err_msg=key)
        assert np.isfinite(c.view(np.float32 if prec == "s" else np.float64)).all(), key
        for j in range(n):
            np.testing.assert_array_equal(b[j * ldb + n:(j + 1) * ldb], b0[j * ldb + n:(j + 1) * ldb])
        ll, lc = golden[key + "/lapack_l"], golden[key + "/lapack_c"]
        L = np.tril(b[:n * ldb].reshape(n, ldb).T[:n].astype(ll.dtype))
        LL = np.tril(ll[:n * ldb].reshape(n, ldb).T[:n])
        tol = 10 * n * eps * np.linalg.cond(LL @ LL.conj().T)
        assert np.max(np.abs(L - LL)) <= tol * np.max(np.abs(LL)), key
        assert np.max(np.abs(c - lc)) <= tol * np.max(np.abs(lc)), key


def test_oracle_no_fma_contract():
    """A case whose result differs between fused and unfused evaluation: the oracle must not
    contract x0*y0 + x1*y1 into an FMA."""
    x = np.array([1.0 + 2.0 ** -30, 1.0 - 2.0 ** -30])
    y = np.array([1.0 - 2.0 ** -30, -(1.0 + 2.0 ** -30)])
    c = np.zeros(1)
    oracle.gemm(T, NT, 1, 1, 2, x, 2, y, 2, c, 1)
    p0 = x[0] * y[0]
    p1 = x[1] * y[1]
    assert c[0] == 0.0 + (p0 + p1)


def test_batched_oracle_matches_single():
    """The batched drivers compose the single routines exactly (threads change nothing)."""
    rng = np.random.default_rng(3)
    n = rng.integers(1, 40, size=37).astype(np.int32)
    a_off = np.concatenate([[0], np.cumsum(n.astype(np.int64) ** 2)[:-1]])
    a = rng.standard_normal(int((n.astype(np.int64) ** 2).sum()))
    piv_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]])
    b_off = piv_off * 2
    b = rng.standard_normal(int(n.sum()) * 2)
    outs = []
    for threads in (1, 4):
        aa, bb = a.copy(), b.copy()
        piv = np.zeros(int(n.sum()), np.int32)
        sign = np.zeros(len(n), np.int32)
        oracle.lu_solve_batched(n, a_off, aa, piv_off, piv, b_off, bb, 2, sign, threads)
        outs.append((aa, bb, piv, sign))
    for x, y in zip(outs[0], outs[1]):
        np.testing.assert_array_equal(x, y)
    # matrix 5 by hand
    i = 5
    ni = int(n[i])
    a5 = a[a_off[i]:a_off[i] + ni * ni].copy()
    p5 = np.zeros(ni, np.int32)
    oracle.lu(ni, ni, a5, ni, p5)
    np.testing.assert_array_equal(a5, outs[0][0][a_off[i]:a_off[i] + ni * ni])
    b5 = b[b_off[i]:b_off[i] + 2 * ni].copy()
    oracle.lu_solve(ni, a5, ni, p5, 2, b5, ni)
    np.testing.assert_array_equal(b5, outs[0][1][b_off[i]:b_off[i] + 2 * ni])
    A = a[a_off[i]:a_off[i] + ni * ni].reshape(ni, ni).T
    X = b5.reshape(2, ni).T
    B = b[b_off[i]:b_off[i] + 2 * ni].reshape(2, ni).T
    assert np.max(np.abs(A @ X - B)) <= 1e-9 * max(1, np.max(np.abs(X)))


# ---- float and Complex overloads --------------------------------------------------------------

def test_lu_complex_oracle_pin(golden):
    keys = cases(golden, "lu_z/")
    assert keys
    for key in keys:
        m, n, lda = map(int, key.split("/")[1].split("_"))
        a = golden[key + "/in"].copy()
        piv = np.zeros(m, np.int32)
        oracle.lu(m, n, a, lda, piv)
        np.testing.assert_array_equal(a.view(np.uint8), golden[key + "/oracle"].view(np.uint8))
        assert np.max(np.abs(a - golden[key + "/lapack"])) <= 1e-12, key   # LuTests.cs:234-235


@pytest.mark.parametrize("prec,tol", [("s", 1e-5), ("z", 1e-12)])
def test_cholesky_float_complex_oracle_pin(golden, prec, tol):
    keys = cases(golden, "chol_%s/" % prec)
    assert keys
    for key in keys:
        _, n, lda = key.split("/")[1].split("_")
        n, lda = int(n), int(lda)
        a = golden[key + "/in"].copy()
        info = oracle.cholesky(n, a, lda)
        assert info == golden[key + "/oracle_info"][0]
        assert (info == 0) == (golden[key + "/lapack_info"][0] == 0), key
        if info == 0:
            np.testing.assert_array_equal(a.view(np.uint8), golden[key + "/oracle"].view(np.uint8))
            exp = golden[key + "/lapack"]
            for j in range(n):
                col = slice(j * lda, j * lda + n)
                assert np.max(np.abs(a[col] - exp[col])) <= tol, key


def test_qr_complex_oracle_pin(golden):
    for key in cases(golden, "qr_z/"):
        m, n, lda, ldq, ldr = map(int, key.split("/")[1].split("_"))
        a = golden[key + "/in"].copy()
        rd = np.zeros(n)
        oracle.qr(m, n, a, lda, rd)
        q = golden[key + "/q_in"].copy()
        oracle.qr_q(m, n, a, lda, q, ldq)
        r = golden[key + "/r_in"].copy()
        oracle.qr_r(m, n, a, lda, r, ldr, rd)
        for got, name in ((a, "oracle"), (rd, "oracle_rdiag"), (q, "oracle_q"), (r, "oracle_r")):
            np.testing.assert_array_equal(got.view(np.uint8), golden[key + "/" + name].view(np.uint8))
        A = golden[key + "/in"][:n * lda].reshape(n, lda).T[:m]
        Q = q[:n * ldq].reshape(n, ldq).T[:m]
        R = r[:n * ldr].reshape(n, ldr).T[:n]
        assert np.max(np.abs(Q @ R - A)) <= 1e-12, key                        # QrTests.cs:452-470
        assert np.max(np.abs(Q.conj().T @ Q - np.eye(n))) <= 1e-12, key


@pytest.mark.parametrize("prec,tol", [("s", 1e-3), ("z", 1e-11)])
def test_trsv_float_complex_oracle_pin(golden, prec, tol):
    keys = cases(golden, "trsv_%s/" % prec)
    assert len(keys) == (40 if prec == "s" else 80)
    for key in keys:
        uplo, trans, n, lda, incx = map(int, key.split("/")[1].split("_"))
        x = golden[key + "/x"].copy()
        assert oracle.trsv(uplo, trans, n, golden[key + "/a"], lda, x, incx) == 0
        np.testing.assert_array_equal(x.view(np.uint8), golden[key + "/oracle"].view(np.uint8))
        exp = golden[key + "/lapack"]
        assert np.max(np.abs(x - exp)) <= tol * max(1.0, np.max(np.abs(exp))), key


@pytest.mark.parametrize("prec,tol", [("s", 1e-6), ("z", 1e-12)])
def test_gemm_float_complex_oracle_pin(golden, prec, tol):
    keys = cases(golden, "gemm_%s/" % prec)
    assert len(keys) == (39 if prec == "s" else 156)
    for key in keys:
        ta, tb, m, n, k, lda, ldb, ldc = map(int, key.split("/")[1].split("_"))
        c = golden[key + "/c"].copy()
        assert oracle.gemm(ta, tb, m, n, k, golden[key + "/a"], lda, golden[key + "/b"], ldb,
                           c, ldc) == 0
        np.testing.assert_array_equal(c.view(np.uint8), golden[key + "/oracle"].view(np.uint8))
        assert np.max(np.abs(c - golden[key + "/lapack"])) <= tol, key

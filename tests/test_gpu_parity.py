"""Parity of the CUDA library with the MatFlat oracle: bit for bit, through the C ABI.

Every test here is marked gpu.  Inputs are the committed golden vectors (the reference test
suite's shapes and literal fixtures) plus larger seeded cases checked against the oracle live.
"""
import numpy as np
import pytest

from oracle import oracle
from tests.conftest import cases

pytestmark = pytest.mark.gpu

U, L, NT, T = 121, 122, 111, 112


def bits(x):
    return np.ascontiguousarray(x).view(np.uint8)


def assert_bits(got, exp, msg=""):
    """Bit-identical, except that a NaN only has to be a NaN: the payload and sign of a NaN
    produced by 0/0 or inf-inf differ between CPU architectures and the GPU."""
    got = np.ascontiguousarray(got)
    exp = np.ascontiguousarray(exp)
    assert got.shape == exp.shape, msg
    gn, en = np.isnan(got), np.isnan(exp)
    np.testing.assert_array_equal(gn, en, err_msg=msg + " (NaN positions)")
    np.testing.assert_array_equal(bits(np.where(gn, 0, got)), bits(np.where(en, 0, exp)),
                                  err_msg=msg)


# ------------------------------------------------------------------------------------------
# Single-matrix drop-ins against the golden vectors (reference test shapes).

def test_lu_golden(mf, golden):
    for key in cases(golden, "lu_d/"):
        dims = key.split("/")[1]
        m, n, lda = (3, 3, 3) if dims.startswith("lit_") else map(int, dims.split("_"))
        a = golden[key + "/in"].copy()
        piv = np.zeros(m, np.int32)
        sign = mf.Factorization.Lu(m, n, a, lda, piv)
        assert_bits(a, golden[key + "/oracle"], key)
        np.testing.assert_array_equal(piv, golden[key + "/oracle_piv"], err_msg=key)
        assert sign == golden[key + "/oracle_sign"][0], key


def test_cholesky_golden(mf, golden):
    for key in cases(golden, "chol_d/"):
        _, n, lda = key.split("/")[1].split("_")
        n, lda = int(n), int(lda)
        a = golden[key + "/in"].copy()
        if golden[key + "/oracle_info"][0] != 0:
            with pytest.raises(mf.MatrixFactorizationException):
                mf.Factorization.Cholesky(n, a, lda)
        else:
            mf.Factorization.Cholesky(n, a, lda)
            assert_bits(a, golden[key + "/oracle"], key)


@pytest.mark.parametrize("prec", ["d", "s"])
def test_qr_golden(mf, golden, prec):
    for key in cases(golden, "qr_%s/" % prec):
        dims = key.split("/")[1]
        if dims.startswith("lit_"):
            m, n, lda, ldq, ldr = 3, 3, 3, 3, 3
            qin = np.zeros(9)
            rin = np.zeros(9)
        else:
            m, n, lda, ldq, ldr = map(int, dims.split("_"))
            qin = golden[key + "/q_in"]
            rin = golden[key + "/r_in"]
        a = golden[key + "/in"].copy()
        rd = np.zeros(n, a.dtype)
        mf.Factorization.Qr(m, n, a, lda, rd)
        assert_bits(a, golden[key + "/oracle"], key)
        assert_bits(rd, golden[key + "/oracle_rdiag"], key)
        q = qin.copy()
        mf.Factorization.QrOrthogonalFactor(m, n, a, lda, q, ldq)
        assert_bits(q, golden[key + "/oracle_q"], key)
        r = rin.copy()
        mf.Factorization.QrUpperTriangularFactor(m, n, a, lda, r, ldr, rd)
        assert_bits(r, golden[key + "/oracle_r"], key)


def test_trsv_golden(mf, golden):
    for key in cases(golden, "trsv_d/"):
        uplo, trans, n, lda, incx = map(int, key.split("/")[1].split("_"))
        x = golden[key + "/x"].copy()
        mf.Blas.SolveTriangular(uplo, trans, n, golden[key + "/a"], lda, x, incx)
        assert_bits(x, golden[key + "/oracle"], key)


def test_gemm_golden(mf, golden):
    for key in cases(golden, "gemm_d/"):
        f = key.split("/")[1].split("_")
        m, n, k, lda, ldb, ldc = map(int, f[1:])
        c = golden[key + "/c"].copy()
        mf.Blas.MulMatMat(NT if f[0][0] == "N" else T, NT if f[0][1] == "N" else T, m, n, k,
                          golden[key + "/a"], lda, golden[key + "/b"], ldb, c, ldc)
        assert_bits(c, golden[key + "/oracle"], key)


@pytest.mark.parametrize("prec", ["d", "s", "z"])
def test_lu_inverse_golden(mf, golden, prec):
    keys = cases(golden, "luinv_%s/" % prec)
    assert keys
    for key in keys:
        n, lda = map(int, key.split("/")[1].split("_"))
        a = golden[key + "/lu"].copy()
        mf.Factorization.LuInverse(n, a, lda, golden[key + "/piv"])
        exp = golden[key + "/oracle"]
        if prec == "z":
            a, exp = a.view(np.float64), exp.view(np.float64)
        assert_bits(a, exp, key)


@pytest.mark.parametrize("prec", ["d", "s", "z"])
def test_gevd_front_golden(mf, golden, prec):
    """The batched GEVD front half on the reference's shapes (GevdTests.cs), all ten pairs in one
    plan with their own lda and ldb, strict lower parts of A and B NaN as the reference passes
    them: B (L and padding) and C bit-identical to the oracle fixture."""
    import torch
    keys = cases(golden, "gevd_%s/" % prec)
    dims = [tuple(map(int, k.split("/")[1].split("_"))) for k in keys]
    n = np.array([d[0] for d in dims], np.int32)
    lda = np.array([d[1] for d in dims], np.int32)
    ldb = np.array([d[2] for d in dims], np.int32)
    a = np.concatenate([golden[k + "/a"] for k in keys])
    b = np.concatenate([golden[k + "/b"] for k in keys])
    off = lambda sz: np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    a_off, b_off = off(lda.astype(np.int64) * n), off(ldb.astype(np.int64) * n)
    c_off = off(n.astype(np.int64) ** 2)
    flat = (lambda x: x.view(np.float64)) if prec == "z" else (lambda x: x)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    dc = torch.from_numpy(np.zeros(int((n.astype(np.int64) ** 2).sum()), a.dtype)).cuda()
    dinfo = torch.full((len(n),), -3, dtype=torch.int32, device="cuda")
    plan = mf.GevdFrontBatch(n, a_off, b_off, c_off, lda=lda, ldb=ldb)
    plan.run(da, db, dc, dinfo)
    mf.context().synchronize()
    assert (dinfo.cpu().numpy() == 0).all()
    gb, gc = db.cpu().numpy(), dc.cpu().numpy()
    for i, k in enumerate(keys):
        sb = slice(b_off[i], b_off[i] + ldb[i] * n[i])
        sc = slice(c_off[i], c_off[i] + n[i] * n[i])
        assert_bits(flat(gb[sb]), flat(golden[k + "/oracle_b"]), k + " B")
        assert_bits(flat(gc[sc]), flat(golden[k + "/oracle_c"]), k + " C")
    plan.close()


# ------------------------------------------------------------------------------------------
# Larger single matrices against the oracle run live.

@pytest.mark.parametrize("m,n,lda", [(64, 64, 64), (100, 100, 101), (128, 128, 128),
                                     (130, 97, 131), (70, 140, 75), (257, 257, 257)])
def test_lu_large(mf, m, n, lda):
    rng = np.random.default_rng(m * 1000 + n)
    a0 = rng.standard_normal(lda * n)
    a, b = a0.copy(), a0.copy()
    pg, po = np.zeros(m, np.int32), np.zeros(m, np.int32)
    sg = mf.Factorization.Lu(m, n, a, lda, pg)
    so = oracle.lu(m, n, b, lda, po)
    assert_bits(a, b)
    np.testing.assert_array_equal(pg, po)
    assert sg == so


@pytest.mark.parametrize("n,lda", [(64, 64), (97, 100), (128, 128), (150, 151)])
def test_cholesky_large(mf, n, lda):
    rng = np.random.default_rng(n)
    bm = rng.standard_normal((n, n))
    s = bm @ bm.T + n * np.eye(n)
    a0 = np.full(lda * n, np.nan)
    for j in range(n):
        a0[j * lda:j * lda + j + 1] = s[:j + 1, j]       # upper triangle, NaN below
    a, b = a0.copy(), a0.copy()
    mf.Factorization.Cholesky(n, a, lda)
    assert oracle.cholesky(n, b, lda) == 0
    assert_bits(a, b)


@pytest.mark.parametrize("m,n", [(200, 50), (512, 64), (65, 65), (300, 1)])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_qr_large(mf, m, n, dtype):
    rng = np.random.default_rng(m + n)
    a0 = rng.standard_normal(m * n).astype(dtype)
    a, b = a0.copy(), a0.copy()
    rg, ro = np.zeros(n, dtype), np.zeros(n, dtype)
    mf.Factorization.Qr(m, n, a, m, rg)
    oracle.qr(m, n, b, m, ro)
    assert_bits(a, b)
    assert_bits(rg, ro)
    qg, qo = np.zeros(m * n, dtype), np.zeros(m * n, dtype)
    mf.Factorization.QrOrthogonalFactor(m, n, a, m, qg, m)
    oracle.qr_q(m, n, b, m, qo, m)
    assert_bits(qg, qo)


@pytest.mark.parametrize("uplo,trans", [(U, NT), (L, NT), (U, T), (L, T)])
def test_trsv_large(mf, uplo, trans):
    n, lda, incx = 200, 203, 3
    rng = np.random.default_rng(7)
    a = rng.standard_normal(lda * n)
    for j in range(n):
        a[j * lda + j] = 4.0 + abs(a[j * lda + j])
    x0 = rng.standard_normal((n - 1) * incx + 1)
    x, y = x0.copy(), x0.copy()
    mf.Blas.SolveTriangular(uplo, trans, n, a, lda, x, incx)
    oracle.trsv(uplo, trans, n, a, lda, y, incx)
    assert_bits(x, y)


def test_lu_special_values(mf):
    """NaN in the first candidate keeps the pivot (strict '>' scan), NaN elsewhere is never
    chosen, signed zeros and infinities follow MatFlat."""
    cases_ = []
    a = np.array([np.nan, 1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0])
    cases_.append(a)
    a = np.array([1.0, np.nan, 5.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0])
    cases_.append(a)
    a = np.array([-0.0, 0.0, -0.0, 1.0, np.inf, 2.0, -np.inf, 3.0, 1e-310])
    cases_.append(a)
    a = np.array([2.0, -2.0, 2.0, 1.0, 1.0, 1.0, 0.0, 5.0, -5.0])
    cases_.append(a)
    for a0 in cases_:
        a, b = a0.copy(), a0.copy()
        pg, po = np.zeros(3, np.int32), np.zeros(3, np.int32)
        sg = mf.Factorization.Lu(3, 3, a, 3, pg)
        so = oracle.lu(3, 3, b, 3, po)
        assert_bits(a, b)
        np.testing.assert_array_equal(pg, po)
        assert sg == so


def test_argument_errors(mf):
    a = np.zeros(9)
    piv = np.zeros(3, np.int32)
    with pytest.raises(mf.ArgumentException):
        mf.Factorization.Lu(0, 3, a, 3, piv)
    with pytest.raises(mf.ArgumentException):
        mf.Factorization.Lu(3, 3, a, 2, piv)
    with pytest.raises(mf.ArgumentNullException):
        mf.Factorization.Lu(3, 3, None, 3, piv)
    with pytest.raises(mf.ArgumentNullException):
        mf.Factorization.Cholesky(3, None, 3)
    with pytest.raises(mf.ArgumentException):
        mf.Factorization.Qr(2, 3, np.zeros(9), 2, np.zeros(3))
    with pytest.raises(mf.ArgumentException):
        mf.Blas.SolveTriangular(U, NT, 3, a, 3, np.zeros(3), 0)
    with pytest.raises(mf.ArgumentException):
        mf.Blas.SolveTriangular(123, NT, 3, a, 3, np.zeros(3), 1)
    with pytest.raises(mf.ArgumentException):
        mf.Blas.MulMatMat(NT, NT, 3, 3, 3, a, 3, a, 3, a, 3)    # in place
    with pytest.raises(mf.MatrixFactorizationException):
        mf.Factorization.LuInverse(3, np.zeros(9), 3, np.arange(3, dtype=np.int32))


# ------------------------------------------------------------------------------------------
# Batched paths (device buffers through torch), uneven sizes, against the oracle.

def _dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def _host(t):
    return t.cpu().numpy()


def test_lu_batched(mf):
    import torch
    rng = np.random.default_rng(11)
    n = rng.integers(1, 141, size=300).astype(np.int32)    # includes n > 128 (global scratch)
    n[:5] = [1, 2, 3, 128, 129]
    nrhs = 4
    sz = n.astype(np.int64) ** 2
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]])
    a = rng.standard_normal(int(sz.sum()))
    a[a_off[7]:a_off[7] + n[7] * n[7]] = 0.0                # an all-zero (singular) matrix
    piv_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]])
    b_off = piv_off * nrhs
    b = rng.standard_normal(int(n.sum()) * nrhs)
    batch = mf.LuBatch(n, a_off, piv_off, nrhs=nrhs, b_off=b_off)
    da, db = _dev(a), _dev(b)
    dpiv = torch.zeros(int(n.sum()), dtype=torch.int32, device="cuda")
    dsign = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    for _ in range(2):   # twice: the second run replays the captured graph
        da.copy_(_dev(a))
        db.copy_(_dev(b))
        torch.cuda.synchronize()     # the copies run on torch's stream, the plan on its own
        batch.run(da, dpiv, db, dsign, dinfo)
        mf.context().synchronize()
    oa, ob = a.copy(), b.copy()
    opiv = np.zeros(int(n.sum()), np.int32)
    osign = np.zeros(len(n), np.int32)
    oracle.lu_solve_batched(n, a_off, oa, piv_off, opiv, b_off, ob, nrhs, osign, 4)
    assert_bits(_host(da), oa)
    np.testing.assert_array_equal(_host(dpiv), opiv)
    np.testing.assert_array_equal(_host(dsign), osign)
    assert_bits(_host(db), ob)
    info = _host(dinfo)
    assert info[7] == 1 and info[0] == 0


def test_cholesky_batched(mf):
    import torch
    rng = np.random.default_rng(12)
    n = rng.integers(1, 141, size=200).astype(np.int32)
    mats = []
    for i, ni in enumerate(n):
        bm = rng.standard_normal((ni, ni))
        s = bm @ bm.T + ni * np.eye(ni)
        if i % 37 == 5:
            s[ni // 2, ni // 2] = -1.0     # not positive definite
        mats.append(np.asfortranarray(s).reshape(-1, order="F"))
    sz = n.astype(np.int64) ** 2
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]])
    a = np.concatenate(mats)
    b_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]])
    b = rng.standard_normal(int(n.sum()))
    batch = mf.CholeskyBatch(n, a_off, nrhs=1, b_off=b_off)
    da, db = _dev(a), _dev(b)
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    batch.run(da, db, dinfo)
    mf.context().synchronize()
    oa, ob = a.copy(), b.copy()
    oinfo = np.zeros(len(n), np.int32)
    oracle.chol_solve_batched(n, a_off, oa, b_off, ob, oinfo, 4)
    ginfo = _host(dinfo)
    np.testing.assert_array_equal(ginfo, oinfo)
    assert (oinfo != 0).any()
    ga, gb = _host(da), _host(db)
    for i in range(len(n)):
        if oinfo[i] == 0:
            sl = slice(a_off[i], a_off[i] + sz[i])
            assert_bits(ga[sl], oa[sl], "matrix %d" % i)
            bl = slice(b_off[i], b_off[i] + n[i])
            assert_bits(gb[bl], ob[bl], "rhs %d" % i)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_qr_batched_least_squares(mf, dtype):
    import torch
    rng = np.random.default_rng(13)
    count = 120
    m = rng.integers(1, 300, size=count).astype(np.int32)
    n = np.minimum(rng.integers(1, 70, size=count), m).astype(np.int32)
    m[:3], n[:3] = [1, 64, 512], [1, 64, 64]
    sz = m.astype(np.int64) * n
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]])
    a = rng.standard_normal(int(sz.sum())).astype(dtype)
    r_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]])
    b_off = np.concatenate([[0], np.cumsum(m.astype(np.int64))[:-1]])
    b = rng.standard_normal(int(m.sum())).astype(dtype)
    batch = mf.QrBatch(m, n, a_off, r_off, nrhs=1, b_off=b_off)
    da, db = _dev(a), _dev(b)
    dr = torch.zeros(int(n.sum()), dtype=da.dtype, device="cuda")
    batch.run(da, dr, db, single=(dtype == np.float32))
    mf.context().synchronize()
    ga, gr, gb = _host(da), _host(dr), _host(db)
    tol = 1e-9 if dtype == np.float64 else 2e-3
    for i in range(count):
        mi, ni = int(m[i]), int(n[i])
        ai = a[a_off[i]:a_off[i] + mi * ni].copy()
        ri = np.zeros(ni, dtype)
        oracle.qr(mi, ni, ai, mi, ri)
        assert_bits(ga[a_off[i]:a_off[i] + mi * ni], ai, "factors %d" % i)
        assert_bits(gr[r_off[i]:r_off[i] + ni], ri, "rdiag %d" % i)
        # Least squares: compare with the oracle's composition of MatFlat routines through the
        # normal-equation residual ||A^T (A x - b)|| relative to ||A|| ||b||.
        a0 = a[a_off[i]:a_off[i] + mi * ni].copy()
        bi = b[b_off[i]:b_off[i] + mi]
        xo = np.zeros(ni, dtype)
        oracle.qr_ls(mi, ni, a0.copy(), mi, bi.copy(), xo)
        xg = gb[b_off[i]:b_off[i] + ni]
        A = a0.reshape(ni, mi).T.astype(np.float64)
        scale = np.linalg.norm(A) * np.linalg.norm(bi) + 1e-300
        for x in (xg, xo):
            res = np.linalg.norm(A.T @ (A @ x.astype(np.float64) - bi))
            assert res / scale <= tol, (i, res / scale)
        assert np.max(np.abs(xg - xo)) <= tol * 1e3 * max(1.0, np.max(np.abs(xo)))


@pytest.mark.parametrize("table", [-1, 0, 1, 2, 3, 4, 5, 6])
def test_lu_batched_every_lanes_table(mf, table, monkeypatch):
    """Every lanes-per-matrix table of the size-bucketed LU (8, 16 or 32 lanes per matrix by
    order; -1 the one-matrix-per-warp queue) gives the oracle's factors, pivots, signs and
    solutions bit for bit, over orders 1..140 and uneven, ragged tasks."""
    import torch
    monkeypatch.setenv("MFG_LU_GROUPS", str(table))
    rng = np.random.default_rng(40 + table)
    n = rng.integers(1, 141, size=157).astype(np.int32)
    n[:9] = [1, 2, 8, 9, 48, 49, 96, 128, 129]
    nrhs = 4
    sz = n.astype(np.int64) ** 2
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]])
    a = rng.standard_normal(int(sz.sum()))
    a[a_off[11]:a_off[11] + n[11] * n[11]] = 0.0
    piv_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]])
    b_off = piv_off * nrhs
    b = rng.standard_normal(int(n.sum()) * nrhs)
    batch = mf.LuBatch(n, a_off, piv_off, nrhs=nrhs, b_off=b_off)
    da, db = _dev(a), _dev(b)
    dpiv = torch.zeros(int(n.sum()), dtype=torch.int32, device="cuda")
    dsign = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    batch.run(da, dpiv, db, dsign, dinfo)
    mf.context().synchronize()
    oa, ob = a.copy(), b.copy()
    opiv = np.zeros(int(n.sum()), np.int32)
    osign = np.zeros(len(n), np.int32)
    oracle.lu_solve_batched(n, a_off, oa, piv_off, opiv, b_off, ob, nrhs, osign, 4)
    assert_bits(_host(da), oa)
    np.testing.assert_array_equal(_host(dpiv), opiv)
    np.testing.assert_array_equal(_host(dsign), osign)
    assert_bits(_host(db), ob)
    assert _host(dinfo)[11] == 1


@pytest.mark.parametrize("env", [
    {"MFG_LU_GROUPS": "0", "MFG_WARPS_PER_SM": "28"},
    {"MFG_LU_GROUPS": "2", "MFG_WARPS_PER_SM": "32"},
    {"MFG_LU_BLK": "1,4,2"},
    {"MFG_LU_BLK": "60,2,5"},
    {"MFG_LU_BLK": "100,4,1"},
    {"MFG_LU_BLK": "1,8,3"},
], ids=["occ28", "occ32", "res-4x2", "res-2x5", "res-4x1", "res-8x3"])
def test_lu_batched_launch_forms(mf, env, monkeypatch):
    """The register-bounded variants of the task kernel (28 and 32 warps per SM) and the resident
    form (one matrix per CTA of 2, 4 or 8 warps, the matrix in shared memory when it fits, in
    global memory otherwise) give the oracle's factors, pivots, signs and solutions bit for bit,
    over orders 1..140 including a zero matrix, NaN and infinite entries and tied pivots."""
    import torch
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    rng = np.random.default_rng(77)
    n = rng.integers(1, 141, size=160).astype(np.int32)
    n[:10] = [1, 2, 8, 9, 48, 60, 96, 100, 128, 129]
    nrhs = 4
    sz = n.astype(np.int64) ** 2
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]])
    a = rng.standard_normal(int(sz.sum()))
    a[a_off[11]:a_off[11] + n[11] * n[11]] = 0.0
    a[a_off[12] + 5] = np.nan
    a[a_off[13] + 3] = np.inf
    m14 = a[a_off[14]:a_off[14] + n[14] * n[14]].reshape(n[14], n[14], order="F")
    m14[:, 0] = 1.0                       # every first-column candidate ties
    a[a_off[14]:a_off[14] + n[14] * n[14]] = m14.reshape(-1, order="F")
    piv_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]])
    b_off = piv_off * nrhs
    b = rng.standard_normal(int(n.sum()) * nrhs)
    batch = mf.LuBatch(n, a_off, piv_off, nrhs=nrhs, b_off=b_off)
    da, db = _dev(a), _dev(b)
    dpiv = torch.zeros(int(n.sum()), dtype=torch.int32, device="cuda")
    dsign = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    batch.run(da, dpiv, db, dsign, dinfo)
    mf.context().synchronize()
    oa, ob = a.copy(), b.copy()
    opiv = np.zeros(int(n.sum()), np.int32)
    osign = np.zeros(len(n), np.int32)
    oracle.lu_solve_batched(n, a_off, oa, piv_off, opiv, b_off, ob, nrhs, osign, 4)
    assert_bits(_host(da), oa)
    np.testing.assert_array_equal(_host(dpiv), opiv)
    np.testing.assert_array_equal(_host(dsign), osign)
    assert_bits(_host(db), ob)
    assert _host(dinfo)[11] == 1
    # Solve-only calls on the factors give the fused call's solutions.
    db2 = _dev(b)
    torch.cuda.synchronize()
    batch.solve(da, dpiv, db2)
    mf.context().synchronize()
    assert_bits(_host(db2), ob)


@pytest.mark.parametrize("table", [0, 1, 2])
def test_cholesky_batched_every_lanes_table(mf, table, monkeypatch):
    """The batched Cholesky + solve with lanes per matrix chosen per size bucket (4/8/16/32 lanes
    by order; 0: one group size for the plan) gives the oracle's factors, solutions and info bit
    for bit over orders 1..140."""
    import torch
    monkeypatch.setenv("MFG_CHOL_TABLE", str(table))
    rng = np.random.default_rng(60 + table)
    n = rng.integers(1, 141, size=150).astype(np.int32)
    n[:8] = [1, 4, 16, 17, 32, 33, 64, 129]
    mats = []
    for k in n:
        bm = rng.standard_normal((k, k))
        mats.append((bm @ bm.T + k * np.eye(k)).reshape(-1, order="F"))
    mats[9] = -mats[9]                                       # not positive definite
    a = np.concatenate(mats)
    sz = n.astype(np.int64) ** 2
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]])
    b_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]])
    b = rng.standard_normal(int(n.sum()))
    batch = mf.CholeskyBatch(n, a_off, nrhs=1, b_off=b_off)
    da, db = _dev(a), _dev(b)
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    batch.run(da, db, dinfo)
    mf.context().synchronize()
    oa, ob = a.copy(), b.copy()
    oinfo = np.zeros(len(n), np.int32)
    oracle.chol_solve_batched(n, a_off, oa, b_off, ob, oinfo, 4)
    gi = _host(dinfo)
    np.testing.assert_array_equal(gi, oinfo)
    ga, gb = _host(da), _host(db)
    for i in range(len(n)):
        if oinfo[i] != 0:
            continue
        s0, s1 = a_off[i], a_off[i] + sz[i]
        assert_bits(ga[s0:s1], oa[s0:s1])
        assert_bits(gb[b_off[i]:b_off[i] + n[i]], ob[b_off[i]:b_off[i] + n[i]])


@pytest.mark.parametrize("cta", ["0", "1"])
def test_lu_batched_large_orders_cta(mf, cta, monkeypatch):
    """Orders above 128 factored by a whole CTA per matrix (MFG_LU_CTA=1, the choice when few
    such matrices cannot fill the GPU with warps) or one warp per matrix (0): the same bits as
    the oracle, with small orders in the same batch."""
    import torch
    monkeypatch.setenv("MFG_LU_CTA", cta)
    rng = np.random.default_rng(70)
    n = np.concatenate([rng.integers(129, 301, size=14), rng.integers(1, 60, size=20),
                        [129, 300, 256]]).astype(np.int32)
    nrhs = 2
    sz = n.astype(np.int64) ** 2
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]])
    a = rng.standard_normal(int(sz.sum()))
    a[a_off[3]:a_off[3] + sz[3]] = 0.0
    piv_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]])
    b_off = piv_off * nrhs
    b = rng.standard_normal(int(n.sum()) * nrhs)
    batch = mf.LuBatch(n, a_off, piv_off, nrhs=nrhs, b_off=b_off)
    da, db = _dev(a), _dev(b)
    dpiv = torch.zeros(int(n.sum()), dtype=torch.int32, device="cuda")
    dsign = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    dinfo = torch.zeros(len(n), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    batch.run(da, dpiv, db, dsign, dinfo)
    mf.context().synchronize()
    oa, ob = a.copy(), b.copy()
    opiv = np.zeros(int(n.sum()), np.int32)
    osign = np.zeros(len(n), np.int32)
    oracle.lu_solve_batched(n, a_off, oa, piv_off, opiv, b_off, ob, nrhs, osign, 4)
    assert_bits(_host(da), oa)
    np.testing.assert_array_equal(_host(dpiv), opiv)
    np.testing.assert_array_equal(_host(dsign), osign)
    assert_bits(_host(db), ob)
    assert _host(dinfo)[3] == 1

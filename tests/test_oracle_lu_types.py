"""The oracle's batched float / Complex LU + solve: equal, bit for bit, to composing its pinned
single-matrix routines (Factorization.Lu, then SolveTriangular Lower with a unit diagonal and
Upper, both NoTrans, after permuting b), and a solution of A x = b to working precision."""
import numpy as np
import pytest

from oracle import oracle

NT, U, L = 111, 121, 122


def _draw(rng, k, dt):
    if dt == np.complex128:
        return rng.standard_normal(k) + 1j * rng.standard_normal(k)
    return rng.standard_normal(k).astype(dt)


@pytest.mark.parametrize("dt", [np.float32, np.complex128])
def test_batched_equals_single_composition(dt):
    rng = np.random.default_rng(21)
    nrhs = 3
    n = np.array([1, 2, 7, 16, 31, 40], np.int32)
    a_off = np.concatenate([[0], np.cumsum(n.astype(np.int64) ** 2)[:-1]]).astype(np.int64)
    piv_off = np.concatenate([[0], np.cumsum(n)[:-1]]).astype(np.int64)
    b_off = np.concatenate([[0], np.cumsum(n.astype(np.int64) * nrhs)[:-1]]).astype(np.int64)
    a = _draw(rng, int((n.astype(np.int64) ** 2).sum()), dt)
    b = _draw(rng, int(n.sum()) * nrhs, dt)
    ga, gb = a.copy(), b.copy()
    piv = np.zeros(int(n.sum()), np.int32)
    sign = np.zeros(len(n), np.int32)
    oracle.lu_solve_batched(n, a_off, ga, piv_off, piv, b_off, gb, nrhs, sign, 2)
    for i, ni in enumerate(n):
        ni = int(ni)
        ai = a[a_off[i]:a_off[i] + ni * ni].copy()
        pi = np.zeros(ni, np.int32)
        s = oracle.lu(ni, ni, ai, ni, pi)
        assert s == sign[i]
        np.testing.assert_array_equal(pi, piv[piv_off[i]:piv_off[i] + ni])
        assert ai.tobytes() == ga[a_off[i]:a_off[i] + ni * ni].tobytes()
        unit = ai.reshape(ni, ni, order="F").copy()
        np.fill_diagonal(unit, 1)
        unit = unit.flatten(order="F")
        bi = b[b_off[i]:b_off[i] + ni * nrhs].reshape(ni, nrhs, order="F")
        xi = gb[b_off[i]:b_off[i] + ni * nrhs].reshape(ni, nrhs, order="F")
        for r in range(nrhs):
            x = bi[pi, r].copy()
            oracle.trsv(L, NT, ni, unit, ni, x, 1)
            oracle.trsv(U, NT, ni, ai, ni, x, 1)
            assert x.tobytes() == np.ascontiguousarray(xi[:, r]).tobytes()
        A = a[a_off[i]:a_off[i] + ni * ni].reshape(ni, ni, order="F").astype(np.complex128)
        eps = 1e-4 if dt == np.float32 else 1e-12
        res = np.abs(A @ xi - bi).max() / max(1.0, np.abs(A).max() * np.abs(xi).max())
        assert res < eps * ni


@pytest.mark.parametrize("dt", [np.float32, np.complex128])
def test_batched_cholesky_solves(dt):
    """float: L y = b, L^T x = y; Complex: L y = b, L^H x = y — a solution of A x = b."""
    rng = np.random.default_rng(22)
    nrhs = 2
    n = np.array([1, 3, 8, 25, 40], np.int32)
    a_off = np.concatenate([[0], np.cumsum(n.astype(np.int64) ** 2)[:-1]]).astype(np.int64)
    b_off = np.concatenate([[0], np.cumsum(n.astype(np.int64) * nrhs)[:-1]]).astype(np.int64)
    mats = []
    for ni in n:
        m = _draw(rng, int(ni) * int(ni), dt).reshape(ni, ni)
        mats.append((m @ m.conj().T + ni * np.eye(ni)).astype(dt).flatten(order="F"))
    a = np.concatenate(mats)
    b = _draw(rng, int(n.sum()) * nrhs, dt)
    ga, gb = a.copy(), b.copy()
    info = np.full(len(n), -1, np.int32)
    oracle.chol_solve_batched(n, a_off, ga, b_off, gb, info, 2, nrhs=nrhs)
    assert (info == 0).all()
    for i, ni in enumerate(n):
        ni = int(ni)
        A = a[a_off[i]:a_off[i] + ni * ni].reshape(ni, ni, order="F").astype(np.complex128)
        Lf = ga[a_off[i]:a_off[i] + ni * ni].reshape(ni, ni, order="F")
        assert not np.triu(Lf, 1).any()
        x = gb[b_off[i]:b_off[i] + ni * nrhs].reshape(ni, nrhs, order="F")
        bi = b[b_off[i]:b_off[i] + ni * nrhs].reshape(ni, nrhs, order="F")
        eps = 1e-5 if dt == np.float32 else 1e-13
        assert np.abs(A @ x - bi).max() < eps * ni * np.abs(A).max() * max(1, np.abs(x).max())

"""Seeded synthetic batches with the shapes of the reference's benchmark configurations.

Host-side generation (libworkloads_synth.so, counter-based SplitMix64 + Box-Muller), so the GPU
path and the CPU oracle see identical bytes.  Every batch is packed: matrix i is column-major with
leading dimension equal to its row count, at element offset a_off[i].
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None


def _synth():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(_build.build())
        lib.mfs_normal.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint64,
                                   ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int]
        lib.mfs_uniform.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint64,
                                    ctypes.c_uint64, ctypes.c_uint64, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_int]
        _lib = lib
    return _lib


def _threads():
    return max(1, min(64, os.cpu_count() or 1))


def normal(count, seed, stream=0, offset=0, out=None):
    out = np.empty(count, np.float64) if out is None else out
    _synth().mfs_normal(out.ctypes.data, count, seed, stream, offset, _threads())
    return out


def uniform(count, seed, stream=0, offset=0, lo=0.0, hi=1.0, out=None):
    out = np.empty(count, np.float64) if out is None else out
    _synth().mfs_uniform(out.ctypes.data, count, seed, stream, offset, lo, hi, _threads())
    return out


def packed_offsets(rows, cols):
    sizes = np.asarray(rows, np.int64) * np.asarray(cols, np.int64)
    off = np.zeros(len(sizes), np.int64)
    if len(sizes) > 1:
        off[1:] = np.cumsum(sizes)[:-1]
    return off, int(sizes.sum())


def lu_batch(count, nmin=8, nmax=128, nrhs=4, seed=0):
    """LU + solve workload: n ~ U{nmin..nmax}, A ~ N(0,1), nrhs right-hand sides ~ N(0,1)."""
    n = (np.floor(uniform(count, seed, stream=1) * (nmax - nmin + 1)) + nmin).astype(np.int32)
    a_off, total = packed_offsets(n, n)
    a = normal(total, seed, stream=2)
    piv_off, piv_total = packed_offsets(n, np.ones_like(n))
    b_off, b_total = packed_offsets(n, np.full_like(n, nrhs))
    b = normal(b_total, seed, stream=3)
    return dict(n=n, a_off=a_off, a=a, piv_off=piv_off, piv_total=piv_total, b_off=b_off, b=b,
                nrhs=nrhs)


def spd_batch(count, n=32, nrhs=1, seed=0):
    """Cholesky + solve workload: A = B B^T + n I with B ~ N(0,1), right-hand sides ~ N(0,1)."""
    ns = np.full(count, n, np.int32)
    bmat = normal(count * n * n, seed, stream=4).reshape(count, n, n)
    a = np.matmul(bmat, np.transpose(bmat, (0, 2, 1)))
    a += n * np.eye(n)[None, :, :]
    a = np.ascontiguousarray(np.transpose(a, (0, 2, 1))).reshape(-1)   # column-major per matrix
    a_off, _ = packed_offsets(ns, ns)
    b_off, b_total = packed_offsets(ns, np.full_like(ns, nrhs))
    b = normal(b_total, seed, stream=5)
    return dict(n=ns, a_off=a_off, a=a, b_off=b_off, b=b, nrhs=nrhs)


def spd_batch_uneven(count, nmin=8, nmax=128, nrhs=1, seed=0):
    """Cholesky + solve workload of uneven orders: n ~ U{nmin..nmax}, A = S + 2n I with S
    symmetric, S_ij = S_ji ~ N(0,1) (the upper triangle of n^2 draws per matrix, mirrored), so
    every A is positive definite (the spectrum of S lies within about +-2 sqrt(n)); right-hand
    sides ~ N(0,1).  O(n^2) per matrix, unlike B B^T, so a 100,000-matrix batch builds in
    seconds."""
    ns = (np.floor(uniform(count, seed, stream=6) * (nmax - nmin + 1)) + nmin).astype(np.int32)
    a_off, total = packed_offsets(ns, ns)
    a = normal(total, seed, stream=7)
    for n in np.unique(ns).tolist():
        idx = np.nonzero(ns == n)[0]
        lower = np.tril_indices(n, -1)
        src = lower[1] * n + lower[0]           # (j, i) with i > j: the upper triangle, row-major
        dst = lower[0] * n + lower[1]           # (i, j): mirrored below the diagonal
        diag = np.arange(n) * (n + 1)
        for i in idx.tolist():
            m = a[a_off[i]:a_off[i] + n * n]
            m[dst] = m[src]
            m[diag] += 2.0 * n
    b_off, b_total = packed_offsets(ns, np.full_like(ns, nrhs))
    b = normal(b_total, seed, stream=8)
    return dict(n=ns, a_off=a_off, a=a, b_off=b_off, b=b, nrhs=nrhs)


def gevd_batch(count, n=64, seed=0, dtype="f64"):
    """GEVD front-half workload: A symmetric (A = S + S^T, S ~ N(0,1)) and B = M M^T + n I with
    M ~ N(0,1), column-major pairs of order n.  dtype "f32": the same pairs rounded to float;
    "c128": Hermitian pairs, A + i (T - T^T) and B + 0.05 i (K - K^T) with T, K ~ N(0,1) (B stays
    positive definite: the skew part's norm is far below n)."""
    ns = np.full(count, n, np.int32)
    tr = lambda x: np.transpose(x, (0, 2, 1))
    s = normal(count * n * n, seed, stream=8).reshape(count, n, n)
    a = s + tr(s)
    m = normal(count * n * n, seed, stream=9).reshape(count, n, n)
    b = np.matmul(m, tr(m))
    b += n * np.eye(n)[None, :, :]
    if dtype == "c128":
        t = normal(count * n * n, seed, stream=10).reshape(count, n, n)
        k = normal(count * n * n, seed, stream=11).reshape(count, n, n)
        # Column-major storage of a Hermitian X is the row-major storage of X^T = conj(X).
        a = np.conj(a + 1j * (t - tr(t)))
        b = np.conj(b + 0.05j * (k - tr(k)))
    a = np.ascontiguousarray(a).reshape(-1)
    b = np.ascontiguousarray(b).reshape(-1)          # symmetric: row- and column-major agree
    if dtype == "f32":
        a, b = a.astype(np.float32), b.astype(np.float32)
    off, _ = packed_offsets(ns, ns)
    return dict(n=ns, a_off=off, a=a, b_off=off, b=b, nrhs=0)


def qr_batch(count, mmin=64, mmax=512, nmin=16, nmax=64, nrhs=1, seed=0):
    """QR least-squares workload: m ~ U{mmin..mmax}, n ~ U{nmin..nmax} (n <= m), N(0,1) data."""
    m = (np.floor(uniform(count, seed, stream=6) * (mmax - mmin + 1)) + mmin).astype(np.int32)
    n = (np.floor(uniform(count, seed, stream=7) * (nmax - nmin + 1)) + nmin).astype(np.int32)
    n = np.minimum(n, m)
    a_off, total = packed_offsets(m, n)
    a = normal(total, seed, stream=8)
    rdiag_off, rd_total = packed_offsets(n, np.ones_like(n))
    b_off, b_total = packed_offsets(m, np.full_like(m, nrhs))
    b = normal(b_total, seed, stream=9)
    return dict(m=m, n=n, a_off=a_off, a=a, rdiag_off=rdiag_off, rdiag_total=rd_total,
                b_off=b_off, b=b, nrhs=nrhs)


def rbf_batch(count, n=128, length=0.3, jitter=1e-6, seed=0):
    """Differentiable-Cholesky workload: K_ij = exp(-|x_i - x_j|^2 / (2 length^2)) + jitter
    delta_ij with x_i ~ U[0,1]^3, and y ~ N(0,1); column-major K per matrix, lda = n."""
    ns = np.full(count, n, np.int32)
    x = uniform(count * n * 3, seed, stream=10).reshape(count, n, 3)
    d2 = ((x[:, :, None, :] - x[:, None, :, :]) ** 2).sum(-1)
    k = np.exp(-d2 / (2.0 * length * length))
    k += jitter * np.eye(n)[None, :, :]
    a = np.ascontiguousarray(np.transpose(k, (0, 2, 1))).reshape(-1)
    a_off, _ = packed_offsets(ns, ns)
    b_off, b_total = packed_offsets(ns, np.ones_like(ns))
    y = normal(b_total, seed, stream=11)
    return dict(n=ns, a_off=a_off, a=a, b_off=b_off, b=y, nrhs=1)


def conditioned_batch(count, n, cond, seed=0):
    """Mixed-precision workload (host, numpy): A = U diag(sigma) V^T with U, V the Q factors of
    N(0,1) matrices and sigma log-spaced from 1 down to 1/cond; x_true ~ N(0,1); b = A x_true.
    Returns column-major A (count*n*n), b, x_true."""
    g = normal(count * n * n * 2 + count * n, seed, stream=12)
    a = np.empty((count, n, n))
    xt = g[2 * count * n * n:].reshape(count, n)
    sigma = np.logspace(0.0, -np.log10(cond), n)
    for i in range(count):
        u = np.linalg.qr(g[(2 * i) * n * n:(2 * i + 1) * n * n].reshape(n, n))[0]
        v = np.linalg.qr(g[(2 * i + 1) * n * n:(2 * i + 2) * n * n].reshape(n, n))[0]
        a[i] = (u * sigma) @ v.T
    b = np.einsum("kij,kj->ki", a, xt)
    return np.ascontiguousarray(np.transpose(a, (0, 2, 1))).reshape(-1), b.reshape(-1), xt


def conditioned_batch_device(count, n, cond, seed=0):
    """The same distribution generated on the GPU with torch (for the large benchmark batch):
    returns device tensors a (count*n*n, column-major per matrix), b, x_true."""
    import torch
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    sigma = torch.logspace(0.0, -float(np.log10(cond)), n, dtype=torch.float64, device="cuda")
    a = torch.empty((count, n, n), dtype=torch.float64, device="cuda")
    chunk = 256
    for s in range(0, count, chunk):
        c = min(chunk, count - s)
        u = torch.linalg.qr(torch.randn((c, n, n), dtype=torch.float64, device="cuda",
                                        generator=gen))[0]
        v = torch.linalg.qr(torch.randn((c, n, n), dtype=torch.float64, device="cuda",
                                        generator=gen))[0]
        a[s:s + c] = (u * sigma) @ v.transpose(1, 2)
    xt = torch.randn((count, n), dtype=torch.float64, device="cuda", generator=gen)
    b = torch.bmm(a, xt.unsqueeze(2)).squeeze(2)
    return a.transpose(1, 2).contiguous().reshape(-1), b.reshape(-1).contiguous(), xt

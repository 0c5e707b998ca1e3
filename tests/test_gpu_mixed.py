"""Mixed-precision LU solve with FP64 refinement: every system reaches the 1e-12 normwise
backward error (refined, or through the exact FP64 fallback) and the forward error is what the
conditioning allows.

The TF32 and BF16 factorizations run their trailing updates on the hand-written tensor-core
kernel (tcgen05.mma fed by TMA); a wrong update would leave the refinement without a usable
factor and every system in the FP64 fallback, so the well-conditioned cases also assert that
refinement converged on its own (info == 0) within a small number of sweeps."""
import numpy as np
import pytest

from workloads import synth

pytestmark = pytest.mark.gpu


def _berr(A, x, b):
    return np.max(np.abs(b - A @ x)) / (np.max(np.sum(np.abs(A), 1)) * np.max(np.abs(x)) +
                                        np.max(np.abs(b)))


def _solve(mf, a, b, count, n, lowp, max_iter):
    import torch
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    dx = torch.zeros_like(db)
    berr = torch.zeros(count, dtype=torch.float64, device="cuda")
    iters = torch.zeros(count, dtype=torch.int32, device="cuda")
    info = torch.zeros(count, dtype=torch.int32, device="cuda")
    solver = mf.MixedSolveBatch(count, n)
    solver.run(da, db, dx, berr, iters, info, lowp=lowp, max_iter=max_iter, tol=1e-12)
    return (dx.cpu().numpy().reshape(count, n), berr.cpu().numpy(), iters.cpu().numpy(),
            info.cpu().numpy())


@pytest.mark.parametrize("lowp", ["fp32", "tf32", "bf16", "tf32x3"])
@pytest.mark.parametrize("cond", [1e2, 1e5, 1e8])
@pytest.mark.parametrize("n,count", [(96, 6), (512, 4)])
def test_mixed_solve(mf, lowp, cond, n, count):
    a, b, xt = synth.conditioned_batch(count, n, cond, seed=int(np.log10(cond)) + n)
    x, gb, it, gi = _solve(mf, a, b, count, n, lowp, 20)
    for i in range(count):
        A = a[i * n * n:(i + 1) * n * n].reshape(n, n).T
        bi = b[i * n:(i + 1) * n]
        be = _berr(A, x[i], bi)
        assert be <= 1e-12, (i, be, gi[i])
        assert abs(be - gb[i]) <= 1e-13
        fe = np.max(np.abs(x[i] - xt[i])) / np.max(np.abs(xt[i]))
        assert fe <= 1e-14 * cond * n, (i, fe)
    if cond <= 1e2 and lowp != "bf16":
        # refinement converges from the FP32 and TF32 factors
        assert (gi == 0).all(), (gi, it)
        assert it.max() <= 8, it
    if cond <= 1e5 and lowp in ("fp32", "tf32x3"):
        # FP32-level factors (FP32 cores, or split TF32 on the tensor cores) at cond 1e5
        assert (gi == 0).all(), (gi, it)
    if cond <= 1e2 and lowp == "bf16":
        assert (gi == 0).any(), (gi, it)   # the BF16 tensor-core factor is usable
    if cond >= 1e8 and lowp != "fp32":
        assert (gi == 1).any()          # too ill-conditioned for TF32/BF16: FP64 fallback


def test_mixed_solve_n1024(mf):
    count, n, cond = 2, 1024, 1e5
    a, b, xt = synth.conditioned_batch(count, n, cond, seed=11)
    for lowp in ("tf32", "bf16", "tf32x3"):
        x, gb, it, gi = _solve(mf, a, b, count, n, lowp, 20)
        for i in range(count):
            A = a[i * n * n:(i + 1) * n * n].reshape(n, n).T
            assert _berr(A, x[i], b[i * n:(i + 1) * n]) <= 1e-12, (lowp, i, gi[i])


def test_mixed_rejects_bad_order(mf):
    with pytest.raises(RuntimeError):
        mf.MixedSolveBatch(4, 100)

"""Mixed-precision LU solve with FP64 refinement: every system reaches the 1e-12 normwise
backward error (refined, or through the exact FP64 fallback) and the forward error is what the
conditioning allows."""
import numpy as np
import pytest

from workloads import synth

pytestmark = pytest.mark.gpu


def _berr(A, x, b):
    return np.max(np.abs(b - A @ x)) / (np.max(np.sum(np.abs(A), 1)) * np.max(np.abs(x)) +
                                        np.max(np.abs(b)))


@pytest.mark.parametrize("lowp", ["fp32", "tf32", "bf16"])
@pytest.mark.parametrize("cond", [1e2, 1e5, 1e8])
def test_mixed_solve(mf, lowp, cond):
    import torch
    count, n = 6, 96
    a, b, xt = synth.conditioned_batch(count, n, cond, seed=int(np.log10(cond)))
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    dx = torch.zeros_like(db)
    berr = torch.zeros(count, dtype=torch.float64, device="cuda")
    iters = torch.zeros(count, dtype=torch.int32, device="cuda")
    info = torch.zeros(count, dtype=torch.int32, device="cuda")
    solver = mf.MixedSolveBatch(count, n)
    solver.run(da, db, dx, berr, iters, info, lowp=lowp, max_iter=20, tol=1e-12)
    x = dx.cpu().numpy().reshape(count, n)
    gb = berr.cpu().numpy()
    gi = info.cpu().numpy()
    for i in range(count):
        A = a[i * n * n:(i + 1) * n * n].reshape(n, n).T
        bi = b[i * n:(i + 1) * n]
        be = _berr(A, x[i], bi)
        assert be <= 1e-12, (i, be, gi[i])
        assert abs(be - gb[i]) <= 1e-13
        fe = np.max(np.abs(x[i] - xt[i])) / np.max(np.abs(xt[i]))
        assert fe <= 1e-14 * cond * n, (i, fe)
    if cond <= 1e2 and lowp != "bf16":
        assert (gi == 0).all()          # refinement converges from the FP32 and TF32 factors
    if cond >= 1e8 and lowp != "fp32":
        assert (gi == 1).any()          # too ill-conditioned for TF32/BF16: FP64 fallback


def test_mixed_rejects_bad_order(mf):
    with pytest.raises(RuntimeError):
        mf.MixedSolveBatch(4, 100)

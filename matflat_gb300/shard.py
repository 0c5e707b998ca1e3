"""Splitting a batch across GPUs (one process per GPU).

Every matrix of a batch is an independent unit and no data is exchanged between them, so a
multi-GPU run needs no collective on the data path: each rank factors its own slice and only the
timing (max over ranks) and, if wanted, small per-matrix results cross processes.
"""
import numpy as np


def shard_bounds(work, world):
    """Contiguous slices [start, stop) of a batch whose per-matrix work is `work`, one per rank,
    balanced by cumulative work (the slice boundaries fall where the running sum crosses
    r/world of the total)."""
    work = np.asarray(work, dtype=np.float64)
    if world < 1:
        raise ValueError("world must be >= 1")
    if len(work) == 0:
        return [(0, 0)] * world
    c = np.cumsum(work)
    total = c[-1]
    cuts = [0]
    for r in range(1, world):
        cuts.append(int(np.searchsorted(c, total * r / world, side="left")) + 1)
    cuts.append(len(work))
    cuts = np.maximum.accumulate(np.minimum(cuts, len(work)))
    return [(int(cuts[r]), int(cuts[r + 1])) for r in range(world)]


def lu_work(n):
    """Relative work of LU on matrices of order n (2n^3/3)."""
    n = np.asarray(n, dtype=np.float64)
    return 2.0 * n ** 3 / 3.0

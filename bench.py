"""Benchmark: batched FP64 LU with partial pivoting + solve (MatFlat arithmetic) on GB300.

Default workload (the reference's batched LU configuration): 100,000 matrices with n uniform in
[8, 128], entries N(0,1), lda = n, 4 right-hand sides per matrix, seed 0, all sizes in one
persistent launch.  A step is one pass of Factorization.Lu + the forward/back solve over the
whole batch.  Other configurations (--config chol|qr|qr32) are secondary measurements.

Output: one JSON line (rank 0).  `value` = matrices/s with inputs resident in HBM (each step
restores the input batch with a device-to-device copy, inside the timed region); `e2e` = the same
through the C ABI from pinned host buffers, copies included; `roofline` for the dominant kernel
against the FP64 peak measured in this run (cuBLAS DGEMM); `cpu_baseline` = the MatFlat
restatement (oracle/) on all host cores over a bounded sample.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config lu]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    "lu": dict(workload="batched FP64 LU (partial pivoting, MatFlat order) + 4-RHS solve, "
                        "100,000 matrices, n~U{8..128}, A~N(0,1), lda=n, seed 0",
               count=100_000, nmin=8, nmax=128, nrhs=4),
    "inv": dict(workload="batched FP64 LuInverse (MatFlat order) of the LU factors of 100,000 "
                         "matrices, n~U{8..128}, A~N(0,1), lda=n, seed 0 (factored once on the "
                         "GPU before timing)",
                count=100_000, nmin=8, nmax=128, nrhs=0),
    "gevd": dict(workload="batched front half of the generalized symmetric eigenproblem "
                          "(Factorization.Gevd up to its eigen-solver): B = L L^T, C = L^-1 A L^-T, "
                          "10,000 pairs n=64, A = S + S^T, B = M M^T + 64 I, S, M ~ N(0,1), seed 0",
                 count=10_000, n=64),
    "gevd32": dict(workload="batched GEVD front half, MatFlat's float overload (float storage, "
                            "double dots): the gevd pairs (10,000, n=64, seed 0) rounded to float",
                   count=10_000, n=64, dtype="f32"),
    "gevdz": dict(workload="batched GEVD front half, MatFlat's Complex overload: B = L L^H, "
                           "C = L^-1 A L^-H, 10,000 pairs n=64, A = S + S^T + i (T - T^T), "
                           "B = M M^T + 64 I + 0.05 i (K - K^T), S, T, M, K ~ N(0,1), seed 0",
                  count=10_000, n=64, dtype="c128"),
    "chol": dict(workload="batched FP64 Cholesky (MatFlat order) + L and L^T solves, "
                          "10,000 SPD matrices n=32, A=B*B^T+32*I, B~N(0,1), 1 RHS, seed 0",
                 count=10_000, n=32, nrhs=1),
    "chol100k": dict(workload="batched FP64 Cholesky (MatFlat order) + L and L^T solves, "
                              "100,000 SPD matrices n~U{8..128}, A=S+2n*I, S symmetric with "
                              "N(0,1) entries, 1 RHS, seed 0",
                     count=100_000, nmin=8, nmax=128, nrhs=1),
    "grad": dict(workload="differentiable Cholesky/log-det/solve: loss y^T K^-1 y + log det K and "
                          "its gradient K^-1 - alpha alpha^T, 4,096 RBF kernel matrices n=128 "
                          "(x~U[0,1]^3, length 0.3, jitter 1e-6), y~N(0,1), seed 0",
                 count=4096, n=128),
    "bwd": dict(workload="reverse mode of Cholesky / log det / solve with random cotangents "
                         "(Lbar lower N(0,1), logdet_bar 1, xbar N(0,1)), factor recomputed in "
                         "MatFlat order, 4,096 RBF kernel matrices n=128 (x~U[0,1]^3, length 0.3, "
                         "jitter 1e-6), seed 0",
                count=4096, n=128),
    "mixed": dict(workload="mixed-precision LU solve + FP64 iterative refinement to 1e-12 "
                           "normwise backward error, 2,048 systems n=512, A=U diag(sigma) V^T "
                           "(U, V Q factors of N(0,1)), sigma log-spaced to cond, x_true~N(0,1), "
                           "b=A x_true",
                  count=2048, n=512),
    "qr": dict(workload="batched FP64 Householder QR (MatFlat order) + least squares, 50,000 "
                        "matrices m~U{64..512}, n~U{16..64}, N(0,1), 1 RHS, seed 0",
               count=50_000, dtype="f64"),
    "qr32": dict(workload="batched FP32 Householder QR (MatFlat float overload) + least squares,"
                          " 50,000 matrices m~U{64..512}, n~U{16..64}, N(0,1), 1 RHS, seed 0",
                 count=50_000, dtype="f32"),
}


def lu_lanes(table, n):
    """Lanes per matrix of the LU's size bucket for order n under a lanes table (the library's
    lu_lanes, csrc/runtime.cu), to count the per-bucket launches of a step."""
    if n > 128 or table <= 0:
        return 32
    if table == 1:
        return 16
    if table == 2:
        return 8 if n <= 48 else 16
    if table == 3:
        return 8
    if table == 4:
        return 8 if n <= 32 else 16 if n <= 96 else 32
    if table == 5:
        return 8 if n <= 24 else 16 if n <= 64 else 32
    if table == 6:
        return 16 if n <= 48 else 32
    return 32


def chol_lanes(table, n):
    """Lanes per matrix of the Cholesky's size bucket (the library's chol_lanes)."""
    if table == 1:
        return 4 if n <= 16 else 8 if n <= 32 else 16 if n <= 64 else 32
    if table == 2:
        return 8 if n <= 32 else 16 if n <= 64 else 32
    return 32


def lu_flops(n, nrhs):
    """Algorithmic flops of LU (2n^3/3 - n^2/2 - n/6) plus nrhs two-triangle solves (2n^2)."""
    n = n.astype(np.float64)
    return float(np.sum(2 * n ** 3 / 3 - n ** 2 / 2 - n / 6 + 2 * n ** 2 * nrhs))


def lu_bytes(n, nrhs):
    """Minimum HBM traffic: read and write A (16 n^2), b (16 n nrhs) and write piv (4 n)."""
    n = n.astype(np.float64)
    return float(np.sum(16 * n ** 2 + 16 * n * nrhs + 4 * n))


def inv_flops(n):
    """Algorithmic flops of the inverse from LU factors (LAPACK's getri count 4n^3/3 - n^2 +
    5n/3; MatFlat's own sequence issues 2n^3, the GPU kernel about 4n^3/3)."""
    n = n.astype(np.float64)
    return float(np.sum(4 * n ** 3 / 3 - n ** 2 + 5 * n / 3))


def inv_bytes(n):
    """Read the factors and pivots, write the inverse."""
    n = n.astype(np.float64)
    return float(np.sum(16 * n ** 2 + 4 * n))


def gevd_flops(n, cplx=False):
    """Cholesky of B (n^3/3) plus two passes of n triangular solves (n^3 each); a Complex
    multiply-add is four real ones."""
    n = n.astype(np.float64)
    return float(np.sum(n ** 3 / 3 + 2 * n ** 3)) * (4 if cplx else 1)


def gevd_bytes(n, es=8):
    """Read A and B, write L and C (es bytes per element)."""
    n = n.astype(np.float64)
    return float(np.sum(4 * es * n ** 2))


def chol_flops(n, nrhs):
    n = n.astype(np.float64)
    return float(np.sum(n ** 3 / 3 + n ** 2 / 2 + n / 6 + 2 * n ** 2 * nrhs))


def chol_bytes(n, nrhs):
    n = n.astype(np.float64)
    return float(np.sum(16 * n ** 2 + 16 * n * nrhs))


def grad_flops(n):
    """Cholesky forward (n^3/3) plus the adjoint (2n^3/3): n^3 per matrix."""
    n = n.astype(np.float64)
    return float(np.sum(n ** 3))


def bwd_flops(n):
    """Recomputed factor (n^3/3), X = L^T Lbar below the diagonal (n^3/3), S L^-1 (n^3) and the
    lower triangle of L^-T Y (n^3/3): 2n^3 per matrix."""
    n = n.astype(np.float64)
    return float(np.sum(2.0 * n ** 3))


def bwd_bytes(n):
    """Read A, Lbar, x, xbar, logdet_bar; write L, abar, bbar."""
    n = n.astype(np.float64)
    return float(np.sum(32 * n ** 2 + 24 * n + 8))


def grad_bytes(n):
    """Read K and y, write L, the gradient, alpha and the loss."""
    n = n.astype(np.float64)
    return float(np.sum(24 * n ** 2 + 16 * n + 8))


def qr_flops(m, n, nrhs):
    m = m.astype(np.float64)
    n = n.astype(np.float64)
    return float(np.sum(2 * m * n ** 2 - 2 * n ** 3 / 3 + nrhs * (4 * m * n - n ** 2)))


def qr_bytes(m, n, nrhs, es):
    m = m.astype(np.float64)
    n = n.astype(np.float64)
    return float(np.sum(es * (2 * m * n + n + 2 * m * nrhs)))


class ClockSampler:
    """nvidia-smi clock and throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=5)

    def summary(self):
        if not self.samples:
            # Timed region shorter than one sampling period: one reading right after it.
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index),
                                      "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"],
                                     capture_output=True, text=True, timeout=20).stdout
                self.samples = [[x.strip() for x in out.strip().split(",")]]
            except (OSError, subprocess.SubprocessError):
                return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = []
        mx = None
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[1]))
                mx = float(s[2])
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, s[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def measure_fp64_peak(torch):
    """FP64 peak of this GPU measured live: cuBLAS DGEMM 4096^3 (torch.matmul), best of 5."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    del a, b
    torch.cuda.empty_cache()
    return 2.0 * n ** 3 / best / 1e12


def read_traffic(kernel_key):
    """Per-launch DRAM bytes of a kernel from the committed ncu summary (profiles/), or None."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        line = line.strip()
        if line.startswith(kernel_key + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def make_inputs(cfg_name, rank):
    from workloads import synth
    cfg = CONFIGS[cfg_name]
    if cfg_name in ("lu", "inv"):
        return synth.lu_batch(cfg["count"], cfg["nmin"], cfg["nmax"], cfg["nrhs"], seed=rank)
    if cfg_name == "chol":
        return synth.spd_batch(cfg["count"], cfg["n"], cfg["nrhs"], seed=rank)
    if cfg_name == "chol100k":
        return synth.spd_batch_uneven(cfg["count"], cfg["nmin"], cfg["nmax"], cfg["nrhs"],
                                      seed=rank)
    if cfg_name in ("grad", "bwd"):
        return synth.rbf_batch(cfg["count"], cfg["n"], seed=rank)
    if cfg_name.startswith("gevd"):
        return synth.gevd_batch(cfg["count"], cfg["n"], seed=rank, dtype=cfg.get("dtype", "f64"))
    return synth.qr_batch(cfg["count"], seed=rank)


def cpu_sample_rate(cfg_name, d, budget_s=15.0, threads=None):
    """Matrices/s of the MatFlat restatement (oracle/) on the host cores over a bounded,
    evenly strided sample of the same batch; a batch that takes less than a quarter of the
    budget is repeated until it does."""
    from oracle import oracle
    threads = threads or os.cpu_count() or 1
    count = len(d["n"])
    # Probe with a small strided sample, then size the sample to the time budget.
    stride = max(1, count // 512)
    sample = np.arange(0, count, stride)
    for _ in range(4):
        t = run_cpu_sample(cfg_name, d, sample, threads, oracle)
        if t >= budget_s / 4 or len(sample) >= count:
            break
        grow = min(count, int(len(sample) * min(8.0, budget_s / 4 / max(t, 1e-3))))
        stride = max(1, count // grow)
        sample = np.arange(0, count, stride)
    done, total_t = len(sample), t
    while total_t < budget_s / 4:
        total_t += run_cpu_sample(cfg_name, d, sample, threads, oracle)
        done += len(sample)
    return done / total_t, done, threads, total_t


def run_cpu_sample(cfg_name, d, sample, threads, oracle):
    if cfg_name.startswith("gevd"):
        n = d["n"][sample].astype(np.int32)
        sz = n.astype(np.int64) ** 2
        off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
        a = np.concatenate([d["a"][d["a_off"][i]:d["a_off"][i] + sz[j]] for j, i in enumerate(sample)])
        b = np.concatenate([d["b"][d["b_off"][i]:d["b_off"][i] + sz[j]] for j, i in enumerate(sample)])
        c = np.zeros_like(a)
        info = np.zeros(len(n), np.int32)
        t0 = time.perf_counter()
        oracle.gevd_front_batched(n, off, a, off, b, c, info, threads)
        return time.perf_counter() - t0
    if cfg_name == "inv":
        n = d["n"][sample].astype(np.int32)
        sz = n.astype(np.int64) ** 2
        a_off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
        piv_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]]).astype(np.int64)
        src = d.get("a_fac", d["a"])
        a = np.concatenate([src[d["a_off"][i]:d["a_off"][i] + sz[j]]
                            for j, i in enumerate(sample)])
        info = np.zeros(len(n), np.int32)
        if "piv" in d:
            piv = np.concatenate([d["piv"][d["piv_off"][i]:d["piv_off"][i] + n[j]]
                                  for j, i in enumerate(sample)])
        else:   # no GPU factors (reference arm): factor the sample first, untimed
            piv = np.zeros(int(n.sum()), np.int32)
            sign = np.zeros(len(n), np.int32)
            oracle.lu_solve_batched(n, a_off, a, piv_off, piv, a_off, a, 0, sign, threads)
        t0 = time.perf_counter()
        oracle.lu_inverse_batched(n, a_off, a, piv_off, piv, info, threads)
        return time.perf_counter() - t0
    if cfg_name in ("lu", "chol", "chol100k", "grad"):
        n = d["n"][sample].astype(np.int32)
        sz = n.astype(np.int64) ** 2
        a_off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
        a = np.concatenate([d["a"][d["a_off"][i]:d["a_off"][i] + sz[j]]
                            for j, i in enumerate(sample)])
        nrhs = d["nrhs"]
        bsz = n.astype(np.int64) * nrhs
        b_off = np.concatenate([[0], np.cumsum(bsz)[:-1]]).astype(np.int64)
        b = np.concatenate([d["b"][d["b_off"][i]:d["b_off"][i] + bsz[j]]
                            for j, i in enumerate(sample)])
        t0 = time.perf_counter()
        if cfg_name == "lu":
            piv_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]]).astype(np.int64)
            piv = np.zeros(int(n.sum()), np.int32)
            sign = np.zeros(len(n), np.int32)
            oracle.lu_solve_batched(n, a_off, a, piv_off, piv, b_off, b, nrhs, sign, threads)
        elif cfg_name in ("chol", "chol100k"):
            info = np.zeros(len(n), np.int32)
            oracle.chol_solve_batched(n, a_off, a, b_off, b, info, threads)
        else:
            info = np.zeros(len(n), np.int32)
            loss = np.zeros(len(n))
            g = np.zeros_like(a)
            t0 = time.perf_counter()
            oracle.chol_grad_batched(n, a_off, a, b_off, b, loss, g, info, threads)
        return time.perf_counter() - t0
    m = d["m"][sample].astype(np.int32)
    n = d["n"][sample].astype(np.int32)
    sz = m.astype(np.int64) * n
    a_off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    dt = np.float32 if cfg_name == "qr32" else np.float64
    a = np.concatenate([d["a"][d["a_off"][i]:d["a_off"][i] + sz[j]]
                        for j, i in enumerate(sample)]).astype(dt)
    b_off = np.concatenate([[0], np.cumsum(m.astype(np.int64))[:-1]]).astype(np.int64)
    b = np.concatenate([d["b"][d["b_off"][i]:d["b_off"][i] + m[j]]
                        for j, i in enumerate(sample)]).astype(dt)
    x_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]]).astype(np.int64)
    x = np.zeros(int(n.sum()), dt)
    t0 = time.perf_counter()
    oracle.qr_ls_batched(m, n, a_off, a, b_off, b, x_off, x, threads)
    return time.perf_counter() - t0


def run_reference(args, cfg_name):
    """--impl reference: the MatFlat restatement on all host cores (the reference is C# and
    cannot run on this machine; the restatement reproduces its arithmetic)."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    d = make_inputs(cfg_name, 0)
    for _ in range(args.warmup):
        cpu_sample_rate(cfg_name, d, budget_s=2.0)
    rates = []
    sample_n = threads = 0
    t_all = 0.0
    for _ in range(args.steps):
        r, sample_n, threads, t = cpu_sample_rate(cfg_name, d, budget_s=args.ref_budget)
        rates.append(r)
        t_all += t
    value = statistics.median(rates)
    cfg = CONFIGS[cfg_name]
    line = {
        "impl": "reference", "metric": metric_name(cfg_name), "value": value,
        "unit": "matrices/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t_all / max(1, args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": dtype_name(cfg_name),
        "data": "synthetic (seeded SplitMix64 + Box-Muller)",
        "config": {"workload": cfg["workload"], "count": cfg["count"]},
        "cpu_baseline": {"value": value, "unit": "matrices/s", "cores": threads, "kind": "port",
                         "sample": "%d matrices evenly strided over the batch per step" % sample_n},
        "e2e": {"value": value, "unit": "matrices/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def metric_name(cfg_name):
    return {"mixed": "mixed-precision LU+IR solves/s at 1e-12 backward error","lu": "batched FP64 LU+solve matrices/s (MatFlat-exact pivots)",
            "inv": "batched FP64 LuInverse matrices/s (MatFlat-exact)",
            "gevd": "batched FP64 GEVD front half (Cholesky + C = L^-1 A L^-T) pairs/s (MatFlat-exact)",
            "gevd32": "batched FP32 GEVD front half (Cholesky + C = L^-1 A L^-T) pairs/s (MatFlat-exact)",
            "gevdz": "batched Complex GEVD front half (Cholesky + C = L^-1 A L^-H) pairs/s (MatFlat-exact)",
            "chol": "batched FP64 Cholesky+solve matrices/s (MatFlat-exact)",
            "chol100k": "batched FP64 Cholesky+solve matrices/s (MatFlat-exact)",
            "grad": "batched FP64 Cholesky/log-det/solve loss+gradient matrices/s",
            "bwd": "batched FP64 Cholesky/log-det/solve reverse mode (VJP) matrices/s",
            "qr": "batched FP64 QR least-squares matrices/s (MatFlat-exact factors)",
            "qr32": "batched FP32 QR least-squares matrices/s (MatFlat-exact factors)"}[cfg_name]


def dtype_name(cfg_name):
    return {"qr32": "f32", "gevd32": "f32", "gevdz": "complex128"}.get(cfg_name, "f64")


def measure_mixed(torch, mf, stream, count, n, cond, lowp, steps, warmup, seed, local,
                  with_e2e=True, cpu_sample=0):
    """Mixed-precision LU + FP64 refinement against the exact FP64 LU on the same systems.

    Returns a dict: solves/s (CUDA events on the solver's stream, L2-sized inputs so no flush is
    needed: A alone is 8 n^2 count bytes), per-system backward/forward error, the exact FP64 GPU
    rate on the same systems, optionally the end-to-end rate and a CPU-oracle sample."""
    from workloads import synth
    ctx = mf.context()
    ctx.set_stream(stream.cuda_stream)
    with torch.cuda.stream(stream):
        a, b, xt = synth.conditioned_batch_device(count, n, cond, seed=seed)
    stream.synchronize()
    x = torch.zeros_like(b)
    berr = torch.zeros(count, dtype=torch.float64, device="cuda")
    iters = torch.zeros(count, dtype=torch.int32, device="cuda")
    info = torch.zeros(count, dtype=torch.int32, device="cuda")
    solver = mf.MixedSolveBatch(count, n)

    def run():
        solver.run(a, b, x, berr, iters, info, lowp=lowp, max_iter=10, tol=1e-12, sync=False)

    with torch.cuda.stream(stream):
        for _ in range(warmup):
            run()
        stream.synchronize()
        clocks = ClockSampler(local)
        clocks.start()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(steps):
            run()
        t1.record(stream)
        stream.synchronize()
        clocks.stop()
    solver.status()
    ms = t0.elapsed_time(t1) / steps

    # End to end through the C ABI: A and b from pinned host memory, x, berr, iters and info
    # back to pinned host memory, every step.
    e2e = None
    if with_e2e:
        ins = [a, b]
        outs = [x, berr, iters, info]
        ins_h = [t.cpu().pin_memory() for t in ins]
        outs_h = [torch.empty(t.shape, dtype=t.dtype).pin_memory() for t in outs]
        with torch.cuda.stream(stream):
            for _ in range(2):
                for t, th in zip(ins, ins_h):
                    t.copy_(th, non_blocking=True)
                run()
                for t, th in zip(outs, outs_h):
                    th.copy_(t, non_blocking=True)
            stream.synchronize()
            q0 = torch.cuda.Event(enable_timing=True)
            q1 = torch.cuda.Event(enable_timing=True)
            q0.record(stream)
            for _ in range(steps):
                for t, th in zip(ins, ins_h):
                    t.copy_(th, non_blocking=True)
                run()
                for t, th in zip(outs, outs_h):
                    th.copy_(t, non_blocking=True)
            q1.record(stream)
            stream.synchronize()
        solver.status()
        e2e_ms = q0.elapsed_time(q1) / steps
        e2e = {"value": count / (e2e_ms / 1e3), "unit": "solves/s",
               "h2d_bytes_per_step": int(sum(t.numel() * t.element_size() for t in ins)),
               "d2h_bytes_per_step": int(sum(t.numel() * t.element_size() for t in outs)),
               "ms_per_step": e2e_ms}
    be = berr.cpu().numpy()
    it = iters.cpu().numpy()
    inf = info.cpu().numpy()
    xv = x.reshape(count, n)
    fe = ((xv - xt).abs().amax(1) / xt.abs().amax(1)).cpu().numpy()

    # The exact FP64 LU (MatFlat arithmetic) on the same systems: plain GPU rate.
    n_arr = np.full(count, n, np.int32)
    a_off = np.arange(count, dtype=np.int64) * n * n
    v_off = np.arange(count, dtype=np.int64) * n
    plain = mf.LuBatch(n_arr, a_off, v_off, nrhs=1, b_off=v_off)
    a2 = torch.empty_like(a)
    b2 = torch.empty_like(b)
    piv = torch.zeros(count * n, dtype=torch.int32, device="cuda")
    sign = torch.zeros(count, dtype=torch.int32, device="cuda")
    pinfo = torch.zeros(count, dtype=torch.int32, device="cuda")
    with torch.cuda.stream(stream):
        a2.copy_(a)
        b2.copy_(b)
        plain.run(a2, piv, b2, sign, pinfo)      # warm-up
        a2.copy_(a)
        b2.copy_(b)
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        plain.run(a2, piv, b2, sign, pinfo)
        p1.record(stream)
        stream.synchronize()
    plain_ms = p0.elapsed_time(p1)
    plain_x = b2.reshape(count, n)
    pfe = ((plain_x - xt).abs().amax(1) / xt.abs().amax(1)).cpu().numpy()
    exact_piv = piv.clone()
    # The same plan in the FMA form (the plain form of the metric: MatFlat's pivots, backward-
    # stable factors; orders above 128 run the blocked CTA kernel).
    plain.set_form("fma")
    with torch.cuda.stream(stream):
        a2.copy_(a)
        b2.copy_(b)
        plain.run(a2, piv, b2, sign, pinfo)      # warm-up
        a2.copy_(a)
        b2.copy_(b)
        p0.record(stream)
        plain.run(a2, piv, b2, sign, pinfo)
        p1.record(stream)
        stream.synchronize()
    fma_ms = p0.elapsed_time(p1)
    fma_fe = ((b2.reshape(count, n) - xt).abs().amax(1) / xt.abs().amax(1)).cpu().numpy()
    fma_plain = {"value": count / (fma_ms / 1e3), "unit": "solves/s", "ms": fma_ms,
                 "fwd_err_max": float(np.max(fma_fe)),
                 "pivots_identical_to_exact": bool(torch.equal(piv, exact_piv)),
                 "redone_exact": plain.form_fallbacks()}
    del exact_piv
    hist = {int(k): int(v) for k, v in zip(*np.unique(it, return_counts=True))}

    cpu = None
    if cpu_sample:
        from oracle import oracle
        ah = a.cpu().numpy()
        bh = b.cpu().numpy()
        k = max(1, min(count, cpu_sample))
        idx = np.linspace(0, count - 1, k).astype(int)
        n_s = np.full(k, n, np.int32)
        aoff = np.arange(k, dtype=np.int64) * n * n
        voff = np.arange(k, dtype=np.int64) * n
        asub = np.concatenate([ah[i * n * n:(i + 1) * n * n] for i in idx])
        bsub = np.concatenate([bh[i * n:(i + 1) * n] for i in idx])
        pv = np.zeros(k * n, np.int32)
        sg = np.zeros(k, np.int32)
        threads = os.cpu_count() or 1
        t = time.perf_counter()
        oracle.lu_solve_batched(n_s, aoff, asub, voff, pv, voff, bsub, 1, sg, threads)
        dt = time.perf_counter() - t
        cpu = {"value": k / dt, "unit": "solves/s", "cores": threads, "kind": "port",
               "sample": "%d of %d systems, MatFlat LU + solve (exact FP64), %.1f s" % (k, count, dt)}
        # error of the mixed solutions against the FP64 oracle's on that sample
        ox = bsub.reshape(k, n)
        gx = xv.cpu().numpy()[idx]
        cpu["mixed_vs_oracle_rel_err_max"] = float(np.max(np.abs(gx - ox) / np.abs(ox).max(1, keepdims=True)))
    del a, b, xt, x, a2, b2
    torch.cuda.empty_cache()
    return {
        "value": count / (ms / 1e3), "unit": "solves/s", "ms": ms, "count": count, "n": n,
        "cond": cond, "lowp": lowp, "tol": 1e-12, "max_iter": 10,
        "berr_max": float(np.nanmax(be)), "berr_median": float(np.nanmedian(be)),
        "fwd_err_max": float(np.max(fe)), "fwd_err_median": float(np.median(fe)),
        "iters_histogram": hist, "fallback_fp64": int((inf == 1).sum()),
        "singular": int((inf == 2).sum()),
        "fp64_plain": {"value": count / (plain_ms / 1e3), "unit": "solves/s", "ms": plain_ms,
                       "fwd_err_max": float(np.max(pfe))},
        "fp64_plain_fma": fma_plain,
        "speedup_vs_fp64_plain": plain_ms / ms,
        "speedup_vs_fp64_plain_fma": fma_ms / ms,
        "flops": count * (2.0 * n ** 3 / 3),
        "e2e": e2e, "cpu": cpu, "clocks": clocks.summary(),
    }


def run_mixed(args, torch, mf, world, rank, local):
    """Mixed-precision LU + FP64 refinement vs the exact FP64 LU on the same batch."""
    cfg = CONFIGS["mixed"]
    count = cfg["count"]
    n = args.n or cfg["n"]
    stream = torch.cuda.Stream()
    r = measure_mixed(torch, mf, stream, count, n, args.cond, args.lowp, args.steps, args.warmup,
                      rank, local, with_e2e=not args.no_e2e,
                      cpu_sample=64 if (rank == 0 and world == 1 and not args.no_cpu_baseline)
                      else 0)
    if rank == 0:
        line = {
            "metric": metric_name("mixed"), "value": world * r["value"], "unit": "solves/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (torch generator on the GPU, seed per rank)",
            "config": {"workload": cfg["workload"], "count": count, "n": n, "cond": args.cond,
                       "lowp": args.lowp, "max_iter": 10, "tol": 1e-12},
            "gpu_launches": 2 * (n // 32) + 12,
            "roofline": {"bound": "tensor" if args.lowp != "fp32" else "fp32",
                         "achieved": r["flops"] / (r["ms"] / 1e3) / 1e12, "unit": "TFLOP/s",
                         "note": "whole solve (factorization + refinement) against the "
                                 "factorization's 2n^3/3; the panel and refinement sweeps, not "
                                 "the tensor-core GEMMs, dominate at n=512"},
            "cpu_baseline": r["cpu"], "e2e": r["e2e"], "clocks": r["clocks"],
        }
        for k in ("berr_max", "berr_median", "fwd_err_max", "fwd_err_median", "iters_histogram",
                  "fallback_fp64", "singular", "fp64_plain", "speedup_vs_fp64_plain",
                  "fp64_plain_fma", "speedup_vs_fp64_plain_fma"):
            line[k] = r[k]
        print(json.dumps(line), flush=True)


def chol_fma_check(torch, d, a_in, a_out, b_in, b_out, info):
    """The FMA form's promise on the whole timed batch (device tensors, after timing): normwise
    backward error of the factor, ||A - L L^T||_1 / ||A||_1, and of the solution,
    ||b - A x||_1 / (||A||_1 ||x||_1 + ||b||_1), both within 1e-13 n; info equal to the oracle's
    (MatFlat's arithmetic) for every matrix; and how many factors happen to equal MatFlat's bits."""
    from oracle import oracle
    n = d["n"]
    info_h = info.cpu().numpy()
    oa = d["a"].copy()
    ob = d["b"].copy()
    oinfo = np.zeros(len(n), np.int32)
    t0 = time.perf_counter()
    oracle.chol_solve_batched(n, d["a_off"], oa, d["b_off"], ob, oinfo, os.cpu_count() or 1,
                              nrhs=d["nrhs"])
    t_or = time.perf_counter() - t0
    a_off = torch.from_numpy(d["a_off"]).cuda()
    b_off = torch.from_numpy(d["b_off"]).cuda()
    oa_d = torch.from_numpy(oa).cuda()
    worst_f = worst_x = 0.0
    same_bits = 0
    for nv in np.unique(n):
        nn = int(nv)
        idx = torch.from_numpy(np.nonzero((n == nv) & (info_h == 0))[0]).cuda()
        if idx.numel() == 0:
            continue
        ca = a_off[idx][:, None] + torch.arange(nn * nn, device="cuda")[None, :]
        A = a_in[ca].view(-1, nn, nn).transpose(1, 2)
        L = a_out[ca].view(-1, nn, nn).transpose(1, 2)
        same_bits += int((a_out[ca] == oa_d[ca]).all(1).sum().item())
        na = A.abs().sum(1).amax(1)
        ef = (A - L @ L.transpose(1, 2)).abs().sum(1).amax(1) / na
        worst_f = max(worst_f, float((ef / nn).max().item()))
        for r in range(d["nrhs"]):
            cb = b_off[idx][:, None] + r * nn + torch.arange(nn, device="cuda")[None, :]
            x = b_out[cb]
            bb = b_in[cb]
            res = (bb - (A @ x[:, :, None])[:, :, 0]).abs().sum(1)
            ex = res / (na * x.abs().sum(1) + bb.abs().sum(1))
            worst_x = max(worst_x, float((ex / nn).max().item()))
    return {"factor_berr_over_n_max": worst_f, "solve_berr_over_n_max": worst_x,
            "bound_over_n": 1e-13, "within_bound": worst_f <= 1e-13 and worst_x <= 1e-13,
            "info_identical_to_oracle": bool((info_h == oinfo).all()),
            "not_positive_definite": int((oinfo != 0).sum()),
            "factors_equal_to_matflat_bits": same_bits, "checked": int(len(n)),
            "checker": "torch FP64 batched products on the device; oracle (MatFlat Cholesky, "
                       "C++) for info, %.1f s" % t_or}


def qr_fma_check(d, a_out, rd_out, b_out, every=25):
    """The FMA-form QR's promise on a strided sample of the timed batch (host copies, after
    timing): the reflectors and R reproduce A to a normwise backward error within 1e-13 m
    (A = H_0 ... H_{n-1} [R; 0], H_k = I - v_k v_k^T / v_k[0], MatFlat's storage), and the
    least-squares solution's normal-equation residual ||A^T (A x - b)|| / (||A|| ||b||) against
    the exact form's bound used by the tests (1e-9)."""
    t0 = time.perf_counter()
    worst_f = worst_ls = 0.0
    checked = 0
    for i in range(0, len(d["m"]), every):
        mi, ni = int(d["m"][i]), int(d["n"][i])
        ao, bo, ro = int(d["a_off"][i]), int(d["b_off"][i]), int(d["rdiag_off"][i])
        A = d["a"][ao:ao + mi * ni].reshape(ni, mi).T
        F = a_out[ao:ao + mi * ni].reshape(ni, mi).T
        rd = rd_out[ro:ro + ni]
        r = np.zeros((mi, ni))
        r[:ni, :] = np.triu(F[:ni, :], 1)
        r[np.arange(ni), np.arange(ni)] = rd
        for k in range(ni - 1, -1, -1):
            v = F[k:, k]
            if rd[k] != 0 and v[0] != 0:
                r[k:, :] -= np.outer(v, v @ r[k:, :]) / v[0]
        na = np.linalg.norm(A)
        worst_f = max(worst_f, np.linalg.norm(A - r) / na / mi)
        bi = d["b"][bo:bo + mi]
        x = b_out[bo:bo + ni]
        worst_ls = max(worst_ls, np.linalg.norm(A.T @ (A @ x - bi)) / (na * np.linalg.norm(bi)))
        checked += 1
    return {"factor_berr_over_m_max": float(worst_f), "bound_over_m": 1e-13,
            "ls_normal_residual_max": float(worst_ls), "ls_bound": 1e-9,
            "within_bound": bool(worst_f <= 1e-13 and worst_ls <= 1e-9), "checked": checked,
            "sample": "every %dth matrix of the timed batch" % every,
            "checker": "numpy FP64 reconstruction from the stored reflectors, %.1f s"
                       % (time.perf_counter() - t0)}


def measure_cholesky(torch, mf, rank, steps, warmup, fp64_peak):
    """The Cholesky half of the metric on the default line: 100,000 SPD matrices n~U{8..128}
    (the chol100k configuration) + 1-RHS solve, the FMA form (backward-error checked over the
    whole batch) and MatFlat's exact form, each autotuned at plan creation, timed like the main
    step (L2 flushed, device-to-device restore of the inputs, one plan execution) with CUDA
    events on the plan's stream."""
    ctx = mf.context()
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    d = make_inputs("chol100k", rank)
    count = len(d["n"])
    a0 = torch.from_numpy(d["a"]).cuda()
    b0 = torch.from_numpy(d["b"]).cuda()
    a = torch.empty_like(a0)
    b = torch.empty_like(b0)
    info = torch.zeros(count, dtype=torch.int32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    flops = chol_flops(d["n"], d["nrhs"])
    out = {"workload": CONFIGS["chol100k"]["workload"], "count": count}
    for form in ("fma", "exact"):
        plan = mf.CholeskyBatch(d["n"], d["a_off"], nrhs=d["nrhs"], b_off=d["b_off"])
        plan.set_form(form)
        tuned = plan.autotune()
        ks, ke = [], []
        with torch.cuda.stream(stream):
            for it in range(warmup + steps):
                flush.zero_()
                a.copy_(a0)
                b.copy_(b0)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                plan.run(a, b, info)
                e1.record(stream)
                if it >= warmup:
                    ks.append(e0)
                    ke.append(e1)
            stream.synchronize()
        kms = statistics.median(s0.elapsed_time(s1) for s0, s1 in zip(ks, ke))
        tf = flops / (kms / 1e3) / 1e12
        rec = {"value": count / (kms / 1e3), "unit": "matrices/s", "kernel_ms": kms,
               "roofline": {"bound": "fp64", "achieved": tf, "peak": fp64_peak,
                            "unit": "TFLOP/s", "frac": tf / fp64_peak},
               "launch_shape": dict(zip(["warps_per_cta", "warps_per_sm", "lanes_per_matrix",
                                         "mul_mode", "dot_pairs_per_block"], tuned))}
        if form == "fma":
            rec["form"] = ("fused multiply-adds in any order, reciprocal column scaling, FMA "
                           "solves (mfg_plan_set_form); not MatFlat's bits, checked by backward "
                           "error over the whole batch")
            rec["form_check"] = chol_fma_check(torch, d, a0, a, b0, b, info)
        else:
            rec["form"] = "MatFlat's arithmetic, bit for bit"
        out[form] = rec
        del plan
    return out


def lu_parity(d, a_out, b_out, piv_out, sign_out, info_out):
    """The oracle (MatFlat's LuCore + solve restated in C++) over the WHOLE timed batch, after
    the timed region, compared with the GPU's outputs of the last timed step bit for bit."""
    from oracle import oracle
    n = d["n"]
    a = d["a"].copy()
    b = d["b"].copy()
    piv = np.zeros(d["piv_total"], np.int32)
    sign = np.zeros(len(n), np.int32)
    t = time.perf_counter()
    oracle.lu_solve_batched(n, d["a_off"], a, d["piv_off"], piv, d["b_off"], b, d["nrhs"], sign,
                            os.cpu_count() or 1)
    dt = time.perf_counter() - t
    ga = a_out.view(np.uint64)
    gb = b_out.view(np.uint64)
    bad_piv = bad_a = bad_b = 0
    a_off, piv_off, b_off = d["a_off"], d["piv_off"], d["b_off"]
    eq_a = ga == a.view(np.uint64)
    eq_b = gb == b.view(np.uint64)
    eq_p = piv_out == piv
    # per-matrix mismatch counts through the packed offsets
    ia = np.add.reduceat(~eq_a, a_off) if len(a_off) else np.zeros(0)
    ip = np.add.reduceat(~eq_p, piv_off) if len(piv_off) else np.zeros(0)
    ib = np.add.reduceat(~eq_b, b_off) if len(b_off) else np.zeros(0)
    bad_a, bad_piv, bad_b = int((ia > 0).sum()), int((ip > 0).sum()), int((ib > 0).sum())
    bad_sign = int((sign_out != sign).sum())
    return {"checked": int(len(n)), "checker": "oracle (MatFlat LuCore + solve, C++), %.1f s on "
                                              "%d threads" % (dt, os.cpu_count() or 1),
            "pivots_identical": bad_piv == 0, "factors_bit_identical": bad_a == 0,
            "x_bit_identical": bad_b == 0, "signs_identical": bad_sign == 0,
            "mismatches": {"pivots": bad_piv, "factors": bad_a, "x": bad_b, "sign": bad_sign},
            "zero_pivot_matrices": int((info_out != 0).sum())}


def lu_berr(torch, d, a_in, a_out, piv_out, b_in, b_out):
    """Normwise backward errors of a batch of LU factors and solutions on the device (torch
    FP64, one batched product per order): max over the matrices with finite factors of
    ||PA - LU||_1 / (||A||_1 n) and of ||b - Ax||_1 / ((||A||_1 ||x||_1 + ||b||_1) n), with
    MatFlat's permutation vector (row i of PA is row piv[i] of A)."""
    n = d["n"]
    a_off = torch.from_numpy(d["a_off"]).cuda()
    p_off = torch.from_numpy(d["piv_off"]).cuda()
    b_off = torch.from_numpy(d["b_off"]).cuda()
    worst_f = worst_x = 0.0
    for nv in np.unique(n):
        nn = int(nv)
        idx = torch.from_numpy(np.nonzero(n == nv)[0]).cuda()
        ca = a_off[idx][:, None] + torch.arange(nn * nn, device="cuda")[None, :]
        A = a_in[ca].view(-1, nn, nn).transpose(1, 2)
        F = a_out[ca].view(-1, nn, nn).transpose(1, 2)
        P = piv_out[p_off[idx][:, None] + torch.arange(nn, device="cuda")[None, :]].long()
        L = torch.tril(F, -1) + torch.eye(nn, dtype=F.dtype, device="cuda")
        U = torch.triu(F)
        PA = torch.gather(A, 1, P[:, :, None].expand(-1, -1, nn))
        na = A.abs().sum(1).amax(1)
        ok = torch.isfinite(F).all(2).all(1)
        ef = (PA - L @ U).abs().sum(1).amax(1) / na
        worst_f = max(worst_f, float((ef[ok] / nn).max().item()) if ok.any() else 0.0)
        for r in range(d["nrhs"]):
            cb = b_off[idx][:, None] + r * nn + torch.arange(nn, device="cuda")[None, :]
            x, bb = b_out[cb], b_in[cb]
            res = (bb - (A @ x[:, :, None])[:, :, 0]).abs().sum(1)
            ex = res / (na * x.abs().sum(1) + bb.abs().sum(1))
            worst_x = max(worst_x, float((ex[ok] / nn).max().item()) if ok.any() else 0.0)
    return worst_f, worst_x


def measure_lu_fma(torch, mf, d, rank, steps, warmup, fp64_peak, flops):
    """The LU's FMA form on the headline batch (mfg_plan_set_form): fused multiply-adds with
    MatFlat's pivots kept by a screen and an exact redo of the matrices it rejects.  Timed like the
    main step (L2 flushed, device-to-device restore, one plan execution, CUDA events on the plan's
    stream); then the pivots and signs of the last timed step against the oracle over the whole
    batch, and the backward errors of the factors and solutions."""
    ctx = mf.context()
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    count = len(d["n"])
    a0 = torch.from_numpy(d["a"]).cuda()
    b0 = torch.from_numpy(d["b"]).cuda()
    a = torch.empty_like(a0)
    b = torch.empty_like(b0)
    piv = torch.zeros(d["piv_total"], dtype=torch.int32, device="cuda")
    sign = torch.zeros(count, dtype=torch.int32, device="cuda")
    info = torch.zeros(count, dtype=torch.int32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    plan = mf.LuBatch(d["n"], d["a_off"], d["piv_off"], nrhs=d["nrhs"], b_off=d["b_off"])
    plan.set_form("fma")
    tuned = plan.autotune()
    ks, ke = [], []
    with torch.cuda.stream(stream):
        for it in range(warmup + steps):
            flush.zero_()
            a.copy_(a0)
            b.copy_(b0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            plan.run(a, piv, b, sign, info)
            e1.record(stream)
            if it >= warmup:
                ks.append(e0)
                ke.append(e1)
        stream.synchronize()
    kms = statistics.median(s0.elapsed_time(s1) for s0, s1 in zip(ks, ke))
    fallbacks = plan.form_fallbacks()
    par = lu_parity(d, a.cpu().numpy(), b.cpu().numpy(), piv.cpu().numpy(), sign.cpu().numpy(),
                    info.cpu().numpy())
    bf, bx = lu_berr(torch, d, a0, a, piv, b0, b)
    # End to end through the host-buffer entry point, as for the main line.
    a_h = torch.from_numpy(d["a"]).pin_memory()
    b_h = torch.from_numpy(d["b"]).pin_memory()
    io = [torch.empty_like(a_h).pin_memory(), torch.empty_like(b_h).pin_memory()]
    extra = [torch.zeros(d["piv_total"], dtype=torch.int32).pin_memory(),
             torch.zeros(count, dtype=torch.int32).pin_memory(),
             torch.zeros(count, dtype=torch.int32).pin_memory()]
    times = []
    for it in range(2 + steps):
        io[0].copy_(a_h)
        io[1].copy_(b_h)
        t0 = time.perf_counter()
        plan.run_host(io[0], extra[0], io[1], extra[1], extra[2])
        t1 = time.perf_counter()
        if it >= 2:
            times.append(t1 - t0)
    e2e_ms = 1e3 * sum(times) / len(times)
    nb = lambda ts: int(sum(t.numel() * t.element_size() for t in ts))
    tf = flops / (kms / 1e3) / 1e12
    return {"value": count / (kms / 1e3), "unit": "matrices/s", "kernel_ms": kms,
            "roofline": {"bound": "fp64", "achieved": tf, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": tf / fp64_peak, "kernel": "getrf_task_fma_kernel",
                         "traffic": read_traffic("getrf_task_fma_kernel")},
            "launch_shape": dict(zip(["warps_per_cta", "warps_per_sm", "lanes_table",
                                      "mul_mode", "dot_pairs_per_block"], tuned)),
            "form": "fused multiply-add dots, reciprocal column scaling, MatFlat's pivot rule "
                    "with a screen (runner-up within ~1.5e-8 of the pivot, ties, zero or "
                    "non-finite candidates) that redoes rejected matrices in MatFlat's arithmetic; "
                    "not MatFlat's bits",
            "fallbacks": fallbacks,
            "e2e": {"value": count / (e2e_ms / 1e3), "unit": "matrices/s", "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": nb(io), "d2h_bytes_per_step": nb(io + extra),
                    "path": "host-buffer entry point on page-locked host arrays, host wall clock"},
            "pivots_identical_to_oracle": par["pivots_identical"],
            "signs_identical_to_oracle": par["signs_identical"],
            "pivot_mismatches": par["mismatches"]["pivots"],
            "factor_berr_over_n_max": bf, "solve_berr_over_n_max": bx, "bound_over_n": 1e-13,
            "within_bound": bf <= 1e-13 and bx <= 1e-13,
            "checker": par["checker"] + "; torch FP64 batched products for the backward errors"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="lu", choices=sorted(CONFIGS))
    ap.add_argument("--cpu-budget", type=float, default=15.0,
                    help="seconds of CPU work for the cpu_baseline sample")
    ap.add_argument("--ref-budget", type=float, default=10.0,
                    help="seconds of CPU work per step of --impl reference")
    ap.add_argument("--count", type=int, default=None,
                    help="override the batch size (small cases for profiling)")
    ap.add_argument("--cond", type=float, default=1e5, help="mixed: condition number")
    ap.add_argument("--lowp", default="tf32x3", choices=["fp32", "tf32", "bf16", "tf32x3"],
                    help="mixed: precision of the factorization")
    ap.add_argument("--n", type=int, default=None, help="mixed: order of the systems")
    ap.add_argument("--no-autotune", action="store_true",
                    help="lu/chol: keep the default launch shape instead of autotuning the plan")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-parity", action="store_true",
                    help="lu: skip the oracle check of the whole timed batch")
    ap.add_argument("--no-mixed", action="store_true",
                    help="lu: skip the mixed-precision sub-measurement")
    ap.add_argument("--no-lu-fma", action="store_true",
                    help="lu: skip the record of the LU's FMA form in the default line")
    ap.add_argument("--fixed-n", type=int, default=None,
                    help="lu, inv, chol100k: every matrix of this order (profiling aid)")
    ap.add_argument("--no-cholesky", action="store_true",
                    help="lu: skip the Cholesky record (100,000 SPD matrices, FMA and exact "
                         "forms) of the default line")
    ap.add_argument("--form", default="exact", choices=["exact", "fma"],
                    help="chol/chol100k: arithmetic form of the factorization (exact: MatFlat's "
                         "bits; fma: fused multiply-adds, checked by backward error)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        print("note: warmup raised to 3", file=sys.stderr)
        args.warmup = 3
    cfg_name = args.config
    if args.count:
        CONFIGS[cfg_name]["count"] = args.count
    if args.fixed_n:
        # Profiling aid: every matrix of the LU / LuInverse batch has this order.
        CONFIGS[cfg_name]["nmin"] = CONFIGS[cfg_name]["nmax"] = args.fixed_n
        CONFIGS[cfg_name]["workload"] += " [all n = %d]" % args.fixed_n
    if args.impl == "reference":
        run_reference(args, cfg_name)
        return

    import torch
    import torch.distributed as dist

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import matflat_gb300 as mf
    from matflat_gb300 import build
    build.build()
    if cfg_name == "mixed":
        run_mixed(args, torch, mf, world, rank, local)
        if world > 1:
            dist.destroy_process_group()
        return

    def barrier():
        if world > 1:
            dist.barrier()

    ctx = mf.context()
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)

    d = make_inputs(cfg_name, rank)
    cfg = CONFIGS[cfg_name]
    count = len(d["n"])
    tuned = None
    traffic_key = None
    if cfg_name in ("qr", "qr32"):
        dt = torch.float32 if cfg_name == "qr32" else torch.float64
        npdt = np.float32 if cfg_name == "qr32" else np.float64
        a_host = torch.from_numpy(d["a"].astype(npdt)).pin_memory()
        b_host = torch.from_numpy(d["b"].astype(npdt)).pin_memory()
        plan = mf.QrBatch(d["m"], d["n"], d["a_off"], d["rdiag_off"], nrhs=1, b_off=d["b_off"])
        if cfg_name == "qr":
            plan.set_form(args.form)
        if not args.no_autotune:
            tuned = plan.autotune()
        a0 = a_host.to("cuda")
        b0 = b_host.to("cuda")
        a = torch.empty_like(a0)
        b = torch.empty_like(b0)
        rdiag = torch.empty(d["rdiag_total"], dtype=dt, device="cuda")
        outs_host = [torch.empty_like(a_host).pin_memory(), torch.empty_like(b_host).pin_memory(),
                     torch.empty(d["rdiag_total"], dtype=dt).pin_memory()]

        def run():
            plan.run(a, rdiag, b, single=(cfg_name == "qr32"))
        outs = [a, b, rdiag]
        flops = qr_flops(d["m"], d["n"], 1)
        byts = qr_bytes(d["m"], d["n"], 1, 4 if cfg_name == "qr32" else 8)
        kernel_key = "qr_batched_kernel_" + ("f32" if cfg_name == "qr32" else "f64")
    else:
        a_host = torch.from_numpy(d["a"]).pin_memory()
        b_host = torch.from_numpy(d["b"]).pin_memory()
        a0 = a_host.to("cuda")
        b0 = b_host.to("cuda")
        a = torch.empty_like(a0)
        b = torch.empty_like(b0)
        info = torch.zeros(count, dtype=torch.int32, device="cuda")
        if cfg_name.startswith("gevd"):
            plan = mf.GevdFrontBatch(d["n"], d["a_off"], d["b_off"], d["a_off"])
            cmat = torch.empty_like(a0)

            def run():
                plan.run(a, b, cmat, info)
            outs = [b, cmat, info]
            flops = gevd_flops(d["n"], cplx=cfg_name == "gevdz")
            byts = gevd_bytes(d["n"], a0.element_size())
            kernel_key = {"gevd": "gevd_front_batched_kernel",
                          "gevd32": "gevd_front_batched_t_kernel_f32",
                          "gevdz": "gevd_front_batched_t_kernel_c128"}[cfg_name]
        elif cfg_name == "inv":
            # Factor once, untimed; the pivots travel as the step's second input.
            piv0 = torch.zeros(d["piv_total"], dtype=torch.int32, device="cuda")
            sign = torch.zeros(count, dtype=torch.int32, device="cuda")
            mf.LuBatch(d["n"], d["a_off"], d["piv_off"]).run(a0, piv0, None, sign, info)
            torch.cuda.synchronize()
            a_host.copy_(a0)
            b_host = piv0.cpu().pin_memory()
            b0 = piv0
            b = torch.empty_like(b0)
            d["a_fac"] = a_host.numpy()
            d["piv"] = b_host.numpy()
            plan = mf.LuInverseBatch(d["n"], d["a_off"], d["piv_off"])

            def run():
                plan.run(a, b, info)
            outs = [a, info]
            flops = inv_flops(d["n"])
            byts = inv_bytes(d["n"])
            kernel_key = "getri_batched_kernel"
        elif cfg_name == "lu":
            plan = mf.LuBatch(d["n"], d["a_off"], d["piv_off"], nrhs=d["nrhs"], b_off=d["b_off"])
            plan.set_form(args.form)
            if not args.no_autotune:
                tuned = plan.autotune()
            piv = torch.zeros(d["piv_total"], dtype=torch.int32, device="cuda")
            sign = torch.zeros(count, dtype=torch.int32, device="cuda")

            def run():
                plan.run(a, piv, b, sign, info)
            outs = [a, b, piv, sign, info]
            flops = lu_flops(d["n"], d["nrhs"])
            byts = lu_bytes(d["n"], d["nrhs"])
            table = tuned[2] if tuned is not None else int(os.environ.get("MFG_LU_GROUPS", "2"))
            if args.form == "fma":
                # FMA form: orders above 152 run the blocked CTA kernel
                big = args.fixed_n is not None and args.fixed_n > 152
                kernel_key = "getrf_big_fma_kernel" if big else "getrf_task_fma_kernel"
            else:
                kernel_key = "getrf_task_kernel" if table >= 0 else "getrf_batched_kernel"
            # traffic.txt holds per-launch figures of the default batch, and of the blocked
            # kernel's 2,048 x n=512 batch; other workloads get none
            if args.fixed_n or args.count:
                traffic_key = ("getrf_big_fma_kernel_n512x2048"
                               if kernel_key == "getrf_big_fma_kernel" and args.fixed_n == 512
                               and count == 2048 else "none")
        elif cfg_name in ("chol", "chol100k"):
            plan = mf.CholeskyBatch(d["n"], d["a_off"], nrhs=d["nrhs"], b_off=d["b_off"])
            plan.set_form(args.form)
            if not args.no_autotune:
                tuned = plan.autotune()

            def run():
                plan.run(a, b, info)
            outs = [a, b, info]
            flops = chol_flops(d["n"], d["nrhs"])
            byts = chol_bytes(d["n"], d["nrhs"])
            kernel_key = "potrf_batched_kernel"
            if cfg_name == "chol100k":
                traffic_key = "potrf_batched_kernel_chol100k"
        elif cfg_name == "bwd":
            plan = mf.CholeskyBatch(d["n"], d["a_off"], nrhs=1, b_off=d["b_off"])
            plan.set_form(args.form)     # fma: the recomputed factor in the FMA form
            g = torch.Generator(device="cuda")
            g.manual_seed(rank)
            lbar = torch.randn(a0.numel(), dtype=torch.float64, device="cuda", generator=g)
            xbar = torch.randn(b0.numel(), dtype=torch.float64, device="cuda", generator=g)
            ldb = torch.ones(count, dtype=torch.float64, device="cuda")
            # x = A^-1 b from the forward pass (factor + solve), once, untimed
            xs = b0.clone()
            fa = a0.clone()
            plan.run(fa, xs, info)
            abar = torch.empty_like(a0)
            bbar = torch.empty_like(b0)
            del fa

            def run():
                plan.backward(a, abar, info, lbar=lbar, logdet_bar=ldb, x=xs, xbar=xbar,
                              bbar=bbar, recompute=True)
            outs = [abar, bbar, info]
            flops = bwd_flops(d["n"])
            byts = bwd_bytes(d["n"])
            kernel_key = "chol_backward_kernel"
        else:
            plan = mf.CholeskyBatch(d["n"], d["a_off"], nrhs=1, b_off=d["b_off"])
            loss = torch.zeros(count, dtype=torch.float64, device="cuda")
            grad = torch.empty_like(a0)

            def run():
                plan.loss_and_grad(a, b, loss, grad, info, keep_factor=True)
            outs = [a, b, loss, grad, info]
            flops = grad_flops(d["n"])
            byts = grad_bytes(d["n"])
            kernel_key = "chol_grad_batched_kernel"
        outs_host = [torch.empty(o.shape, dtype=o.dtype).pin_memory() for o in outs]

    def restore():
        a.copy_(a0, non_blocking=True)
        b.copy_(b0, non_blocking=True)

    # Launches of the library's kernels in one step: the LU runs one persistent launch per
    # lanes-per-matrix bucket present in the batch, every other configuration one launch.
    launches_per_step = 1
    if cfg_name == "lu":
        table = tuned[2] if tuned is not None else int(os.environ.get("MFG_LU_GROUPS", "2"))
        launches_per_step = len({lu_lanes(table, int(v)) for v in np.unique(d["n"])}) \
            if table >= 0 else 1
    elif cfg_name == "bwd":
        launches_per_step = 2     # the recomputed factor, then the backward pass
    elif cfg_name in ("chol", "chol100k") and tuned is not None and tuned[2] < 0:
        launches_per_step = len({chol_lanes(-tuned[2], int(v)) for v in np.unique(d["n"])})

    # ---- device-resident throughput --------------------------------------------------------
    # Every step starts from a cold L2: a 256 MB buffer (twice the L2) is overwritten before the
    # step's timed interval (restore + run), so configurations whose inputs fit in L2 are
    # measured from HBM too.
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.zero_()
            restore()
            run()
        stream.synchronize()
        barrier()
        torch.cuda.synchronize()
        clocks = ClockSampler(local)
        clocks.start()
        sstart = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        kstart = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        kend = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        for i in range(args.steps):
            flush.zero_()
            sstart[i].record(stream)
            restore()
            kstart[i].record(stream)
            run()
            kend[i].record(stream)
        stream.synchronize()
        torch.cuda.synchronize()
        clocks.stop()
        barrier()
    total_ms = sum(s.elapsed_time(e) for s, e in zip(sstart, kend))
    kernel_ms = [s.elapsed_time(e) for s, e in zip(kstart, kend)]
    # The last timed step's outputs, for the parity check against the oracle (after timing).
    parity_outs = None
    if cfg_name == "lu" and rank == 0 and not args.no_parity:
        parity_outs = [t.cpu().numpy() for t in (a, b, piv, sign, info)]
    form_check = None
    if cfg_name in ("chol", "chol100k") and args.form == "fma" and rank == 0:
        form_check = chol_fma_check(torch, d, a0, a, b0, b, info)
    if cfg_name == "qr" and args.form == "fma" and rank == 0:
        form_check = qr_fma_check(d, a.cpu().numpy(), rdiag.cpu().numpy(), b.cpu().numpy())
    if world > 1:
        tt = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        total_ms = float(tt.item())
    ms_per_step = total_ms / args.steps
    value = world * count * args.steps / (total_ms / 1e3)

    # ---- end to end through the C ABI from pinned host memory -------------------------------
    # The host-buffer entry points (mfg_*_batched_host): copies and compute pipelined over chunks
    # of the batch inside one synchronous call, timed by the host clock.  The calls work in
    # place, so the input arrays are restored from pristine pinned copies before each (untimed).
    e2e = None
    if not args.no_e2e and cfg_name != "bwd":
        def pinned_like(t, dtype=None):
            return torch.empty(t.shape, dtype=dtype or t.dtype).pin_memory()

        ins = [a_host, b_host]                       # pristine inputs
        io = [pinned_like(a_host), pinned_like(b_host)]
        if cfg_name == "lu":
            extra = [torch.zeros(d["piv_total"], dtype=torch.int32).pin_memory(),
                     torch.zeros(count, dtype=torch.int32).pin_memory(),
                     torch.zeros(count, dtype=torch.int32).pin_memory()]
            call = lambda: plan.run_host(io[0], extra[0], io[1], extra[1], extra[2])
            up = [io[0], io[1]]
            down = [io[0], io[1]] + extra
        elif cfg_name == "inv":
            extra = [torch.zeros(count, dtype=torch.int32).pin_memory()]
            io[1] = b_host                           # the pivots: read only
            call = lambda: plan.run_host(io[0], io[1], extra[0])
            up = [io[0], io[1]]
            down = [io[0]] + extra
        elif cfg_name in ("chol", "chol100k"):
            extra = [torch.zeros(count, dtype=torch.int32).pin_memory()]
            call = lambda: plan.run_host(io[0], io[1], extra[0])
            up = [io[0], io[1]]
            down = [io[0], io[1]] + extra
        elif cfg_name == "grad":
            extra = [torch.zeros(count, dtype=torch.float64).pin_memory(), pinned_like(a_host),
                     torch.zeros(count, dtype=torch.int32).pin_memory()]
            call = lambda: plan.loss_and_grad_host(io[0], io[1], extra[0], extra[1], extra[2],
                                                   keep_factor=True)
            up = [io[0], io[1]]
            down = [io[0], io[1]] + extra
        elif cfg_name.startswith("gevd"):
            extra = [pinned_like(a_host), torch.zeros(count, dtype=torch.int32).pin_memory()]
            io[0] = a_host                           # A: read only
            call = lambda: plan.run_host(io[0], io[1], extra[0], extra[1])
            up = [io[0], io[1]]
            down = [io[1]] + extra
        else:                                        # qr, qr32
            extra = [pinned_like(outs_host[2])]
            single = cfg_name == "qr32"
            call = lambda: plan.run_host(io[0], extra[0], io[1], single=single)
            up = [io[0], io[1]]
            down = [io[0], io[1]] + extra
        times = []
        for it in range(2 + args.steps):
            for src, dst in zip(ins, io):
                if dst is not src:
                    dst.copy_(src)
            torch.cuda.synchronize()
            barrier()
            t_0 = time.perf_counter()
            call()
            t_1 = time.perf_counter()
            if it >= 2:
                times.append(t_1 - t_0)
        e2e_ms = 1e3 * sum(times) / len(times)
        if world > 1:
            tt = torch.tensor([e2e_ms], device="cuda")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            e2e_ms = float(tt.item())
        nbytes = lambda ts: int(sum(t.numel() * t.element_size() for t in ts))
        e2e = {"value": world * count / (e2e_ms / 1e3), "unit": "matrices/s",
               "h2d_bytes_per_step": nbytes(up), "d2h_bytes_per_step": nbytes(down),
               "ms_per_step": e2e_ms,
               "path": "host-buffer entry point on page-locked host arrays (copies pipelined "
                       "with compute over chunks of the batch), host wall clock per call"}

    # ---- roofline of the dominant kernel -----------------------------------------------------
    fp64_peak = measure_fp64_peak(torch)
    kmed = statistics.median(kernel_ms)
    achieved_tf = flops / (kmed / 1e3) / 1e12
    traffic = read_traffic(traffic_key or kernel_key)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    roof = {
        "bound": "fp64",
        "achieved": achieved_tf, "peak": fp64_peak, "unit": "TFLOP/s",
        "frac": achieved_tf / fp64_peak,
        "peak_source": "measured in this run: cuBLAS DGEMM 4096^3 (FP64 has no entry in "
                       "MEASURED_PEAKS.json)",
        "exact_order_ceiling_frac": 0.5,
        "note": "MatFlat-exact arithmetic issues every multiply and add separately (no FMA): on "
                "the FP64 pipe alone that caps a kernel at half the DFMA peak; kernels that move "
                "the multiplies to the integer pipes (getrf, potrf) can pass that ceiling",
        "traffic": traffic, "algorithmic_bytes_per_launch": byts,
        "hbm_achieved_gbs": byts / (kmed / 1e3) / 1e9, "hbm_peak_gbs": hbm,
        "hbm_frac": byts / (kmed / 1e3) / 1e9 / hbm,
        "kernel_ms": kmed, "kernel": kernel_key,
    }

    # ---- CPU baseline (rank 0, N=1 only) ----------------------------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and cfg_name != "bwd":
        rate, sample_n, threads, t = cpu_sample_rate(cfg_name, d, budget_s=args.cpu_budget)
        cpu = {"value": rate, "unit": "matrices/s", "cores": threads, "kind": "port",
               "sample": "%d matrices (batch of %d, evenly strided, repeated if smaller than "
                         "the budget; %.1f s)" % (sample_n, count, t)}
        rate1, n1, _, t1s = cpu_sample_rate(cfg_name, d, budget_s=max(1.0, args.cpu_budget / 4),
                                            threads=1)
        cpu["single_thread"] = {"value": rate1, "sample": "%d matrices, 1 thread (%.1f s)"
                                                          % (n1, t1s)}

    # ---- parity of the whole timed batch against the oracle (rank 0, after timing) -----------
    parity = None
    if parity_outs is not None:
        parity = lu_parity(d, *parity_outs)

    # ---- the mixed-precision half of the metric (2,048 systems n=512, cond 1e5) --------------
    mixed = None
    if cfg_name == "lu" and not args.no_mixed:
        mcfg = CONFIGS["mixed"]
        r = measure_mixed(torch, mf, torch.cuda.Stream(), mcfg["count"], mcfg["n"], 1e5,
                          args.lowp, 3, 3, rank, local, with_e2e=False)
        if world > 1:
            tt = torch.tensor([r["ms"], r["fp64_plain"]["ms"]], device="cuda")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            r["ms"], r["fp64_plain"]["ms"] = float(tt[0].item()), float(tt[1].item())
        mixed = {"workload": mcfg["workload"] + ", cond 1e5", "lowp": args.lowp,
                 "value": world * mcfg["count"] / (r["ms"] / 1e3), "unit": "solves/s",
                 "ms_per_solve_batch": r["ms"],
                 "fp64_plain_value": world * mcfg["count"] / (r["fp64_plain"]["ms"] / 1e3),
                 "fp64_plain_ms": r["fp64_plain"]["ms"],
                 "speedup_vs_fp64_plain": r["fp64_plain"]["ms"] / r["ms"],
                 "fp64_plain_fma": r["fp64_plain_fma"],
                 "speedup_vs_fp64_plain_fma": r["fp64_plain_fma"]["ms"] / r["ms"],
                 "berr_max": r["berr_max"], "berr_median": r["berr_median"],
                 "fwd_err_max": r["fwd_err_max"], "fp64_plain_fwd_err_max": r["fp64_plain"]["fwd_err_max"],
                 "iters_histogram": r["iters_histogram"], "fallback_fp64": r["fallback_fp64"],
                 "timing": "CUDA events on the solver's stream, 3 warm-up + 3 timed solves; "
                           "plain rates: one timed FP64 LU + solve of the same systems in the "
                           "exact form and one in the FMA form"}

    # ---- the Cholesky half of the metric (100,000 SPD matrices n~U{8..128}) -------------------
    cholesky = None
    if cfg_name == "lu" and not args.no_cholesky:
        cholesky = measure_cholesky(torch, mf, rank, 5, 3, fp64_peak)
    lu_fma = None
    if cfg_name == "lu" and args.form == "exact" and not args.no_lu_fma:
        lu_fma = measure_lu_fma(torch, mf, d, rank, 5, 3, fp64_peak, flops)

    if rank == 0:
        line = {
            "metric": metric_name(cfg_name), "value": value, "unit": "matrices/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype_name(cfg_name),
            "data": "synthetic (seeded SplitMix64 + Box-Muller, identical bytes for CPU and GPU)",
            "config": {"workload": cfg["workload"], "count": count,
                       "per_rank_batch": count,
                       "l2": "L2 flushed (256 MB write) before every step, outside its timed "
                             "interval; inputs %.2f GB" % (a0.numel() * a0.element_size() / 1e9),
                       "step_includes": "device-to-device restore of the input batch + the "
                                        "batched factorization/solve (one graph replay)"},
            "kernel_ms_per_step": kmed,
            "launch_shape": None if tuned is None else dict(
                zip(["warps_per_cta", "warps_per_sm",
                     "lanes_table" if cfg_name == "lu" else "lanes_per_matrix", "mul_mode",
                     "dot_pairs_per_block"], tuned),
                source="mfg_plan_autotune at plan creation (outside the timed region)"),
            "gpu_launches": args.steps * launches_per_step,
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "clocks": clocks.summary(),
        }
        if parity is not None:
            line["parity"] = parity
        if form_check is not None:
            line["config"]["form"] = ("fma: fused multiply-adds, reciprocal column scaling "
                                      "(mfg_plan_set_form); not MatFlat's bits, checked by "
                                      "backward error")
            line["form_check"] = form_check
        if mixed is not None:
            line["mixed"] = mixed
        if cholesky is not None:
            line["cholesky"] = cholesky
        if lu_fma is not None:
            line["lu_fma"] = lu_fma
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

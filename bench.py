"""Benchmark: batched FP64 Cholesky solve on GB300 (BLAST potrf + two trsm), plus the other four
workloads of the same library on the same GPU in the same run.

Headline workload (one "step"): 50,000 SPD matrices n = 48, A = G*G^T + 48*I with G i.i.d. N(0,1),
B (48 x 8) i.i.d. N(0,1); potrf(A, L) then L*Y = B, L^T*X = Y, all binary64, inputs resident in HBM
(1.07 GB of inputs, larger than the 129 MB L2, so no L2 flush is needed between steps). The inputs
are drawn on the host from numpy's default_rng(7), so the GPU arm, the CPU baseline and the
reference arm solve the same matrices, and the parity figures compare the GPU's timed results
with the oracle (BLAST's algorithm restated in C++) and with LAPACK on a strided sample of them.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line. `value` is matrices/s measured with CUDA events on the launching stream
(max over ranks); `e2e` is the same metric through the public API with pinned host buffers and
the host<->device traffic inside the timed region; `roofline` is the binary64 issue bound of the
dominant kernel; `cpu_baseline` times the CPU restatement of BLAST's algorithm on this host.
The keys `gemm24`, `lu_ragged`, `mixed_ir` and `adjoint` carry the other workloads (24x24 gemm
batch, ragged LU, mixed precision + refinement, differentiable solve), each with its timing,
roofline, CPU baseline and parity against the oracle and LAPACK on its own inputs.
With --impl reference the CPU restatement of BLAST (one instance per call, instances spread over
all host cores with OpenMP) is timed on the same workload and metric.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N, NRHS, BATCH = 48, 8, 50_000
FLOPS_PER = N ** 3 / 3 + N ** 2 / 2 + N / 6 + 2 * N * N * NRHS          # 74,888
BYTES_PER = 8 * (N * (N + 1) // 2 * 2 + 2 * N * NRHS)                     # 24,960 (lower A in, L out, B in, X out)
METRIC = "matrices/s, GFLOP/s on 1 GB300: FP64 vs mixed+IR batched potrf at 1e-12 bwd err"
WORKLOAD = "FP64 batched Cholesky solve: potrf + 2 trsm, 50,000 SPD n=48 (A = G*G^T + 48*I), B 48x8"
SEED = 7
EPS = 2.0 ** -52


def contract_config(batch: int = BATCH) -> dict:
    """The workload-defining keys, identical in both arms."""
    return {"workload": WORKLOAD, "batch_per_gpu": batch, "n": N, "nrhs": NRHS, "dtype": "f64", "seed": SEED}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.out = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        if not self.out:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------------------------
# Inputs (seeded, on the host, shared by every arm)
# ---------------------------------------------------------------------------------------------
def host_inputs(batch: int, seed: int = SEED):
    """The headline batch: A = G G^T + 48 I (G i.i.d. N(0,1)), B i.i.d. N(0,1), numpy float64."""
    import numpy as np

    rng = np.random.default_rng(seed)
    A = np.empty((batch, N, N))
    step = 4096
    for b0 in range(0, batch, step):
        G = rng.standard_normal((min(step, batch - b0), N, N))
        np.matmul(G, np.swapaxes(G, 1, 2), out=A[b0:b0 + len(G)])
    A += N * np.eye(N)
    B = rng.standard_normal((batch, N, NRHS))
    return A, B


def _to_dev_batch(h, device):
    """numpy (batch, r, c) -> column-major-per-matrix float64 CUDA tensor of the same shape."""
    import torch

    import blast_gb300 as bg

    t = bg.col_major((h.shape[0],), h.shape[1], h.shape[2], device)
    step = 8192
    for b0 in range(0, h.shape[0], step):
        t[b0:b0 + step].copy_(torch.from_numpy(h[b0:b0 + step]))
    return t


def _sample(batch: int, k: int):
    import numpy as np

    return np.unique(np.linspace(0, batch - 1, min(k, batch)).astype(np.int64))


def _normwise(x, ref) -> float:
    import numpy as np

    den = np.linalg.norm(ref)
    return float(np.linalg.norm(np.asarray(x) - ref) / (den if den > 0 else 1.0))


def peak_fp64_tflops() -> float:
    """Binary64 FMA throughput of this GPU, measured by the library's probe kernel."""
    import ctypes

    import torch

    from blast_gb300 import _lib

    out = ctypes.c_double(0.0)
    _lib.call("blastgpu_probe_fp64_tflops", ctypes.byref(out), torch.cuda.current_stream().cuda_stream)
    return out.value


def peak_dmma_tflops() -> float:
    """Binary64 tensor-core (DMMA) throughput of this GPU, measured by the library's probe kernel."""
    import ctypes

    import torch

    from blast_gb300 import _lib

    out = ctypes.c_double(0.0)
    _lib.call("blastgpu_probe_fp64_dmma_tflops", ctypes.byref(out), torch.cuda.current_stream().cuda_stream)
    return out.value


def peak_mma_tflops(kind: int) -> float:
    """mma.sync throughput (0: TF32 m16n8k8, 1: BF16 m16n8k16) measured by the library's probe kernel."""
    import ctypes

    import torch

    from blast_gb300 import _lib

    out = ctypes.c_double(0.0)
    _lib.call("blastgpu_probe_mma_tflops", kind, ctypes.byref(out), torch.cuda.current_stream().cuda_stream)
    return out.value


def _hbm_peak():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("hbm_gbs")
    except (OSError, ValueError):
        return None


def _roofline(flops: float, nbytes: float, ms: float, peak: float, kernel: str) -> dict:
    achieved = flops / (ms * 1e-3) / 1e12
    hbm = _hbm_peak()
    gbs = nbytes / (ms * 1e-3) / 1e9
    return {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak if peak else None, "kernel": kernel,
            "peak_source": "binary64 FMA probe kernel run in this process (MEASURED_PEAKS.json has no FP64 figure)",
            "hbm": {"achieved_gbs": gbs, "peak_gbs": hbm, "frac": gbs / hbm if hbm else None,
                    "algorithmic_bytes": nbytes}}


def _timed(fn, steps, warm=3):
    import torch

    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


# ---------------------------------------------------------------------------------------------
# Headline parity (same inputs, strided sample, oracle and LAPACK)
# ---------------------------------------------------------------------------------------------
def posv_parity(A_h, B_h, L_dev, X_dev, k: int = 256) -> dict:
    """The GPU's factors and solutions of a strided sample of the timed batch, against the oracle
    (BLAST's algorithm in C++) and against LAPACK (SciPy dpotrf/dpotrs), normwise per instance."""
    import numpy as np
    import scipy.linalg.lapack as lapack

    from oracle import oracle as orc

    idx = _sample(A_h.shape[0], k)
    ti = __import__("torch").from_numpy(idx).to(L_dev.device)
    Lg = np.tril(L_dev.index_select(0, ti).cpu().numpy())
    Xg = X_dev.index_select(0, ti).cpu().numpy()
    Lo, Xo, info = orc.posv_batch(A_h[idx], B_h[idx])
    el_o, ex_o, el_l, ex_l = [], [], [], []
    for j, b in enumerate(idx):
        c, st = lapack.dpotrf(A_h[b], lower=1, clean=1)
        x, st2 = lapack.dpotrs(c, B_h[b], lower=1)
        el_o.append(_normwise(Lg[j], np.tril(Lo[j])))
        ex_o.append(_normwise(Xg[j], Xo[j]))
        el_l.append(_normwise(Lg[j], c))
        ex_l.append(_normwise(Xg[j], x))
    bound = 10 * N * EPS
    return {"n_checked": int(len(idx)), "sample": f"every {A_h.shape[0] // len(idx)}th instance of the timed batch",
            "L_max_normwise_vs_oracle": max(el_o), "X_max_normwise_vs_oracle": max(ex_o),
            "L_max_normwise_vs_lapack": max(el_l), "X_max_normwise_vs_lapack": max(ex_l),
            "bound_10_n_eps": bound,
            "within_bound": bool(max(el_o + ex_o + el_l + ex_l) <= bound),
            "oracle_info_nonzero": int(np.count_nonzero(info))}


# ---------------------------------------------------------------------------------------------
# CPU baseline and reference arm
# ---------------------------------------------------------------------------------------------
def cpu_baseline(A_h, B_h, min_seconds: float = 1.5):
    """The oracle's BLAST restatement on all of this host's cores: whole passes over the bench's
    50,000-matrix workload (the GPU arm's own inputs), repeated for at least min_seconds of wall
    time (16 threads x 1.5 s is about 24 s of CPU work)."""
    from oracle import oracle as orc

    prep = orc.posv_prepare(A_h, B_h)
    sample = A_h.shape[0]
    threads = orc.max_threads()
    orc.posv_run(prep, threads)  # warm-up
    reps, t0 = 0, time.perf_counter()
    while True:
        orc.posv_run(prep, threads)
        reps += 1
        el = time.perf_counter() - t0
        if el >= min_seconds and reps >= 2:
            break
    rate = reps * sample / el
    return {"value": rate, "unit": "matrices/s", "cores": threads, "kind": "port",
            "gflops": rate * FLOPS_PER / 1e9, "host_cpus": os.cpu_count(),
            "build": "g++ -O3 -fopenmp -ffp-contract=off (no -march=native: host code is built "
                     "identically on every machine)",
            "sample": f"{reps} passes over the {sample} matrices of the workload (n=48, 8 RHS, the GPU "
                      f"arm's inputs), one instance per call, OpenMP over {threads} threads of "
                      f"{os.cpu_count()} host CPUs, {el:.2f} s wall"}


def run_reference(args):
    """The reference arm: the oracle (BLAST's algorithm restated in C++, compiled -O3) on all host
    cores; a step is one pass over the same 50,000-matrix workload; W untimed steps, K timed."""
    ws, rank = _dist()
    if rank != 0:
        return
    from oracle import oracle as orc

    A_h, B_h = host_inputs(BATCH)
    prep = orc.posv_prepare(A_h, B_h)
    del A_h, B_h
    threads = orc.max_threads()
    for _ in range(max(1, args.warmup)):
        orc.posv_run(prep, threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        orc.posv_run(prep, threads)
    el = time.perf_counter() - t0
    rate = args.steps * BATCH / el
    line = {"metric": METRIC, "value": rate, "unit": "matrices/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, numpy default_rng(7))",
            "impl": "reference",
            "config": contract_config(),
            "setup": {"parallelism": f"host cores of rank 0 ({threads} threads of {os.cpu_count()} CPUs)"},
            "gflops": rate * FLOPS_PER / 1e9,
            "cpu_baseline": {"value": rate, "unit": "matrices/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} timed passes over {BATCH} matrices after "
                                       f"{max(1, args.warmup)} untimed, OpenMP over {threads} "
                                       f"threads, {el:.2f} s wall"},
            "e2e": {"value": rate, "unit": "matrices/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------------
# Config 1: gemm 10,000 x 24x24x24
# ---------------------------------------------------------------------------------------------
def config_gemm24(steps: int, peak: float | None, cpu: bool = True) -> dict:
    """D = A*B + C (alpha = beta = 1), 10,000 instances of 24x24x24, U[-1,1], column-major."""
    import numpy as np
    import torch

    import blast_gb300 as bg
    from oracle import oracle as orc

    batch, m = 10_000, 24
    rng = np.random.default_rng(99)
    Ah, Bh, Ch = (rng.uniform(-1.0, 1.0, (batch, m, m)) for _ in range(3))
    A, B, C = (_to_dev_batch(h, "cuda") for h in (Ah, Bh, Ch))
    D = bg.col_major((batch,), m, m, "cuda")
    ms = _timed(lambda: bg.gemm(A, B, C, D), steps)
    flops = 2.0 * m ** 3 * batch
    nbytes = 8.0 * 4 * m * m * batch
    Dg = D.cpu().numpy()
    threads = orc.max_threads()
    Do = orc.gemm_batch(1.0, Ah, Bh, 1.0, Ch, threads)
    Dn = Ah @ Bh + Ch
    out = {"workload": "gemm D = A*B + C, 10,000 x 24x24x24, U[-1,1], seed 99", "ms_per_step": ms,
           "matrices_per_s": batch / ms * 1e3, "gflops": flops / ms / 1e6, "steps": steps,
           "roofline": _roofline(flops, nbytes, ms, peak, "gemm_warp_kernel"),
           "parity": {"n_checked": batch,
                      "bitwise_equal_to_oracle": bool(np.array_equal(Dg, Do)),
                      "max_normwise_vs_oracle": max(_normwise(Dg[b], Do[b]) for b in range(batch)),
                      "max_normwise_vs_numpy_blas": max(_normwise(Dg[b], Dn[b]) for b in range(batch)),
                      "bound_10_n_eps": 10 * m * EPS}}
    if cpu:
        prep = orc.gemm_prepare(1.0, Ah, Bh, 1.0, Ch)
        orc.gemm_run(prep, threads)  # warm-up
        reps, t0 = 0, time.perf_counter()
        while True:
            orc.gemm_run(prep, threads)
            reps += 1
            el = time.perf_counter() - t0
            if el >= 1.0 and reps >= 3:
                break
        rate = reps * batch / el
        out["cpu_baseline"] = {"value": rate, "unit": "matrices/s", "cores": threads, "kind": "port",
                               "gflops": rate * 2.0 * m ** 3 / 1e9,
                               "sample": f"{reps} passes over the 10,000 instances, OpenMP over {threads} threads"}
        out["gpu_over_cpu"] = out["matrices_per_s"] / rate
    return out


# ---------------------------------------------------------------------------------------------
# Config 3: ragged LU, 20,000 x n log-uniform [4, 256]
# ---------------------------------------------------------------------------------------------
def lu_inputs(count: int, seed: int = 2020):
    import numpy as np

    rng = np.random.default_rng(seed)
    ns = np.floor(np.exp(rng.uniform(np.log(4), np.log(257), count))).astype(np.int64)
    ns = np.minimum(ns, 256)
    Abuf = rng.standard_normal(int(np.sum(ns * ns)))
    bbuf = rng.standard_normal(int(np.sum(ns)))
    return ns, Abuf, bbuf


def config_lu_ragged(steps: int, peak: float | None, count: int = 20_000, cpu: bool = True) -> dict:
    """getrf + getrs on 20,000 general matrices, n log-uniform in [4, 256], N(0,1), one RHS."""
    import numpy as np
    import scipy.linalg.lapack as lapack
    import torch

    from blast_gb300.ragged import GesvPlan, Packed
    from oracle import oracle as orc

    ns, Abuf, bbuf = lu_inputs(count)
    A = Packed(ns, ns, "cuda")
    B = Packed(ns, np.ones_like(ns), "cuda")
    A0 = torch.from_numpy(Abuf).to("cuda")
    B0 = torch.from_numpy(bbuf).to("cuda")
    plan = GesvPlan(A, B)

    def step():
        A.buf[:A0.numel()].copy_(A0)
        B.buf[:B0.numel()].copy_(B0)
        plan.run()

    ms_copy = _timed(lambda: (A.buf[:A0.numel()].copy_(A0), B.buf[:B0.numel()].copy_(B0)), steps)
    ms = _timed(step, steps) - ms_copy
    step()
    torch.cuda.synchronize()
    flops = float(np.sum(2 * ns ** 3 / 3 - ns ** 2 / 2 + 5 * ns / 6 + 2 * ns ** 2 - ns))
    nbytes = float(np.sum(16 * ns * ns + 16 * ns + 4 * ns))
    LUg = A.buf.cpu().numpy()
    xg = B.buf.cpu().numpy()
    pg = plan.pivots()
    info_g = plan.info_host()
    offA = A.offsets
    offb = B.offsets
    A_list = [Abuf[offA[i]:offA[i] + ns[i] ** 2].reshape(ns[i], ns[i], order="F") for i in range(count)]
    b_list = [bbuf[offb[i]:offb[i] + ns[i]] for i in range(count)]
    threads = orc.max_threads()
    t0 = time.perf_counter()
    LUo, xo, po, info_o = orc.gesv_ragged(ns, A_list, b_list, threads)
    cpu_s = time.perf_counter() - t0
    piv_mismatch = sum(int(not np.array_equal(pg[i], po[i])) for i in range(count))
    lu_err = max(_normwise(LUg[offA[i]:offA[i] + ns[i] ** 2], LUo[i].reshape(-1, order="F")) for i in range(count))
    x_err = max(_normwise(xg[offb[i]:offb[i] + ns[i]], xo[i]) for i in range(count))
    # LAPACK on a strided sample: solution error and pivot agreement (LAPACK's blocked getrf may
    # pick another row where two candidates are within rounding of each other)
    idx = _sample(count, 256)
    xl_err, piv_diff_lapack = [], 0
    for i in idx:
        lu, piv, st = lapack.dgetrf(A_list[i])
        x, st2 = lapack.dgetrs(lu, piv, b_list[i])
        xl_err.append(_normwise(xg[offb[i]:offb[i] + ns[i]], x))
        if not np.array_equal(piv.astype(np.int32), pg[i]):
            piv_diff_lapack += 1
    out = {"workload": "getrf + getrs, 20,000 x n log-uniform [4,256], N(0,1), 1 RHS, seed 2020",
           "ms_per_step": ms, "matrices_per_s": count / ms * 1e3, "gflops": flops / ms / 1e6, "steps": steps,
           "timing_note": "each step re-copies the inputs (getrf works in place); the copy time, timed "
                          "alone, is subtracted",
           "roofline": _roofline(flops, nbytes, ms, peak, "getrf_cta_kernel + getrf_warp_kernel + getrs_kernel"),
           "parity": {"n_checked": count,
                      "pivot_sequences_identical_to_oracle": count - piv_mismatch,
                      "pivot_mismatches_vs_oracle": piv_mismatch,
                      "LU_max_normwise_vs_oracle": lu_err, "x_max_normwise_vs_oracle": x_err,
                      "info_equal_to_oracle": bool(np.array_equal(info_g, info_o)),
                      "lapack_n_checked": int(len(idx)),
                      "x_max_normwise_vs_lapack": max(xl_err),
                      "pivot_sequences_differing_from_lapack": piv_diff_lapack}}
    if cpu:
        out["cpu_baseline"] = {"value": count / cpu_s, "unit": "matrices/s", "cores": threads, "kind": "port",
                               "gflops": flops / cpu_s / 1e9,
                               "sample": f"one pass over the 20,000 instances (the GPU's inputs), OpenMP over "
                                         f"{threads} threads, {cpu_s:.2f} s"}
        out["gpu_over_cpu"] = out["matrices_per_s"] / out["cpu_baseline"]["value"]
    out["mixed"] = lu_mixed_comparison(steps, ns, A0, B0, A_list, b_list, xg, offb, ms)
    return out


def lu_mixed_comparison(steps, ns, A0, B0, A_list, b_list, x64, offb, ms64) -> dict:
    """The same 20,000 systems through the mixed-precision LU solve (binary32 factor, binary64
    refinement to a normwise backward error <= 1e-12), against the binary64 getrf + getrs."""
    import numpy as np
    import scipy.linalg.lapack as lapack
    import torch

    from blast_gb300.ragged import MixedGesvPlan, Packed

    count = len(ns)
    A = Packed(ns, ns, "cuda")
    B = Packed(ns, np.ones_like(ns), "cuda")
    A.buf[:A0.numel()].copy_(A0)
    plan = MixedGesvPlan(A, B, tol=1e-12, max_iter=10)

    def step():
        B.buf[:B0.numel()].copy_(B0)  # X overwrites B; A is read only
        plan.run()

    ms_copy = _timed(lambda: B.buf[:B0.numel()].copy_(B0), steps)
    ms = _timed(step, steps) - ms_copy
    step()
    torch.cuda.synchronize()
    info, iters, berr = plan.results()
    xm = B.buf.cpu().numpy()
    ok = info == 0
    fwd_vs_fp64 = max(_normwise(xm[offb[i]:offb[i] + ns[i]], x64[offb[i]:offb[i] + ns[i]])
                      for i in range(count) if ok[i])
    idx = _sample(count, 256)
    be_cpu, fwd_lapack = [], []
    for i in idx:
        if not ok[i]:
            continue
        x = xm[offb[i]:offb[i] + ns[i]]
        r = b_list[i] - A_list[i] @ x
        be_cpu.append(float(np.abs(r).max() / (np.abs(A_list[i]).sum(1).max() * np.abs(x).max()
                                                 + np.abs(b_list[i]).max())))
        lu, piv, _ = lapack.dgetrf(A_list[i])
        xl, _ = lapack.dgetrs(lu, piv, b_list[i])
        fwd_lapack.append(_normwise(x, xl))
    hist = {str(k): int(v) for k, v in zip(*np.unique(iters[ok], return_counts=True))}
    return {"ms_per_step": ms, "matrices_per_s": count / ms * 1e3, "steps": steps,
            "speedup_over_fp64_lu": ms64 / ms,
            "converged": int(np.sum(ok & (berr <= 1e-12))), "zero_pivot_instances": int(np.sum(~ok)),
            "max_backward_error": float(berr[ok].max()), "corrections_histogram": hist,
            "parity": {"x_max_normwise_vs_fp64_path": fwd_vs_fp64,
                       "lapack_n_checked": len(fwd_lapack), "x_max_normwise_vs_lapack": max(fwd_lapack),
                       "backward_error_recomputed_on_cpu_max": max(be_cpu)},
            "timing_note": "each step re-copies B (X overwrites it); the copy time, timed alone, is subtracted"}


# ---------------------------------------------------------------------------------------------
# Config 4: mixed precision + refinement vs the binary64 path
# ---------------------------------------------------------------------------------------------
def make_mixed_inputs(count: int, seed: int, device, gen: str = "qr"):
    """The mixed-precision workload: n ~ U{64..512}; A = Q diag(lambda) Q^T with Q from the QR of a
    seeded Gaussian and lambda log-spaced so that cond(A) is 1e2, 1e4 or 1e6 (a third each);
    one N(0,1) right-hand side. Built on the device in binary64, grouped by size."""
    import numpy as np
    import torch

    from blast_gb300.ragged import Packed

    rng = np.random.default_rng(seed)
    ns = rng.integers(64, 513, count)
    conds = np.array([1e2, 1e4, 1e6])[np.arange(count) % 3]
    A = Packed(ns, ns, device)
    B = Packed(ns, np.ones_like(ns), device)
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    for n in np.unique(ns):
        idx = np.nonzero(ns == n)[0]
        G = torch.randn(len(idx), n, n, generator=g, device=device, dtype=torch.float64)
        if gen == "gram":
            # Profiling stand-in without torch.linalg (SPD, same sizes, well conditioned).
            M = G @ G.mT / n + torch.eye(n, device=device, dtype=torch.float64)
            for j, i in enumerate(idx):
                A.view(int(i)).copy_(M[j])
            continue
        Q, _ = torch.linalg.qr(G)
        lam = torch.stack([torch.logspace(0, -float(np.log10(conds[i])), n, device=device,
                                          dtype=torch.float64) for i in idx])
        M = (Q * lam[:, None, :]) @ Q.mT
        M = 0.5 * (M + M.mT)
        for j, i in enumerate(idx):
            A.view(int(i)).copy_(M[j])
        del G, Q, M
    B.buf.copy_(torch.randn(B.buf.numel(), generator=g, device=device, dtype=torch.float64))
    return ns, conds, A, B


def mixed_ir_comparison(steps: int, count: int = 8192, gen: str = "qr", parity: bool = True):
    """FP64 vs mixed-precision + refinement on the ragged n in [64, 512] batch (one CTA per
    matrix, one launch per size bin and step for each path)."""
    import numpy as np
    import torch

    from blast_gb300.ragged import Packed, PosvPlan

    dev = torch.device("cuda", torch.cuda.current_device())
    ns, conds, A, B = make_mixed_inputs(count, 4321, dev, gen)
    ones = np.ones_like(ns)
    X64, X32 = Packed(ns, ones, dev), Packed(ns, ones, dev)
    L = Packed(ns, ns, dev)
    p64 = PosvPlan(A, B, X64, L)
    pmx = PosvPlan(A, B, X32, mixed=True, tol=1e-12, max_iter=10)
    flops = float(np.sum(ns.astype(np.float64) ** 3 / 3 + ns ** 2 / 2 + ns / 6 + 2 * ns ** 2))
    out = {}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for name, plan, k in (("fp64", p64, max(1, steps // 4)), ("mixed", pmx, steps)):
        plan.run()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(k):
            plan.run()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / k
        out[name] = {"ms_per_step": ms, "matrices_per_s": count / ms * 1e3,
                     "gflops_nominal": flops / ms / 1e6, "steps": k}
    info, iters, berr = pmx.results()
    info64, _, _ = p64.results()
    out["mixed"].update({"max_backward_error": float(np.max(berr)),
                         "converged": int(np.sum((berr <= 1e-12) & (info == 0))),
                         "iterations_histogram": {int(k): int(v) for k, v in zip(*np.unique(iters, return_counts=True))},
                         "factorisation_breakdowns": int(np.sum(info != 0))})
    out["fp64"]["info_nonzero"] = int(np.sum(info64 != 0))
    out["speedup_matrices_per_s"] = out["mixed"]["matrices_per_s"] / out["fp64"]["matrices_per_s"]
    out["workload"] = (f"{count} SPD matrices, n ~ U{{64..512}}, A = Q diag(lambda) Q^T, "
                       "cond in {1e2,1e4,1e6}, 1 RHS; tol 1e-12" if gen == "qr" else
                       f"{count} SPD matrices, n ~ U{{64..512}}, A = G G^T/n + I (profiling)")
    if parity:
        out["parity"] = mixed_parity(ns, conds, A, B, X64, X32)
    return out


def mixed_parity(ns, conds, A, B, X64, X32, per_bucket: int = 24) -> dict:
    """Per condition-number bucket: the mixed path's solutions against the binary64 path's (all
    instances) and, with the binary64 path's, against LAPACK (SciPy dpotrf/dpotrs) and its
    backward error, on a strided sample."""
    import numpy as np
    import scipy.linalg.lapack as lapack

    x64, x32 = X64.to_list(), X32.to_list()
    res = {}
    for c in (1e2, 1e4, 1e6):
        idx = np.nonzero(conds == c)[0]
        fe = [_normwise(x32[i], x64[i]) for i in idx]
        samp = idx[np.unique(np.linspace(0, len(idx) - 1, min(per_bucket, len(idx))).astype(int))]
        fl_mixed, fl_64, be64 = [], [], []
        for i in samp:
            a = A.view(int(i)).cpu().numpy()
            b = B.view(int(i)).cpu().numpy()
            cf, st = lapack.dpotrf(a, lower=1, clean=1)
            x, st2 = lapack.dpotrs(cf, b, lower=1)
            fl_mixed.append(_normwise(x32[i], x))
            fl_64.append(_normwise(x64[i], x))
            r = b - a @ x64[i]
            be64.append(float(np.abs(r).max() / (np.abs(a).sum(1).max() * np.abs(x64[i]).max() + np.abs(b).max())))
        res[f"cond_{c:.0e}"] = {"instances": int(len(idx)),
                                "mixed_max_normwise_vs_fp64_path": float(max(fe)),
                                "lapack_n_checked": int(len(samp)),
                                "mixed_max_normwise_vs_lapack": float(max(fl_mixed)),
                                "fp64_max_normwise_vs_lapack": float(max(fl_64)),
                                "fp64_max_backward_error": float(max(be64))}
    return res


# ---------------------------------------------------------------------------------------------
# Config 5: differentiable SPD solve (forward potrf + potrs, hand-written adjoint)
# ---------------------------------------------------------------------------------------------
def config_adjoint(steps: int, peak: float | None, count: int = 8192) -> dict:
    """8,192 SPD n ~ U{32..128} (A = G G^T + n I), b, t ~ N(0,1); loss 1/2 |x - t|^2: the forward
    solve and the adjoint (factor kept), with gradients against a CPU binary64 reference."""
    import numpy as np
    import scipy.linalg.lapack as lapack
    import torch

    from blast_gb300 import _lib, desc
    from blast_gb300.ragged import Packed, PosvPlan
    from oracle import oracle as orc

    rng = np.random.default_rng(55)
    ns = rng.integers(32, 129, count)
    A = Packed(ns, ns, "cuda")
    A_h = []
    for n in ns:
        G = rng.standard_normal((n, n))
        A_h.append(G @ G.T + n * np.eye(n))
    A.fill_from(A_h)
    ones = np.ones_like(ns)
    B, X, T = Packed(ns, ones, "cuda"), Packed(ns, ones, "cuda"), Packed(ns, ones, "cuda")
    b_h = [rng.standard_normal((n, 1)) for n in ns]
    t_h = [rng.standard_normal((n, 1)) for n in ns]
    B.fill_from(b_h)
    T.fill_from(t_h)
    L = Packed(ns, ns, "cuda")
    fwd = PosvPlan(A, B, X, L)
    G_, GB, GA = Packed(ns, ones, "cuda"), Packed(ns, ones, "cuda"), Packed(ns, ns, "cuda")
    recs = np.zeros(count, dtype=desc.POSV_BWD_DTYPE)
    order = np.argsort(-ns, kind="stable")
    for slot, i in enumerate(order):
        recs[slot] = (A.record(i), L.record(i), X.record(i), G_.record(i), GB.record(i), GA.record(i))
    d = desc.upload(recs, "cuda")
    info = torch.zeros(count, dtype=torch.int32, device="cuda")

    def bwd():
        torch.sub(X.buf, T.buf, out=G_.buf)  # dl/dx for l = |x - t|^2 / 2
        _lib.call("blastgpu_dposv_bwd_batched", d.data_ptr(), count, int(ns.max()), 0, info.data_ptr(),
                  torch.cuda.current_stream().cuda_stream)

    ms_f = _timed(fwd.run, steps)
    ms_b = _timed(bwd, steps)
    torch.cuda.synchronize()
    f_flops = float(np.sum(ns ** 3 / 3 + ns ** 2 / 2 + ns / 6 + 2 * ns ** 2))
    b_flops = float(np.sum(6 * ns ** 2))
    f_bytes = float(np.sum(8 * (ns * (ns + 1) // 2 * 2 + 2 * ns)))
    b_bytes = float(np.sum(8 * (ns * (ns + 1) // 2 + ns * ns + 4 * ns)))
    xg, gbg, gag = X.to_list(), GB.to_list(), GA.to_list()
    idx = _sample(count, 64)
    ex_o, ex_l, egb, ega = [], [], [], []
    for i in idx:
        a, b, t = A_h[i], b_h[i], t_h[i]
        Lo = np.zeros_like(a, order="F")
        orc.potrf(np.asfortranarray(a), Lo)
        xo = np.zeros_like(b, order="F")
        orc.potrs(Lo, np.asfortranarray(b), xo)
        cf, _ = lapack.dpotrf(a, lower=1, clean=1)
        x, _ = lapack.dpotrs(cf, b, lower=1)
        gb, _ = lapack.dpotrs(cf, x - t, lower=1)
        ga = -0.5 * (gb @ x.T + x @ gb.T)
        ex_o.append(_normwise(xg[i], xo))
        ex_l.append(_normwise(xg[i], x))
        egb.append(_normwise(gbg[i], gb))
        ega.append(_normwise(gag[i], ga))
    return {"workload": "differentiable SPD solve, 8,192 x n ~ U{32..128}, A = G G^T + n I, 1 RHS, seed 55",
            "forward_ms": ms_f, "backward_ms": ms_b, "steps": steps,
            "forward_matrices_per_s": count / ms_f * 1e3, "backward_matrices_per_s": count / ms_b * 1e3,
            "forward_roofline": _roofline(f_flops, f_bytes, ms_f, peak, "posv_cta_f64_kernel"),
            "backward_roofline": _roofline(b_flops, b_bytes, ms_b, peak, "posv_bwd_kernel"),
            "parity": {"n_checked": int(len(idx)),
                       "x_max_normwise_vs_oracle": max(ex_o), "x_max_normwise_vs_lapack": max(ex_l),
                       "dL_db_max_normwise_vs_cpu_fp64": max(egb), "dL_dA_max_normwise_vs_cpu_fp64": max(ega),
                       "reference_gradient": "db = A^-1 (x - t), dA = -(db x^T + x db^T)/2 with SciPy LAPACK "
                                             "dpotrf/dpotrs in binary64"}}


# ---------------------------------------------------------------------------------------------
# Riccati step (BLAST's syrk + potrf benchmark), opt-in
# ---------------------------------------------------------------------------------------------
def workload_riccati(args):
    """BLAST's Riccati kernel (bench/blas/SyrkPotrf.cpp): D = chol(C + A^T*A), A 30 x 60, C 60 x 60
    SPD, 50,000 instances; the fused kernel against the entry point's default, syrkLower followed
    by potrf (two launches)."""
    import numpy as np
    import torch

    import blast_gb300 as bg
    from oracle import oracle as orc

    batch, m, n = args.count or 50_000, 30, 60
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    At = bg.col_major((batch,), m, n, "cuda")  # A (m x n), used as op(A) = A^T through .mT
    At.copy_(torch.rand(batch, m, n, generator=g, device="cuda", dtype=torch.float64))
    A = At.mT
    Acol = bg.col_major((batch,), n, m, "cuda")
    Acol.copy_(A)
    G = torch.rand(batch, n, n, generator=g, device="cuda", dtype=torch.float64)
    C = bg.col_major((batch,), n, n, "cuda")
    C.copy_(G @ G.mT + n * torch.eye(n, device="cuda", dtype=torch.float64))
    del G
    D, S = bg.col_major((batch,), n, n, "cuda"), bg.col_major((batch,), n, n, "cuda")
    from blast_gb300 import _lib

    _lib.tune_set("syrk_potrf.fused_min_batch", 0)  # the fused kernel ...
    fused = _timed(lambda: bg.syrk_potrf(1.0, A, 1.0, C, D), args.steps)
    _lib.tune_set("syrk_potrf.fused_min_batch", 0x7FFFFFFF)  # ... and the entry point's default

    comp = _timed(lambda: bg.syrk_potrf(1.0, A, 1.0, C, S), args.steps)
    torch.cuda.synchronize()
    same = bool(torch.equal(torch.tril(D), torch.tril(S)))
    flops = n * (n + 1) * m + n ** 3 / 3 + n ** 2 / 2 + n / 6
    # CPU: the oracle's syrkLower then potrf, one instance per call, one thread
    hA, hC = Acol[:256].cpu().numpy(), C[:256].cpu().numpy()
    F = np.asfortranarray
    t0 = time.perf_counter()
    done = 0
    while time.perf_counter() - t0 < 2.0:
        for b in range(len(hA)):
            Sb = F(np.zeros((n, n)))
            orc.syrk_lower(1.0, F(hA[b]), 1.0, F(hC[b]), Sb)
            orc.potrf(Sb, Sb)
        done += len(hA)
    cpu = done / (time.perf_counter() - t0)
    return {"workload": f"syrk+potrf (Riccati) {batch} x D = chol(C + A^T A), A {m}x{n}",
            "fused_ms": fused, "fused_matrices_per_s": batch / fused * 1e3,
            "fused_tflops": flops * batch / fused / 1e9, "composed_ms": comp,
            "composed_matrices_per_s": batch / comp * 1e3, "bitwise_equal": same,
            "cpu_port_matrices_per_s_1thread": cpu}


# ---------------------------------------------------------------------------------------------
# The GPU arm
# ---------------------------------------------------------------------------------------------
def workload_posv_batches(args) -> dict:
    """Cholesky solves n = 48 with 8 right-hand sides (A = G G^T + 48 I, B ~ N(0,1)) at batch sizes
    from 500 to 50,000: the library's launch choice (one thread per matrix, or a quad of lanes per
    matrix for batches that hold fewer than 1.5 full warps per SM sub-partition) against the
    thread-per-matrix kernel alone ("posv.quad" = 0), with the two results compared bit for bit."""
    import numpy as np
    import torch

    import blast_gb300 as bg
    from blast_gb300 import _lib

    dev = torch.device("cuda", 0)
    key = "posv.quad.n64"
    default = _lib.tune_get(key)
    rows = []
    for batch in (500, 2_000, 8_000, 16_000, 24_000, 50_000):
        A_h, B_h = host_inputs(batch, SEED)
        A, B = _to_dev_batch(A_h, dev), _to_dev_batch(B_h, dev)
        L = bg.col_major((batch,), N, N, dev)
        X = bg.col_major((batch,), N, NRHS, dev)
        row = {"batch": batch}
        outs = {}
        for name, q in (("library", default), ("thread_kernel", 0)):
            if q is None:
                q = 150
            _lib.tune_set(key, q)
            row[f"{name}_ms"] = _timed(lambda: bg.posv(A, L, B, X), args.steps)
            outs[name] = (L.cpu().numpy(), X.cpu().numpy())
        _lib.tune_set(key, 150 if default is None else default)
        row["speedup"] = row["thread_kernel_ms"] / row["library_ms"]
        row["bit_identical"] = all(np.array_equal(a, b) for a, b in zip(outs["library"], outs["thread_kernel"]))
        rows.append(row)
        del A, B, L, X
    return {"workload": "posv n = 48, 8 RHS, batch 500 .. 50,000", "steps": args.steps, "rows": rows}


def _traffic_from_profile(batch: int):
    p = ROOT / "profiles" / "posv_thread_n48_traffic.json"
    try:
        t = json.loads(p.read_text())
    except (OSError, ValueError):
        return None, None
    if t.get("batch") != batch:
        return None, None
    return t.get("bytes_per_launch"), f"ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on the " \
                                      f"same batch ({p.relative_to(ROOT)}; not measured in this run)"


def run_ours(args):
    import numpy as np
    import torch

    import blast_gb300 as bg
    from blast_gb300 import _lib

    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    stream = torch.cuda.current_stream()

    BATCH = args.batch
    A_h, B_h = host_inputs(BATCH, SEED + rank)
    A, B = _to_dev_batch(A_h, dev), _to_dev_batch(B_h, dev)
    L = bg.col_major((BATCH,), N, N, dev)
    X = bg.col_major((BATCH,), N, NRHS, dev)

    def step():
        return bg.posv(A, L, B, X)

    for _ in range(max(args.warmup, 3)):
        info = step()
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = _lib.launch_count()
    barrier()
    with ClockSampler(local) as clocks:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    launches = _lib.launch_count() - launches0
    ms = e0.elapsed_time(e1) / args.steps
    if ws > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())

    parity = posv_parity(A_h, B_h, L, X) if rank == 0 and not args.no_parity else None

    if args.no_e2e:
        print(json.dumps({"ms_per_step": ms, "value": ws * BATCH / (ms * 1e-3), "batch": BATCH,
                          "parity": parity}))
        return

    # End to end through the public host-buffer API: pinned host A, B in, L, X (and info) back in
    # pinned host memory, every step. Each transport of PosvHostPipeline is timed (staged copies
    # over three streams; the kernel reading the host inputs directly with staged result copies;
    # one launch reading and writing host memory); the fastest is the e2e figure, the others are
    # reported beside it.
    from blast_gb300.host import PosvHostPipeline, pinned_col_major

    hA, hB = pinned_col_major(BATCH, N, N), pinned_col_major(BATCH, N, NRHS)
    hA.copy_(A)
    hB.copy_(B)
    hL, hX = pinned_col_major(BATCH, N, N), pinned_col_major(BATCH, N, NRHS)
    hinfo = torch.empty(BATCH, dtype=torch.int32, pin_memory=True)
    X_device_path = X.cpu()  # the device-timed solutions, to check every e2e output against
    del A, B, L, X
    torch.cuda.empty_cache()
    chunks = max(1, args.e2e_chunks)
    e2e_steps = max(3, min(args.steps, 12))
    depth = max(1, args.e2e_depth)
    # batches in flight together write to output buffers of their own
    outs = [(hL, hX, hinfo)] + [(pinned_col_major(BATCH, N, N), pinned_col_major(BATCH, N, NRHS),
                                 torch.empty(BATCH, dtype=torch.int32, pin_memory=True))
                                for _ in range(depth - 1)]
    e2e_runs = {}
    variants = [("copy", "copy", chunks, 1), ("direct", "direct", 1, 1), ("mirror", "mirror", 1, 1)]
    if depth > 1:
        variants.append((f"mirror_depth{depth}", "mirror", 1, depth))
    for name, transport, nchunks, dpt in variants:
        pipe = PosvHostPipeline(N, NRHS, (BATCH + nchunks - 1) // nchunks, dev, transport=transport, depth=dpt)
        for i in range(2 * dpt):
            pipe.run(hA, hB, *outs[i % dpt])
        pipe.wait()
        torch.cuda.synchronize()
        barrier()
        e0.record(stream)
        for i in range(e2e_steps):
            pipe.run(hA, hB, *outs[i % dpt])
        pipe.wait()
        e1.record(stream)
        torch.cuda.synchronize()
        t_ms = e0.elapsed_time(e1) / e2e_steps
        if ws > 1:
            t = torch.tensor([t_ms], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            t_ms = float(t.item())
        ok = all(int(outs[i][2].abs().sum()) == 0 and bool(torch.equal(outs[i][1], X_device_path))
                 for i in range(dpt))
        e2e_runs[name] = (t_ms, nchunks, dpt, ok)
        del pipe
        torch.cuda.empty_cache()
    best = min(e2e_runs, key=lambda k: e2e_runs[k][0])
    e2e_ms, e2e_chunks, e2e_depth, e2e_same = e2e_runs[best]
    del X_device_path
    # bytes that cross the host link per step: the mirror kernel reads only lower(A) and writes
    # only lower(L); the copy transports move whole matrices
    tri = N * (N + 1) // 2
    if best.startswith("mirror"):
        h2d = BATCH * (tri + N * NRHS) * 8
        d2h = BATCH * (tri + N * NRHS) * 8 + BATCH * 4
    elif best == "direct":
        h2d = BATCH * (tri + N * NRHS) * 8
        d2h = hL.numel() * 8 + hX.numel() * 8 + BATCH * 4
    else:
        h2d = hA.numel() * 8 + hB.numel() * 8
        d2h = hL.numel() * 8 + hX.numel() * 8 + BATCH * 4
    e2e_ok = all(int(o[2].abs().sum()) == 0 for o in outs)

    if rank != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return

    peak = peak_fp64_tflops()
    peak_dmma = peak_dmma_tflops()
    achieved = BATCH * FLOPS_PER / (ms * 1e-3) / 1e12
    traffic, traffic_src = _traffic_from_profile(BATCH)
    value = ws * BATCH / (ms * 1e-3)
    line = {
        "metric": METRIC, "value": value, "unit": "matrices/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded N(0,1), numpy default_rng(7 + rank) on the host, copied to the device)",
        "config": contract_config(BATCH),
        "setup": {"parallelism": f"replicas x{ws}",
                  "l2": f"inputs {BATCH * (N * N + N * NRHS) * 8 / 1e9:.2f} GB"
                        + (" > L2 (129 MB), no flush" if BATCH * (N * N + N * NRHS) * 8 > 129e6 else ", L2-resident")},
        "gflops": value * FLOPS_PER / 1e9,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None,
                     "traffic": traffic, "traffic_source": traffic_src,
                     "algorithmic_bytes": BATCH * BYTES_PER,
                     "peak_source": "binary64 FMA probe kernel run in this process (MEASURED_PEAKS.json has no FP64 figure)",
                     "peak_dmma_tflops": peak_dmma,
                     "kernel": "posv_thread_kernel"},
        "parity": parity,
        "e2e": {"value": ws * BATCH / (e2e_ms * 1e-3), "unit": "matrices/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms, "chunks": e2e_chunks, "depth": e2e_depth, "info_all_zero": e2e_ok,
                "x_bitwise_equal_to_device_path": e2e_same,
                "x_bitwise_equal_all_transports": all(v[3] for v in e2e_runs.values()),
                "path": f"blast_gb300.host.PosvHostPipeline(transport='{best.split('_')[0]}', depth={e2e_depth}), "
                        "pinned host buffers" + (f", {e2e_depth} batches in flight, each with its own output "
                                                 "buffers" if e2e_depth > 1 else ""),
                "other_transports": [{"transport": t, "ms_per_step": v[0], "chunks": v[1], "depth": v[2],
                                      "value": ws * BATCH / (v[0] * 1e-3)}
                                     for t, v in e2e_runs.items() if t != best]},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
    }
    hbm = _hbm_peak()
    gbs = BATCH * BYTES_PER / (ms * 1e-3) / 1e9
    line["roofline_hbm"] = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                            "frac": gbs / hbm if hbm else None}
    if ws == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(A_h, B_h)
    del A_h, B_h
    extra_steps = max(3, min(args.steps, 20))
    legs = []
    if not args.no_extra:
        legs += [("gemm24", lambda: config_gemm24(extra_steps, peak, cpu=not args.no_cpu)),
                 ("lu_ragged", lambda: config_lu_ragged(max(3, min(args.steps, 10)), peak, cpu=not args.no_cpu))]
    if not args.no_mixed:
        legs.append(("mixed_ir", lambda: mixed_ir_comparison(max(4, min(args.steps, 20)))))
    if not args.no_extra:
        legs.append(("adjoint", lambda: config_adjoint(extra_steps, peak)))
    for key, fn in legs:
        try:
            line[key] = fn()
        except Exception as exc:  # the contract line must still be printed
            line[key] = {"error": f"{type(exc).__name__}: {exc}"}
        torch.cuda.empty_cache()
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_mixed_only(args):
    """Only the FP64-vs-mixed comparison (profiling runs on a smaller ragged batch)."""
    import torch

    torch.cuda.set_device(0)
    if args.mixed_mode is not None:
        from blast_gb300 import _lib

        # the per-bin keys (set by the tuning cache) take precedence over the global one
        for key in ("posv.mixed", "posv.mixed.n64", "posv.mixed.n128", "posv.mixed.n256", "posv.mixed.n512"):
            _lib.tune_set(key, args.mixed_mode)
    print(json.dumps(mixed_ir_comparison(max(1, args.steps), args.mixed_count, args.mixed_gen,
                                         parity=not args.no_parity)), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline legs")
    ap.add_argument("--no-e2e", action="store_true",
                    help="device-timed leg only (small profiling runs); prints a reduced line")
    ap.add_argument("--no-parity", action="store_true", help="skip the parity checks")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the gemm, ragged LU and differentiable-solve workloads of the default line")
    ap.add_argument("--batch", type=int, default=BATCH, help="matrices per GPU (default 50,000)")
    ap.add_argument("--no-mixed", action="store_true",
                    help="skip the FP64-vs-mixed comparison on the ragged n in [64, 512] batch")
    ap.add_argument("--workload", choices=["cholesky48", "gemm24", "lu_ragged", "adjoint", "riccati", "posv_batches"],
                    default="cholesky48", help="cholesky48 (default) prints the contract line; the "
                    "others print one JSON object for that workload alone")
    ap.add_argument("--count", type=int, default=0,
                    help="instances for --workload lu_ragged / riccati (smaller for profiling)")
    ap.add_argument("--e2e-depth", type=int, default=3,
                    help="batches in flight for the pipelined mirror transport (1: not timed)")
    ap.add_argument("--e2e-chunks", type=int, default=3,
                    help="chunks of the staged-copy transport in the end-to-end leg")
    ap.add_argument("--only-mixed", action="store_true",
                    help="run only the FP64-vs-mixed comparison (with --mixed-count matrices)")
    ap.add_argument("--mixed-count", type=int, default=8192)
    ap.add_argument("--mixed-mode", type=int, choices=[0, 1, 2, 3], default=None,
                    help="mixed factorisation for --only-mixed: 0 binary32 CUDA cores, 1 tensor cores "
                         "(3xTF32), 2 tensor cores with binary64 diagonal blocks, 3 CUDA cores with "
                         "binary64 diagonal blocks (default: the library's)")
    ap.add_argument("--getrf-lazy", type=int, choices=[0, 1], default=None,
                    help="lu_ragged: right-looking (0) or left-looking (1) CTA LU in every size bin")
    ap.add_argument("--mixed-gen", choices=["qr", "gram"], default="qr",
                    help="qr: the workload's Q diag(lambda) Q^T matrices; gram: G G^T/n + I, for "
                         "profilers under which torch.linalg cannot load")
    args = ap.parse_args()
    if args.workload != "cholesky48":
        import torch

        torch.cuda.set_device(0)
        peak = None
        if args.workload == "gemm24":
            res = config_gemm24(args.steps, peak, cpu=not args.no_cpu)
        elif args.workload == "lu_ragged":
            if args.getrf_lazy is not None:
                from blast_gb300 import _lib

                for b in (8, 16, 32, 64, 128, 256, 512):
                    _lib.tune_set(f"getrf.lazy.n{b}", args.getrf_lazy)
            res = config_lu_ragged(args.steps, peak, count=args.count or 20_000, cpu=not args.no_cpu)
        elif args.workload == "adjoint":
            res = config_adjoint(args.steps, peak)
        elif args.workload == "posv_batches":
            res = workload_posv_batches(args)
        else:
            res = workload_riccati(args)
        print(json.dumps(res), flush=True)
    elif args.only_mixed:
        run_mixed_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

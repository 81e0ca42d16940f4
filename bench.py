"""Benchmark: batched FP64 Cholesky solve on GB300 (BLAST potrf + two trsm).

Workload (one "step"): 50,000 SPD matrices n = 48, A = G*G^T + 48*I with G i.i.d. N(0,1),
B (48 x 8) i.i.d. N(0,1); potrf(A, L) then L*Y = B, L^T*X = Y, all binary64, inputs resident in
HBM (1.07 GB of inputs, larger than the 129 MB L2, so no L2 flush is needed between steps).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line. `value` is matrices/s measured with CUDA events on the launching stream
(max over ranks); `e2e` is the same metric through the public API with pinned host buffers and
the host<->device copies inside the timed region; `roofline` is the binary64 issue bound of the
dominant kernel; `cpu_baseline` times the CPU restatement of BLAST's algorithm on this host.
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
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N, NRHS, BATCH = 48, 8, 50_000
FLOPS_PER = N ** 3 / 3 + N ** 2 / 2 + N / 6 + 2 * N * N * NRHS          # 74,888
BYTES_PER = 8 * (N * (N + 1) // 2 * 2 + 2 * N * NRHS)                     # 24,960 (lower A in, L out, B in, X out)
METRIC = "matrices/s, GFLOP/s on 1 GB300: FP64 vs mixed+IR batched potrf at 1e-12 bwd err"
WORKLOAD = "FP64 batched Cholesky solve: potrf + 2 trsm, 50,000 SPD n=48 (A = G*G^T + 48*I), B 48x8"


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


def make_inputs(batch: int, seed: int, device):
    """Seeded synthetic Cholesky-solve batch, generated on the device."""
    import torch

    import blast_gb300 as bg

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    G = torch.randn(batch, N, N, generator=g, device=device, dtype=torch.float64)
    A = bg.col_major((batch,), N, N, device)
    torch.baddbmm(torch.eye(N, device=device, dtype=torch.float64).mul_(N), G, G.mT, out=A.mT)
    del G
    B = bg.col_major((batch,), N, NRHS, device)
    B.copy_(torch.randn(batch, N, NRHS, generator=g, device=device, dtype=torch.float64))
    return A, B


def peak_fp64_tflops() -> float:
    """Binary64 FMA throughput of this GPU, measured by the library's probe kernel."""
    import ctypes

    import torch

    from blast_gb300 import _lib

    out = ctypes.c_double(0.0)
    _lib.call("blastgpu_probe_fp64_tflops", ctypes.byref(out), torch.cuda.current_stream().cuda_stream)
    return out.value


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


def mixed_ir_comparison(steps: int, count: int = 8192, gen: str = "qr"):
    """FP64 vs mixed-precision + refinement on the ragged n in [64, 512] batch (one CTA per
    matrix, one launch per step for each path)."""
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
    # backward error of the binary64 path, computed on the device
    be64 = []
    for i in range(0, count, max(1, count // 64)):
        a, b, x = A.view(i), B.view(i), X64.view(i)
        r = b - a @ x
        be64.append(float(r.abs().max() / (a.abs().sum(1).max() * x.abs().max() + b.abs().max())))
    out["mixed"].update({"max_backward_error": float(np.max(berr)),
                         "converged": int(np.sum((berr <= 1e-12) & (info == 0))),
                         "iterations_histogram": {int(k): int(v) for k, v in zip(*np.unique(iters, return_counts=True))},
                         "factorisation_breakdowns": int(np.sum(info != 0))})
    out["fp64"]["sampled_max_backward_error"] = float(np.max(be64))
    out["fp64"]["info_nonzero"] = int(np.sum(info64 != 0))
    out["speedup_matrices_per_s"] = out["mixed"]["matrices_per_s"] / out["fp64"]["matrices_per_s"]
    out["workload"] = (f"{count} SPD matrices, n ~ U{{64..512}}, A = Q diag(lambda) Q^T, "
                       "cond in {1e2,1e4,1e6}, 1 RHS; tol 1e-12" if gen == "qr" else
                       f"{count} SPD matrices, n ~ U{{64..512}}, A = G G^T/n + I (profiling)")
    return out


def load_traffic():
    p = ROOT / "profiles" / "posv_thread_n48_traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            return None
    return None


def _cpu_workload(sample: int):
    """The bench workload (n = 48, 8 RHS, A = G G^T + 48 I) as the oracle's column-major batch."""
    import numpy as np

    from oracle import oracle as orc

    rng = np.random.default_rng(7)
    G = rng.standard_normal((sample, N, N))
    A = G @ np.swapaxes(G, 1, 2) + N * np.eye(N)
    del G
    B = rng.standard_normal((sample, N, NRHS))
    return orc, orc.posv_prepare(A, B)


def cpu_baseline(min_seconds: float = 1.5, sample: int = BATCH):
    """The oracle's BLAST restatement on all of this host's cores: whole passes over the bench's
    50,000-matrix workload, repeated for at least min_seconds of wall time (16 threads x 1.5 s
    is about 24 s of CPU work)."""
    orc, prep = _cpu_workload(sample)
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
            "gflops": rate * FLOPS_PER / 1e9,
            "sample": f"{reps} passes over {sample} matrices of the workload (n=48, 8 RHS), one "
                      f"instance per call, OpenMP over {threads} threads, {el:.2f} s wall"}


def run_reference(args):
    """The reference arm: the oracle (BLAST's algorithm restated in C++, compiled -O3) on all host
    cores; a step is one pass over the same 50,000-matrix workload; W untimed steps, K timed."""
    ws, rank = _dist()
    if rank != 0:
        return
    orc, prep = _cpu_workload(BATCH)
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
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "batch_per_gpu": BATCH, "n": N, "nrhs": NRHS,
                       "parallelism": f"host cores of rank 0 ({threads} threads)"},
            "gflops": rate * FLOPS_PER / 1e9,
            "cpu_baseline": {"value": rate, "unit": "matrices/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} timed passes over {BATCH} matrices after "
                                       f"{max(1, args.warmup)} untimed, OpenMP over {threads} "
                                       f"threads, {el:.2f} s wall"},
            "e2e": {"value": rate, "unit": "matrices/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
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
    A, B = make_inputs(BATCH, 1234 + rank, dev)
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

    if args.no_e2e:
        print(json.dumps({"ms_per_step": ms, "value": ws * BATCH / (ms * 1e-3), "batch": BATCH}))
        return

    # End to end through the public host-buffer API: pinned host A, B in, L, X (and info) back in
    # pinned host memory, every step. Each transport of PosvHostPipeline is timed (staged copies
    # over three streams; the kernel reading the host inputs directly with staged result copies;
    # one launch writing the results to host memory too); the fastest is the e2e figure, the
    # others are reported beside it.
    from blast_gb300.host import PosvHostPipeline, pinned_col_major

    hA, hB = pinned_col_major(BATCH, N, N), pinned_col_major(BATCH, N, NRHS)
    hA.copy_(A)
    hB.copy_(B)
    hL, hX = pinned_col_major(BATCH, N, N), pinned_col_major(BATCH, N, NRHS)
    hinfo = torch.empty(BATCH, dtype=torch.int32, pin_memory=True)
    del A, B, L, X
    torch.cuda.empty_cache()
    chunks = max(1, args.e2e_chunks)
    e2e_steps = max(2, min(args.steps, 10))
    e2e_runs = {}
    for transport, nchunks in (("copy", chunks), ("direct", 1), ("mirror", 1)):
        pipe = PosvHostPipeline(N, NRHS, (BATCH + nchunks - 1) // nchunks, dev, transport=transport)
        for _ in range(2):
            pipe.run(hA, hB, hL, hX, hinfo)
        torch.cuda.synchronize()
        barrier()
        e0.record(stream)
        for _ in range(e2e_steps):
            pipe.run(hA, hB, hL, hX, hinfo)
        e1.record(stream)
        torch.cuda.synchronize()
        t_ms = e0.elapsed_time(e1) / e2e_steps
        if ws > 1:
            t = torch.tensor([t_ms], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            t_ms = float(t.item())
        e2e_runs[transport] = (t_ms, nchunks)
        del pipe
        torch.cuda.empty_cache()
    best = min(e2e_runs, key=lambda k: e2e_runs[k][0])
    e2e_ms, e2e_chunks = e2e_runs[best]

    if rank != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return

    peak = peak_fp64_tflops()
    achieved = BATCH * FLOPS_PER / (ms * 1e-3) / 1e12
    traffic = load_traffic()
    value = ws * BATCH / (ms * 1e-3)
    line = {
        "metric": METRIC, "value": value, "unit": "matrices/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded N(0,1), generated on device)",
        "config": {"workload": WORKLOAD, "batch_per_gpu": BATCH, "n": N, "nrhs": NRHS,
                   "parallelism": f"replicas x{ws}",
                   "l2": f"inputs {BATCH * (N * N + N * NRHS) * 8 / 1e9:.2f} GB"
                         + (" > L2 (129 MB), no flush" if BATCH * (N * N + N * NRHS) * 8 > 129e6 else ", L2-resident")},
        "gflops": value * FLOPS_PER / 1e9,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None,
                     # the capture's DRAM bytes hold for the captured batch only
                     "traffic": traffic.get("bytes_per_launch") if traffic and traffic.get("batch") == BATCH
                     else None,
                     "algorithmic_bytes": BATCH * BYTES_PER,
                     "peak_source": "binary64 FMA probe kernel run in this process (MEASURED_PEAKS.json has no FP64 figure)",
                     "kernel": "posv_thread_kernel"},
        "e2e": {"value": ws * BATCH / (e2e_ms * 1e-3), "unit": "matrices/s",
                "h2d_bytes_per_step": hA.numel() * 8 + hB.numel() * 8,
                "d2h_bytes_per_step": hL.numel() * 8 + hX.numel() * 8 + BATCH * 4,
                "ms_per_step": e2e_ms, "chunks": e2e_chunks,
                "path": f"blast_gb300.host.PosvHostPipeline(transport='{best}'), pinned host buffers",
                "other_transports": [{"transport": t, "ms_per_step": v[0], "chunks": v[1],
                                      "value": ws * BATCH / (v[0] * 1e-3)}
                                     for t, v in e2e_runs.items() if t != best]},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
    }
    hbm = None
    try:
        hbm = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("hbm_gbs")
    except (OSError, ValueError):
        pass
    gbs = BATCH * BYTES_PER / (ms * 1e-3) / 1e9
    line["roofline_hbm"] = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                            "frac": gbs / hbm if hbm else None}
    if ws == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline()
    if not args.no_mixed:
        try:
            line["mixed_ir"] = mixed_ir_comparison(max(4, min(args.steps, 20)))
        except Exception as exc:  # the contract line must still be printed
            line["mixed_ir"] = {"error": f"{type(exc).__name__}: {exc}"}
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def _timed(fn, steps, warm=2):
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


def workload_gemm24(args):
    """10,000 x (24x24x24) D = A*B + C, alpha = beta = 1, U[-1,1] (the gemm workload)."""
    import numpy as np
    import torch

    import blast_gb300 as bg
    from oracle import oracle as orc

    batch, m = 10_000, 24
    g = torch.Generator(device="cuda")
    g.manual_seed(99)
    A, B, C = (bg.col_major((batch,), m, m, "cuda") for _ in range(3))
    for t in (A, B, C):
        t.copy_(torch.rand(batch, m, m, generator=g, device="cuda", dtype=torch.float64) * 2 - 1)
    D = bg.col_major((batch,), m, m, "cuda")
    ms = _timed(lambda: bg.gemm(A, B, C, D), args.steps)
    flops = 2.0 * m ** 3 * batch
    # CPU: the oracle's restatement of BLAST's gemm, one instance per call, all host threads
    hA, hB, hC = (t.cpu().numpy() for t in (A, B, C))
    t0 = time.perf_counter()
    reps = 0
    while time.perf_counter() - t0 < 2.0:
        orc.gemm_batch(1.0, hA, hB, 1.0, hC)
        reps += 1
    cpu = reps * batch / (time.perf_counter() - t0)
    return {"workload": "gemm 10,000 x 24x24x24", "ms_per_step": ms, "matrices_per_s": batch / ms * 1e3,
            "tflops": flops / ms / 1e9, "cpu_port_matrices_per_s": cpu, "cpu_threads": orc.max_threads()}


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


def workload_lu_ragged(args):
    """20,000 general matrices, n log-uniform in [4, 256], N(0,1), one RHS: getrf + getrs."""
    import numpy as np
    import torch

    from blast_gb300.ragged import GesvPlan, Packed

    rng = np.random.default_rng(2020)
    count = args.count or 20_000
    ns = np.floor(np.exp(rng.uniform(np.log(4), np.log(257), count))).astype(np.int64)
    A = Packed(ns, ns, "cuda")
    B = Packed(ns, np.ones_like(ns), "cuda")
    g = torch.Generator(device="cuda")
    g.manual_seed(2020)
    A0 = torch.randn(A.buf.numel(), generator=g, device="cuda", dtype=torch.float64)
    B0 = torch.randn(B.buf.numel(), generator=g, device="cuda", dtype=torch.float64)
    plan = GesvPlan(A, B)

    def step():
        A.buf.copy_(A0)
        B.buf.copy_(B0)
        plan.run()

    ms_copy = _timed(lambda: (A.buf.copy_(A0), B.buf.copy_(B0)), args.steps)
    ms = _timed(step, args.steps) - ms_copy
    flops = float(np.sum(2 * ns ** 3 / 3 - ns ** 2 / 2 + 5 * ns / 6 + 2 * ns ** 2 - ns))
    return {"workload": "getrf+getrs ragged, 20,000 x n log-uniform [4,256]", "ms_per_step": ms,
            "matrices_per_s": count / ms * 1e3, "tflops": flops / ms / 1e9,
            "note": "time excludes re-copying the inputs (measured separately and subtracted)"}


def workload_adjoint(args):
    """8,192 SPD n ~ U{32..128} (A = G G^T + n I): forward solve and adjoint (factor kept)."""
    import numpy as np
    import torch

    from blast_gb300 import _lib, desc
    from blast_gb300.ragged import Packed, PosvPlan

    rng = np.random.default_rng(55)
    count = 8192
    ns = rng.integers(32, 129, count)
    A = Packed(ns, ns, "cuda")
    g = torch.Generator(device="cuda")
    g.manual_seed(55)
    for n in np.unique(ns):
        idx = np.nonzero(ns == n)[0]
        G = torch.randn(len(idx), n, n, generator=g, device="cuda", dtype=torch.float64)
        M = G @ G.mT + n * torch.eye(n, device="cuda", dtype=torch.float64)
        for j, i in enumerate(idx):
            A.view(int(i)).copy_(M[j])
    ones = np.ones_like(ns)
    B, X, T = Packed(ns, ones, "cuda"), Packed(ns, ones, "cuda"), Packed(ns, ones, "cuda")
    B.buf.copy_(torch.randn(B.buf.numel(), generator=g, device="cuda", dtype=torch.float64))
    T.buf.copy_(torch.randn(T.buf.numel(), generator=g, device="cuda", dtype=torch.float64))
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

    ms_f = _timed(fwd.run, args.steps)
    ms_b = _timed(bwd, args.steps)
    return {"workload": "differentiable SPD solve, 8,192 x n ~ U{32..128}, 1 RHS",
            "forward_ms": ms_f, "backward_ms": ms_b,
            "forward_matrices_per_s": count / ms_f * 1e3, "backward_matrices_per_s": count / ms_b * 1e3}


def run_mixed_only(args):
    """Only the FP64-vs-mixed comparison (profiling runs on a smaller ragged batch)."""
    import torch

    torch.cuda.set_device(0)
    print(json.dumps(mixed_ir_comparison(max(1, args.steps), args.mixed_count, args.mixed_gen)), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true",
                    help="device-timed leg only (small profiling runs); prints a reduced line")
    ap.add_argument("--batch", type=int, default=BATCH, help="matrices per GPU (default 50,000)")
    ap.add_argument("--no-mixed", action="store_true",
                    help="skip the FP64-vs-mixed comparison on the ragged n in [64, 512] batch")
    ap.add_argument("--workload", choices=["cholesky48", "gemm24", "lu_ragged", "adjoint", "riccati"],
                    default="cholesky48", help="cholesky48 (default) prints the contract line; the "
                    "others print one JSON object for that workload")
    ap.add_argument("--count", type=int, default=0,
                    help="instances for --workload lu_ragged (default 20,000; smaller for profiling)")
    ap.add_argument("--e2e-chunks", type=int, default=3,
                    help="chunks of the staged-copy transport in the end-to-end leg")
    ap.add_argument("--only-mixed", action="store_true",
                    help="run only the FP64-vs-mixed comparison (with --mixed-count matrices)")
    ap.add_argument("--mixed-count", type=int, default=8192)
    ap.add_argument("--mixed-gen", choices=["qr", "gram"], default="qr",
                    help="qr: the workload's Q diag(lambda) Q^T matrices; gram: G G^T/n + I, for "
                         "profilers under which torch.linalg cannot load")
    args = ap.parse_args()
    if args.workload != "cholesky48":
        import torch

        torch.cuda.set_device(0)
        fn = {"gemm24": workload_gemm24, "lu_ragged": workload_lu_ragged, "adjoint": workload_adjoint,
              "riccati": workload_riccati}
        print(json.dumps(fn[args.workload](args)), flush=True)
    elif args.only_mixed:
        run_mixed_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

"""Autotuner: per size bin, time the candidate kernel variants on this GPU and keep the fastest.

Tunable choices (read by the library through blastgpu_tune_set / tune_get_bin):

* ``posv.variant.n<bin>`` — thread-per-matrix Cholesky solve: CTA size and the register budget
  the kernel is compiled for (0: 64 threads, 213 registers; 1: 64 x 168; 2: 128 x 168;
  3: 32 x 168; 4: 32 x 168 with one column of load look-ahead in the tile updates).
* ``gemm.shape.m<8k>`` — warp tile of the batched gemm (0: 8x8, 1: 16x16, 2: 24x24, 3: 32x32),
  per largest dimension rounded up to a multiple of 8.
* ``getrf.cta.n<bin>`` — ragged LU: one warp (0) or one 256-thread CTA (1) per matrix, per size bin
  of the launch's largest n (same bits either way).
* ``getrf.lazy.n<bin>`` — the CTA kernel's schedule: right-looking (0) or left-looking with the left
  row swaps deferred (1); same bits either way.
* ``posv.mixed.n<bin>`` — ragged mixed-precision Cholesky factorisation per size bin (the modes of
  posv_cta_mixed_kernel); timed on the mixed workload's matrices (cond 1e2, 1e4, 1e6) and kept only
  if every instance converges.
* ``posv.cta_min_n`` — uniform Cholesky batches from this n on run one CTA per matrix instead of one
  thread per matrix.
* ``posv.warp.n<bin>`` — ragged binary64 Cholesky batches with every n <= 128: one warp (1) or one
  CTA (0) per matrix (same bits as the thread kernel, or within 10 n eps of it).
* ``posv.quad.n<bin>`` — uniform Cholesky batches (thread-per-matrix sizes) run a quad of lanes per
  matrix when they hold fewer than value / 100 full warps per SM sub-partition (same bits; not
  timed by this module: the library's defaults, 0 / 50 / 150 / 150 / 150 / 150 for the bins 8 to
  128, come from ``bench.py --workload posv_batches`` style measurements).

Results are cached as JSON keyed by GPU name (``blast_gb300/tuning/<gpu>.json``); ``apply()``
loads the cache for the current GPU into the library, and ``import blast_gb300`` calls it.
Cholesky bins are powers of two (the smallest power of two >= n, at least 8).
"""
from __future__ import annotations

import json
import re
from pathlib import Path

import torch

from . import _lib

CACHE_DIR = Path(__file__).resolve().parent / "tuning"


def size_bin(n: int) -> int:
    b = 8
    while b < n:
        b <<= 1
    return b


def _gpu_key() -> str:
    name = torch.cuda.get_device_name() if torch.cuda.is_available() else "none"
    return re.sub(r"[^A-Za-z0-9]+", "_", name).strip("_").lower()


def cache_path() -> Path:
    return CACHE_DIR / f"{_gpu_key()}.json"


def load() -> dict:
    p = cache_path()
    if p.exists():
        try:
            return json.loads(p.read_text()).get("choices", {})
        except ValueError:
            return {}
    return {}


def apply(choices: dict | None = None) -> dict:
    """Pushes cached (or given) choices into the library; returns them."""
    choices = load() if choices is None else choices
    for k, v in choices.items():
        _lib.tune_set(k, int(v))
    return choices


def _time(fn, reps=10) -> float:
    for _ in range(2):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def tune_posv(ns=(8, 16, 24, 32, 48, 64), nrhs=8, batch=50_000, variants=(0, 1, 2, 3, 4)) -> dict:
    from .blast import col_major, posv

    out = {}
    for n in ns:
        A = col_major((batch,), n, n, "cuda")
        G = torch.randn(batch, n, n, device="cuda", dtype=torch.float64)
        A.copy_(G @ G.mT + n * torch.eye(n, device="cuda", dtype=torch.float64))
        del G
        B = col_major((batch,), n, nrhs, "cuda")
        B.copy_(torch.randn(batch, n, nrhs, device="cuda", dtype=torch.float64))
        L, X = col_major((batch,), n, n, "cuda"), col_major((batch,), n, nrhs, "cuda")
        key = f"posv.variant.n{size_bin(n)}"
        times = {}
        for v in variants:
            _lib.tune_set(key, v)
            times[v] = _time(lambda: posv(A, L, B, X))
        out[key] = min(times, key=times.get)
        _lib.tune_set(key, out[key])
        del A, B, L, X
    return out


def tune_gemm(sizes=(8, 16, 24, 32, 40, 48, 56, 64), batch=10_000, shapes=(0, 1, 2, 3)) -> dict:
    from .blast import col_major, gemm

    out = {}
    for m in sizes:
        A, B, C, D = (col_major((batch,), m, m, "cuda") for _ in range(4))
        for t in (A, B, C):
            t.copy_(torch.rand(batch, m, m, device="cuda", dtype=torch.float64))
        key = f"gemm.shape.m{(m + 7) // 8 * 8}"
        times = {}
        for sh in shapes:
            _lib.tune_set(key, sh)
            times[sh] = _time(lambda: gemm(A, B, C, D))
        out[key] = min(times, key=times.get)
        _lib.tune_set(key, out[key])
    return out


def _log_uniform_sizes(rng, lo: int, hi: int, count: int):
    import numpy as np

    return np.clip(np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi + 1), count))).astype(np.int64), lo, hi)


def tune_getrf(bins=(8, 16, 32, 64, 128, 256), count: int = 4000) -> dict:
    """Warp-per-matrix LU, or CTA-per-matrix LU right- or left-looking, per size bin, on ragged
    batches with n log-uniform in the bin."""
    import numpy as np

    from .ragged import GesvPlan, Packed

    rng = np.random.default_rng(2)
    out = {}
    for b in bins:
        ns = _log_uniform_sizes(rng, max(1, b // 2 + 1), b, count)
        A = Packed(ns, ns, "cuda")
        B = Packed(ns, np.ones_like(ns), "cuda")
        A0 = torch.randn(A.buf.numel(), device="cuda", dtype=torch.float64)
        plan = GesvPlan(A, B)
        key = f"getrf.cta.n{size_bin(int(ns.max()))}"
        lazy_key = f"getrf.lazy.n{size_bin(int(ns.max()))}"
        times = {}
        for v in ((0, 0), (1, 0), (1, 1)):
            _lib.tune_set(key, v[0])
            _lib.tune_set(lazy_key, v[1])

            def step():
                A.buf.copy_(A0)
                _lib.call("blastgpu_dgetrf_batched", plan.d.data_ptr(), plan.info.data_ptr(), plan.count,
                          int(ns.max()), torch.cuda.current_stream().cuda_stream)

            times[v] = _time(step, reps=5)
        best = min(times, key=times.get)
        out[key], out[lazy_key] = best
        _lib.tune_set(key, best[0])
        _lib.tune_set(lazy_key, best[1])
    return out


def tune_posv_mixed(bins=(64, 128, 256, 512), count: int = 1536, modes=(0, 1, 2, 3)) -> dict:
    """Mixed-precision factorisation per size bin, on SPD matrices with n uniform in the bin and
    cond(A) in {1e2, 1e4, 1e6}; a mode counts only if every instance converges."""
    import numpy as np

    from .ragged import Packed, PosvPlan

    rng = np.random.default_rng(4)
    out = {}
    for b in bins:
        ns = rng.integers(max(1, b // 2 + 1), b + 1, count)
        A = Packed(ns, ns, "cuda")
        B = Packed(ns, np.ones_like(ns), "cuda")
        X = Packed(ns, np.ones_like(ns), "cuda")
        conds = np.array([1e2, 1e4, 1e6])[np.arange(count) % 3]
        for n in np.unique(ns):
            idx = np.nonzero(ns == n)[0]
            G = torch.randn(len(idx), int(n), int(n), device="cuda", dtype=torch.float64)
            Q, _ = torch.linalg.qr(G)
            lam = torch.stack([torch.logspace(0, -float(np.log10(conds[i])), int(n), device="cuda",
                                              dtype=torch.float64) for i in idx])
            M = (Q * lam[:, None, :]) @ Q.mT
            for j, i in enumerate(idx):
                A.view(int(i)).copy_(0.5 * (M[j] + M[j].T))
        B.buf.copy_(torch.randn(B.buf.numel(), device="cuda", dtype=torch.float64))
        plan = PosvPlan(A, B, X, mixed=True, tol=1e-12, max_iter=10)
        key = f"posv.mixed.n{size_bin(b)}"
        times = {}
        for mode in modes:
            _lib.tune_set(key, mode)
            t = _time(plan.run, reps=4)
            info, _, berr = plan.results()
            if not np.any(info) and np.all(berr <= 1e-12):
                times[mode] = t
        if times:
            out[key] = min(times, key=times.get)
            _lib.tune_set(key, out[key])
    return out


def tune_posv_cta_min_n(ns=(48, 56, 64, 72, 80, 96, 112, 128), nrhs=8, batch=20_000) -> dict:
    """The smallest n from which a uniform Cholesky solve stays faster one CTA per matrix."""
    from .blast import col_major, posv

    best = None
    for n in ns:
        A = col_major((batch,), n, n, "cuda")
        G = torch.randn(batch, n, n, device="cuda", dtype=torch.float64)
        A.copy_(G @ G.mT + n * torch.eye(n, device="cuda", dtype=torch.float64))
        del G
        B = col_major((batch,), n, nrhs, "cuda")
        B.copy_(torch.randn(batch, n, nrhs, device="cuda", dtype=torch.float64))
        L, X = col_major((batch,), n, n, "cuda"), col_major((batch,), n, nrhs, "cuda")
        _lib.tune_set("posv.cta_min_n", 1 << 20)
        t_thread = _time(lambda: posv(A, L, B, X), reps=5)
        _lib.tune_set("posv.cta_min_n", n)
        t_cta = _time(lambda: posv(A, L, B, X), reps=5)
        del A, B, L, X
        if t_cta < t_thread:
            best = n if best is None else best
        else:
            best = None  # the CTA kernels must stay ahead from the chosen n on
    value = best if best is not None else ns[-1] + 1
    _lib.tune_set("posv.cta_min_n", value)
    return {"posv.cta_min_n": int(value)}


def tune_posv_warp(bins=(32, 64, 128), count: int = 4096) -> dict:
    """Ragged binary64 Cholesky solves per size bin (n <= 128): one warp (1) or one CTA (0) per
    matrix, on SPD matrices with n uniform in the bin and one right-hand side."""
    import numpy as np

    from .ragged import Packed, PosvPlan

    rng = np.random.default_rng(6)
    out = {}
    for b in bins:
        ns = rng.integers(max(1, b // 2 + 1), b + 1, count)
        A = Packed(ns, ns, "cuda")
        A.fill_from([G @ G.T + n * np.eye(n) for G, n in ((rng.standard_normal((n, n)), n) for n in ns)])
        ones = np.ones_like(ns)
        B, X, L = Packed(ns, ones, "cuda"), Packed(ns, ones, "cuda"), Packed(ns, ns, "cuda")
        B.buf.normal_()
        plan = PosvPlan(A, B, X, L)
        key = f"posv.warp.n{size_bin(int(ns.max()))}"
        times = {}
        for v in (0, 1):
            _lib.tune_set(key, v)
            times[v] = _time(plan.run, reps=5)
        out[key] = min(times, key=times.get)
        _lib.tune_set(key, out[key])
    return out


def run(save: bool = True) -> dict:
    """Tunes every choice on the current GPU and (optionally) writes the cache."""
    choices = {}
    choices.update(tune_posv())
    choices.update(tune_gemm())
    choices.update(tune_getrf())
    choices.update(tune_posv_mixed())
    choices.update(tune_posv_cta_min_n())
    choices.update(tune_posv_warp())
    if save:
        CACHE_DIR.mkdir(parents=True, exist_ok=True)
        cache_path().write_text(json.dumps({"gpu": torch.cuda.get_device_name(),
                                            "choices": choices}, indent=1, sort_keys=True) + "\n")
    return choices


if __name__ == "__main__":
    print(json.dumps(run(), indent=1))

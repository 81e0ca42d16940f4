"""Autotuner: per size bin, time the candidate kernel variants on this GPU and keep the fastest.

Tunable choices (read by the library through blastgpu_tune_set / tune_get_bin):

* ``posv.variant.n<bin>`` — thread-per-matrix Cholesky solve: CTA size and the register budget
  the kernel is compiled for (0: 64 threads, 213 registers; 1: 64 x 168; 2: 128 x 168;
  3: 32 x 168).
* ``gemm.shape.m<8k>`` — warp tile of the batched gemm (0: 8x8, 1: 16x16, 2: 24x24, 3: 32x32),
  per largest dimension rounded up to a multiple of 8.

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


def tune_posv(ns=(8, 16, 24, 32, 48, 64), nrhs=8, batch=50_000, variants=(0, 1, 2, 3)) -> dict:
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


def run(save: bool = True) -> dict:
    """Tunes every choice on the current GPU and (optionally) writes the cache."""
    choices = {}
    choices.update(tune_posv())
    choices.update(tune_gemm())
    if save:
        CACHE_DIR.mkdir(parents=True, exist_ok=True)
        cache_path().write_text(json.dumps({"gpu": torch.cuda.get_device_name(),
                                            "choices": choices}, indent=1, sort_keys=True) + "\n")
    return choices


if __name__ == "__main__":
    print(json.dumps(run(), indent=1))

"""Shared helpers of the test-suite: seeded inputs, device transfers and BLAST's tolerances."""
from __future__ import annotations

import numpy as np

EPS = np.finfo(np.float64).eps

# BLAST's test tolerances (include/test/Tolerance.hpp:18-43; trsm/trmm/syrk use 1e-10).
ABS_TOL = 1e-11
REL_TOL = 1e-11


def approx_equal(a, b, abs_tol=ABS_TOL, rel_tol=REL_TOL) -> bool:
    """BLAST's elementwise check |a - b| <= abs_tol + rel_tol*|b| (include/test/Testing.hpp:58-83)."""
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and bool(np.all(np.abs(a - b) <= abs_tol + rel_tol * np.abs(b)))


def normwise(x, ref) -> float:
    x, ref = np.asarray(x), np.asarray(ref)
    den = np.linalg.norm(ref)
    return float(np.linalg.norm(x - ref) / (den if den > 0 else 1.0))


def spd(rng, n, shift=None):
    G = rng.standard_normal((n, n))
    return G @ G.T + (n if shift is None else shift) * np.eye(n)


def spd_batch(rng, batch, n):
    G = rng.standard_normal((batch, n, n))
    return G @ np.swapaxes(G, 1, 2) + n * np.eye(n)


def to_dev(h: np.ndarray, ld: int | None = None):
    """numpy (…, r, c) -> column-major float64 CUDA tensor (leading dimension ld)."""
    import torch

    from blast_gb300 import col_major

    r, c = h.shape[-2], h.shape[-1]
    t = col_major(h.shape[:-2], r, c, "cuda", ld)
    t.copy_(torch.from_numpy(np.ascontiguousarray(h)))
    return t

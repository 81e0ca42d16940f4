"""Generates the golden vectors in tests/golden/lapack_golden.npz.

BLAST ships no golden vectors (its tests regenerate random inputs and check reconstructions), and
BLAST itself cannot be built here, so these vectors come from an independent implementation of
the same operations: SciPy's bundled LAPACK/BLAS (dpotrf, dgetrf, dtrtrs, dgemm via numpy).
They pin the oracle: factors and solutions must agree to a normwise 10*n*eps, and getrf pivot
sequences must agree exactly (LAPACK's idamax also takes the first maximum, like BLAST's iamax,
dense/Iamax.hpp:82-95).

Run:  python tests/golden/make_golden.py
"""
from pathlib import Path

import numpy as np
import scipy
import scipy.linalg as sl

OUT = Path(__file__).resolve().parent / "lapack_golden.npz"


def main():
    rng = np.random.default_rng(20261203)
    data = {"scipy_version": np.array(scipy.__version__)}
    for n in (1, 2, 4, 5, 13, 24, 48):
        G = rng.standard_normal((n, n))
        A = G @ G.T + n * np.eye(n)
        L, info = sl.lapack.dpotrf(A, lower=1, clean=1)
        assert info == 0
        B = rng.standard_normal((n, 3))
        X, info = sl.lapack.dpotrs(L, B, lower=1)
        assert info == 0
        data[f"potrf_A_{n}"], data[f"potrf_L_{n}"] = A, L
        data[f"potrs_B_{n}"], data[f"potrs_X_{n}"] = B, X
    for n in (1, 3, 4, 5, 8, 9, 17, 33, 64):
        A = rng.standard_normal((n, n))
        lu, piv, info = sl.lapack.dgetrf(A)
        assert info == 0
        b = rng.standard_normal(n)
        x, info = sl.lapack.dgetrs(lu, piv, b)
        data[f"getrf_A_{n}"], data[f"getrf_LU_{n}"] = A, lu
        data[f"getrf_piv_{n}"] = piv.astype(np.int32)  # 0-based, as BLAST's ipiv
        data[f"getrs_b_{n}"], data[f"getrs_x_{n}"] = b, x
    for (m, n, k) in ((1, 1, 1), (3, 5, 7), (24, 24, 24), (20, 13, 9)):
        A = rng.uniform(-1, 1, (m, k))
        B = rng.uniform(-1, 1, (k, n))
        C = rng.uniform(-1, 1, (m, n))
        data[f"gemm_A_{m}_{n}_{k}"], data[f"gemm_B_{m}_{n}_{k}"] = A, B
        data[f"gemm_C_{m}_{n}_{k}"] = C
        data[f"gemm_D_{m}_{n}_{k}"] = 0.75 * (A @ B) - 0.5 * C
    for uplo in (0, 1):
        for unit in (0, 1):
            n = 17
            A = rng.standard_normal((n, n)) + n * np.eye(n)
            B = rng.standard_normal((n, 4))
            X, info = sl.lapack.dtrtrs(A, B, lower=1 - uplo, unitdiag=unit)
            data[f"trsm_A_{uplo}{unit}"], data[f"trsm_B_{uplo}{unit}"] = A, B
            data[f"trsm_X_{uplo}{unit}"] = X
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    main()

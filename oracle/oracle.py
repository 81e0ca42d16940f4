"""numpy binding of the CPU oracle (oracle/blast_oracle.h).

TEST INFRASTRUCTURE: imported only by tests/, the smoke check and the benchmark's CPU-baseline
leg. Matrices are numpy float64 arrays; column-major (Fortran-ordered) and row-major (C-ordered)
arrays are both accepted and described to the oracle by their strides.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libblast_oracle.so"


class oracle_mat(C.Structure):
    _fields_ = [("data", C.c_void_p), ("rows", C.c_int32), ("cols", C.c_int32), ("ld", C.c_int32),
                ("layout", C.c_int32), ("ps", C.c_int32), ("pad_", C.c_int32)]


_lib = None


def build() -> Path:
    res = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        h = C.CDLL(str(LIB_PATH))
        M, D, I, I64, P = oracle_mat, C.c_double, C.c_int, C.c_int64, C.c_void_p
        sig = {
            "oracle_dgemm": [D, M, M, D, M, M],
            "oracle_dgemm_naive": [D, M, M, D, M, M],
            "oracle_dsyrk_lower": [D, M, D, M, M],
            "oracle_dpotrf": [M, M],
            "oracle_dpotrf_panel": [M, M, I, I],
            "oracle_dgetrf": [M, P],
            "oracle_dgetf2": [M, P],
            "oracle_dlaswp": [M, I, I, P],
            "oracle_idamax": [I, P, I],
            "oracle_dger": [D, P, I, P, I, M, M],
            "oracle_dtrsm": [I, I, I, M, M, M],
            "oracle_dtrmm": [I, I, I, D, M, M, M],
            "oracle_dtrmm_any": [I, I, I, D, M, M, M],
            "oracle_dtrsm_right": [I, I, I, M, M, M],
            "oracle_dpotrs": [M, M, M],
            "oracle_dgetrs": [M, P, M, M],
            "oracle_dposv_batch": [I, I, I64, P, I64, P, P, I64, P, P, I],
            "oracle_dgemm_batch": [I, I, I, D, P, I64, P, I64, D, P, I64, P, I64, I64, I],
            "oracle_dgesv_ragged": [I64, P, P, P, P, P, P, P, P, I],
            "oracle_max_threads": [],
        }
        for name, args in sig.items():
            fn = getattr(h, name)
            fn.argtypes = args
            fn.restype = None if name == "oracle_dlaswp" else C.c_int
        _lib = h
    return _lib


def mat(a: np.ndarray) -> oracle_mat:
    """Describes a 2-D float64 numpy array (column- or row-major) to the oracle."""
    if a.dtype != np.float64 or a.ndim != 2:
        raise TypeError("float64 2-D array expected")
    r, c = a.shape
    if r == 0 or c == 0:
        return oracle_mat(a.ctypes.data, r, c, max(r, 1), 0, 0, 0)
    s0, s1 = (s // 8 for s in a.strides)
    if s0 == 1 and (s1 >= max(r, 1) or c <= 1):
        return oracle_mat(a.ctypes.data, r, c, max(s1, r, 1), 0, 0, 0)
    if s1 == 1 and (s0 >= max(c, 1) or r <= 1):
        return oracle_mat(a.ctypes.data, r, c, max(s0, c, 1), 1, 0, 0)
    raise ValueError(f"unsupported strides {a.strides}")


def panel_mat(buf: np.ndarray, rows: int, cols: int, ps: int, spacing: int) -> oracle_mat:
    return oracle_mat(buf.ctypes.data, rows, cols, spacing, 2, ps, 0)


def _check(st, name):
    if st < 0:
        raise ValueError(f"{name}: invalid argument ({st})")
    return st


def gemm(alpha, A, B, beta, C, D):
    return _check(lib().oracle_dgemm(alpha, mat(A), mat(B), beta, mat(C), mat(D)), "gemm")


def gemm_naive(alpha, A, B, beta, C, D):
    return _check(lib().oracle_dgemm_naive(alpha, mat(A), mat(B), beta, mat(C), mat(D)), "gemm_naive")


def syrk_lower(alpha, A, beta, C, D):
    return _check(lib().oracle_dsyrk_lower(alpha, mat(A), beta, mat(C), mat(D)), "syrk")


def potrf(A, L) -> int:
    return _check(lib().oracle_dpotrf(mat(A), mat(L)), "potrf")


def getrf(A, ipiv) -> int:
    assert ipiv.dtype == np.int32
    return _check(lib().oracle_dgetrf(mat(A), ipiv.ctypes.data), "getrf")


def getf2(A, ipiv) -> int:
    assert ipiv.dtype == np.int32
    return _check(lib().oracle_dgetf2(mat(A), ipiv.ctypes.data), "getf2")


def laswp(A, k0, k1, ipiv):
    lib().oracle_dlaswp(mat(A), k0, k1, ipiv.ctypes.data)


def idamax(x) -> int:
    x = np.ascontiguousarray(x, dtype=np.float64)
    return lib().oracle_idamax(len(x), x.ctypes.data, 1)


def ger(alpha, x, y, A, B):
    """B = A + alpha*x*y^T in place into B (blast::ger, dense/Ger.hpp:40-135)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    return _check(lib().oracle_dger(alpha, x.ctypes.data, 1, y.ctypes.data, 1, mat(A), mat(B)), "ger")


def swap(x, y):
    """blast::swap (dense/Swap.hpp:35-44): exchanges the contents of two vectors."""
    t = x.copy()
    x[...] = y
    y[...] = t


def trsm(uplo: int, unit: int, A, B, X, trans_a: int = 0):
    return _check(lib().oracle_dtrsm(uplo, unit, trans_a, mat(A), mat(B), mat(X)), "trsm")


def trmm(side: int, uplo: int, unit: int, alpha, A, B, Cm):
    return lib().oracle_dtrmm(side, uplo, unit, alpha, mat(A), mat(B), mat(Cm))


def trmm_any(side: int, uplo: int, unit: int, alpha, A, B, Cm):
    """Every (side, uplo, unit) trmm, the implemented variants' pattern (no reference algorithm)."""
    return _check(lib().oracle_dtrmm_any(side, uplo, unit, alpha, mat(A), mat(B), mat(Cm)), "trmm_any")


def trsm_right(uplo: int, unit: int, A, B, X, trans_a: int = 0):
    """X op(A) = B (no reference counterpart; see oracle_dtrsm_right)."""
    return _check(lib().oracle_dtrsm_right(uplo, unit, trans_a, mat(A), mat(B), mat(X)), "trsm_right")


def potrs(L, B, X):
    return _check(lib().oracle_dpotrs(mat(L), mat(B), mat(X)), "potrs")


def getrs(LU, ipiv, B, X):
    return _check(lib().oracle_dgetrs(mat(LU), ipiv.ctypes.data, mat(B), mat(X)), "getrs")


def max_threads() -> int:
    return lib().oracle_max_threads()


def posv_batch(A: np.ndarray, B: np.ndarray, threads: int = 0):
    """A: (batch, n, n) Fortran-ordered per matrix (A[b] column-major), B: (batch, n, nrhs).
    Returns (L, X, info)."""
    batch, n, _ = A.shape
    nrhs = B.shape[2]
    A = _batch_colmajor(A)
    B = _batch_colmajor(B)
    L = np.empty_like(A)
    X = np.empty_like(B)
    info = np.zeros(batch, dtype=np.int32)
    lib().oracle_dposv_batch(n, nrhs, batch, A.ctypes.data, n * n, L.ctypes.data, B.ctypes.data,
                             n * nrhs, X.ctypes.data, info.ctypes.data, threads)
    return _from_batch(L, n, n), _from_batch(X, n, nrhs), info


def posv_prepare(A: np.ndarray, B: np.ndarray) -> dict:
    """Column-major flat buffers for repeated timed runs of posv_run."""
    batch, n, _ = A.shape
    nrhs = B.shape[2]
    a, b = _batch_colmajor(A), _batch_colmajor(B)
    return {"n": n, "nrhs": nrhs, "batch": batch, "A": a, "B": b, "L": np.empty_like(a),
            "X": np.empty_like(b), "info": np.zeros(batch, dtype=np.int32)}


def posv_run(p: dict, threads: int = 0) -> None:
    n, nrhs = p["n"], p["nrhs"]
    lib().oracle_dposv_batch(n, nrhs, p["batch"], p["A"].ctypes.data, n * n, p["L"].ctypes.data,
                             p["B"].ctypes.data, n * nrhs, p["X"].ctypes.data,
                             p["info"].ctypes.data, threads)


def gemm_batch(alpha, A, B, beta, C, threads: int = 0):
    batch, m, k = A.shape
    n = B.shape[2]
    A, B, C = (_batch_colmajor(x) for x in (A, B, C))
    D = np.empty_like(C)
    lib().oracle_dgemm_batch(m, n, k, alpha, A.ctypes.data, m * k, B.ctypes.data, k * n, beta,
                             C.ctypes.data, m * n, D.ctypes.data, m * n, batch, threads)
    return _from_batch(D, m, n)


def gemm_prepare(alpha, A, B, beta, C) -> dict:
    """Column-major flat buffers of a uniform gemm batch for repeated timed runs of gemm_run."""
    batch, m, k = A.shape
    n = B.shape[2]
    a, b, c = (_batch_colmajor(x) for x in (A, B, C))
    return {"m": m, "n": n, "k": k, "alpha": alpha, "beta": beta, "batch": batch, "A": a, "B": b, "C": c,
            "D": np.empty_like(c)}


def gemm_run(p: dict, threads: int = 0) -> None:
    m, n, k = p["m"], p["n"], p["k"]
    lib().oracle_dgemm_batch(m, n, k, p["alpha"], p["A"].ctypes.data, m * k, p["B"].ctypes.data, k * n,
                             p["beta"], p["C"].ctypes.data, m * n, p["D"].ctypes.data, m * n, p["batch"],
                             threads)


def _batch_colmajor(x: np.ndarray) -> np.ndarray:
    """(batch, r, c) -> flat buffer holding each matrix column-major, contiguous per instance."""
    return np.ascontiguousarray(np.swapaxes(x, 1, 2)).reshape(-1)


def _from_batch(buf: np.ndarray, r: int, c: int) -> np.ndarray:
    return np.swapaxes(buf.reshape(-1, c, r), 1, 2)


def gesv_ragged(ns, A_list, b_list, threads: int = 0):
    """Ragged LU solve; A_list[i] (n_i x n_i), b_list[i] (n_i,). Returns (LU list, x list, ipiv
    list, info)."""
    batch = len(ns)
    ns = np.asarray(ns, dtype=np.int32)
    offA = np.zeros(batch, dtype=np.int64)
    offb = np.zeros(batch, dtype=np.int64)
    if batch:
        offA[1:] = np.cumsum(ns.astype(np.int64) ** 2)[:-1]
        offb[1:] = np.cumsum(ns.astype(np.int64))[:-1]
    Abuf = np.concatenate([np.asfortranarray(a).reshape(-1, order="F") for a in A_list]) if batch else np.zeros(0)
    bbuf = np.concatenate([np.asarray(b, dtype=np.float64) for b in b_list]) if batch else np.zeros(0)
    Abuf = np.ascontiguousarray(Abuf, dtype=np.float64)
    bbuf = np.ascontiguousarray(bbuf, dtype=np.float64)
    ipiv = np.zeros(int(ns.sum()) if batch else 0, dtype=np.int32)
    info = np.zeros(batch, dtype=np.int32)
    lib().oracle_dgesv_ragged(batch, ns.ctypes.data, offA.ctypes.data, Abuf.ctypes.data,
                              offb.ctypes.data, bbuf.ctypes.data, ipiv.ctypes.data, offb.ctypes.data,
                              info.ctypes.data, threads)
    LU = [Abuf[offA[i]:offA[i] + ns[i] ** 2].reshape(ns[i], ns[i], order="F") for i in range(batch)]
    xs = [bbuf[offb[i]:offb[i] + ns[i]] for i in range(batch)]
    pv = [ipiv[offb[i]:offb[i] + ns[i]] for i in range(batch)]
    return LU, xs, pv, info

"""ctypes binding of the blastgpu C ABI (include/blastgpu.h).

Loads the in-tree lib/libblastgpu.so. There is no fallback: if the library is missing, every call
raises, so a test or benchmark can never silently run something other than the CUDA kernels.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path

# The in-tree build; BLASTGPU_LIBRARY may name another build of the same ABI.
LIB_PATH = Path(os.environ.get("BLASTGPU_LIBRARY") or Path(__file__).resolve().parent / "lib" / "libblastgpu.so")

_lib = None
_lock = threading.Lock()


class BlastGpuError(RuntimeError):
    """A non-zero status returned by the C ABI."""

    def __init__(self, func: str, status: int, detail: str = ""):
        self.status = status
        msg = f"{func} returned {status}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


class blastgpu_mat(C.Structure):
    _fields_ = [("data", C.c_void_p), ("rows", C.c_int32), ("cols", C.c_int32), ("ld", C.c_int32),
                ("layout", C.c_int32), ("ps", C.c_int32), ("reserved", C.c_int32)]


class blastgpu_gemm_desc(C.Structure):
    _fields_ = [("A", blastgpu_mat), ("B", blastgpu_mat), ("C", blastgpu_mat), ("D", blastgpu_mat),
                ("alpha", C.c_double), ("beta", C.c_double)]


I32, I64, DBL, PTR = C.c_int, C.c_int64, C.c_double, C.c_void_p

NOALLOC_SCRATCH_BYTES = 32 << 20  # BLASTGPU_NOALLOC_SCRATCH_BYTES in include/blastgpu.h

# name -> argtypes (restype is int unless listed in _RESTYPES)
SIGNATURES: dict[str, list] = {
    "blastgpu_version": [],
    "blastgpu_status_string": [I32],
    "blastgpu_last_cuda_error": [],
    "blastgpu_launch_count": [],
    "blastgpu_selftest_recip": [I32, PTR, PTR, I32, PTR],
    "blastgpu_probe_fp64_tflops": [PTR, PTR],
    "blastgpu_probe_fp64_dmma_tflops": [PTR, PTR],
    "blastgpu_probe_mma_tflops": [I32, PTR, PTR],
    "blastgpu_tune_set": [C.c_char_p, I32],
    "blastgpu_tune_get": [C.c_char_p, PTR],
    "blastgpu_dgemm_strided": [I32, I32, I32, I32, I32, DBL, PTR, I32, I64, PTR, I32, I64, DBL,
                               PTR, I32, I64, PTR, I32, I64, I64, PTR],
    "blastgpu_dgemm_batched": [PTR, I64, I32, I32, I32, PTR],
    "blastgpu_dpotrf_strided": [I32, PTR, I32, I64, PTR, I32, I64, PTR, I64, PTR],
    "blastgpu_dposv_strided": [I32, I32, PTR, I32, I64, PTR, I32, I64, PTR, I32, I64, PTR, I32,
                               I64, PTR, I64, PTR],
    "blastgpu_dpotrs_strided": [I32, I32, PTR, I32, I64, PTR, I32, I64, PTR, I32, I64, I64, PTR],
    "blastgpu_dpotrf_batched": [PTR, I64, I32, I32, PTR, PTR],
    "blastgpu_dcopy_batched": [PTR, I64, PTR, PTR],
    "blastgpu_dposv_mirror_strided": [I32, I32, PTR, I32, I64, PTR, I32, I64, PTR, I32, I64, PTR, I32, I64,
                                      PTR, PTR, PTR, I64, PTR],
    "blastgpu_dsyrk_potrf_strided": [I32, I32, I32, DBL, PTR, I32, I64, DBL, PTR, I32, I64, PTR, I32, I64, PTR,
                                     I64, PTR],
    "blastgpu_dtrsm_right_strided": [I32, I32, I32, I32, I32, PTR, I32, I64, PTR, I32, I64, PTR, I32, I64, I64,
                                     PTR],
    "blastgpu_dger_strided": [I32, I32, DBL, PTR, I32, I64, PTR, I32, I64, PTR, I32, I64, PTR, I32, I64, I64, PTR],
    "blastgpu_idamax_strided": [I32, PTR, I32, I64, PTR, I64, PTR],
    "blastgpu_dlaswp_strided": [I32, PTR, I32, I64, I32, I32, PTR, I64, I64, PTR],
    "blastgpu_dswap_strided": [I32, PTR, I32, I64, PTR, I32, I64, I64, PTR],
    "blastgpu_dgetrf_strided": [I32, I32, PTR, I32, I64, PTR, I64, PTR, I64, PTR],
    "blastgpu_dgetrs_strided": [I32, I32, PTR, I32, I64, PTR, I64, PTR, I32, I64, PTR, I64, PTR],
    "blastgpu_dgetrf_batched": [PTR, PTR, I64, I32, PTR],
    "blastgpu_dgetrs_batched": [PTR, PTR, I64, I32, PTR],
    "blastgpu_dgesv_batched": [PTR, PTR, I64, I32, PTR],
    "blastgpu_dgesv_mixed_workspace_bytes": [I32],
    "blastgpu_dgesv_mixed_batched": [PTR, I64, I32, PTR, DBL, I32, PTR, PTR, PTR, PTR],
    "blastgpu_dposv_mixed_workspace_bytes": [I32],
    "blastgpu_dsyrk_lower_strided": [I32, I32, DBL, PTR, I32, I64, DBL, PTR, I32, I64, PTR, I32, I64, I64, PTR],
    "blastgpu_dgemm_bwd_strided": [I32, I32, I32, I32, I32, DBL, PTR, I32, I64, PTR, I32, I64, DBL, PTR, I32, I64,
                                   PTR, I32, I64, PTR, I32, I64, PTR, I32, I64, I64, PTR],
    "blastgpu_dtrsm_bwd_strided": [I32, I32, I32, I32, I32, PTR, I32, I64, PTR, I32, I64, PTR, I32, I64, PTR, I32,
                                   I64, PTR, I32, I64, I64, PTR],
    "blastgpu_dpotrf_bwd_strided": [I32, PTR, I32, I64, PTR, I32, I64, PTR, I32, I64, I64, PTR],
    "blastgpu_dtrsm_strided": [I32, I32, I32, I32, I32, PTR, I32, I64, PTR, I32, I64, PTR, I32, I64, I64, PTR],
    "blastgpu_dtrmm_strided": [I32, I32, I32, I32, I32, DBL, PTR, I32, I64, PTR, I32, I64, PTR, I32, I64, I64, PTR],
    "blastgpu_dposv_batched": [PTR, I64, I32, PTR, PTR],
    "blastgpu_dposv_mixed_batched": [PTR, I64, I32, PTR, DBL, I32, PTR, PTR, PTR, PTR],
    "blastgpu_dposv_bwd_batched": [PTR, I64, I32, I32, PTR, PTR],
    "blastgpu_dposv_mixed_batched_noalloc": [PTR, I64, I32, C.c_size_t, DBL, I32, PTR, PTR, PTR, PTR],
    "blastgpu_dpotrf_mn_strided": [I32, I32, PTR, I32, I64, PTR, I32, I64, PTR, I64, PTR],
    "blastgpu_dsyrk_lower_batched": [PTR, I64, PTR, PTR],
    "blastgpu_dtrsm_batched": [I32, I32, I32, PTR, I64, PTR, PTR],
    "blastgpu_dtrmm_batched": [I32, I32, I32, PTR, I64, PTR, PTR],
    "blastgpu_dger_batched": [PTR, I64, PTR, PTR],
    "blastgpu_idamax_batched": [PTR, I64, PTR, PTR],
    "blastgpu_dlaswp_batched": [PTR, I64, PTR, PTR],
    "blastgpu_dswap_batched": [PTR, I64, PTR, PTR],
    "blastgpu_dgemm_bwd_batched": [PTR, I64, I32, PTR, PTR],
    "blastgpu_dtrsm_bwd_batched": [I32, I32, PTR, I64, PTR, PTR],
    "blastgpu_dpotrf_bwd_batched": [PTR, I64, PTR, PTR],
}
_RESTYPES = {"blastgpu_status_string": C.c_char_p, "blastgpu_launch_count": C.c_int64,
             "blastgpu_dposv_mixed_workspace_bytes": C.c_size_t,
             "blastgpu_dgesv_mixed_workspace_bytes": C.c_size_t}


def lib() -> C.CDLL:
    """The loaded library (loads it on first use)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build the CUDA library first "
                    "(python -c 'import __graft_entry__ as g; g.build()')")
            h = C.CDLL(str(LIB_PATH))
            for name, args in SIGNATURES.items():
                fn = getattr(h, name)
                fn.argtypes = args
                fn.restype = _RESTYPES.get(name, C.c_int)
            _lib = h
    return _lib


def call(name: str, *args) -> int:
    """Calls a C ABI function and raises BlastGpuError on a non-zero status."""
    fn = getattr(lib(), name)
    st = fn(*args)
    if st != 0:
        detail = lib().blastgpu_status_string(st).decode()
        if st == -1002:
            detail += f", cudaError {lib().blastgpu_last_cuda_error()}"
        raise BlastGpuError(name, st, detail)
    return st


def tune_set(key: str, value: int) -> None:
    call("blastgpu_tune_set", key.encode(), int(value))


def tune_get(key: str):
    v = C.c_int(0)
    st = lib().blastgpu_tune_get(key.encode(), C.byref(v))
    return v.value if st == 0 else None


def launch_count() -> int:
    return int(lib().blastgpu_launch_count())

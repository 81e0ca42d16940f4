"""blast_gb300: batched GB300 (sm_103a) kernels for BLAST's small-matrix dense routines.

The product is the C ABI library lib/libblastgpu.so (include/blastgpu.h). This package holds its
build script, a ctypes binding, and ``blast``, a Python mirror of BLAST's function names over
torch device tensors.
"""
from . import _lib
from .blast import (LEFT, LOWER, RIGHT, UPPER, col_major, gemm, gemm_bwd, ger, getrf, getrs, iamax, laswp,
                    posv, potrf, potrf_bwd, potrs, swap, syrk_lower, syrk_potrf, trmm, trsm, trsm_bwd, trsm_right,
                    trsv_left_lower, trsv_left_upper)

__all__ = ["gemm", "potrf", "posv", "potrs", "getrf", "getrs", "syrk_lower", "syrk_potrf", "trsm", "trsm_right", "trmm", "ger",
           "iamax", "laswp", "swap", "trsv_left_lower", "trsv_left_upper", "gemm_bwd", "trsm_bwd", "potrf_bwd",
           "col_major", "LOWER", "UPPER", "LEFT", "RIGHT", "_lib"]


def _apply_tuning():
    """Loads the autotuner's cached per-bin choices for this GPU (blast_gb300/tuning/*.json)."""
    try:
        import torch

        if torch.cuda.is_available():
            from . import tune

            tune.apply()
    except (OSError, RuntimeError):
        pass  # no library or no cache yet: the built-in defaults apply


_apply_tuning()

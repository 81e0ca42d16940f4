"""Descriptor arrays for the ragged ("batched") entry points of the C ABI.

numpy structured dtypes with exactly the layout of blastgpu_mat / blastgpu_gemm_desc in
include/blastgpu.h, plus helpers that fill them from torch tensors and upload them.
"""
from __future__ import annotations

import numpy as np
import torch

MAT_DTYPE = np.dtype([("data", "<u8"), ("rows", "<i4"), ("cols", "<i4"), ("ld", "<i4"),
                      ("layout", "<i4"), ("ps", "<i4"), ("reserved", "<i4")], align=True)
assert MAT_DTYPE.itemsize == 32

GEMM_DTYPE = np.dtype([("A", MAT_DTYPE), ("B", MAT_DTYPE), ("C", MAT_DTYPE), ("D", MAT_DTYPE),
                       ("alpha", "<f8"), ("beta", "<f8")], align=True)
assert GEMM_DTYPE.itemsize == 144


GETRF_DTYPE = np.dtype([("A", MAT_DTYPE), ("ipiv", "<u8"), ("B", MAT_DTYPE)], align=True)
assert GETRF_DTYPE.itemsize == 72

GESV_MIXED_DTYPE = np.dtype([("A", MAT_DTYPE), ("ipiv", "<u8"), ("B", MAT_DTYPE), ("ws_offset", "<i8")],
                            align=True)
assert GESV_MIXED_DTYPE.itemsize == 80

POSV_DTYPE = np.dtype([("A", MAT_DTYPE), ("L", MAT_DTYPE), ("B", MAT_DTYPE), ("X", MAT_DTYPE),
                       ("ws_offset", "<i8")], align=True)
assert POSV_DTYPE.itemsize == 136

POSV_BWD_DTYPE = np.dtype([("A", MAT_DTYPE), ("L", MAT_DTYPE), ("X", MAT_DTYPE),
                           ("Xbar", MAT_DTYPE), ("Bbar", MAT_DTYPE), ("Abar", MAT_DTYPE)], align=True)
assert POSV_BWD_DTYPE.itemsize == 192

POTRF_DTYPE = np.dtype([("A", MAT_DTYPE), ("L", MAT_DTYPE)], align=True)
assert POTRF_DTYPE.itemsize == 64

COPY_DTYPE = np.dtype([("src", MAT_DTYPE), ("dst", MAT_DTYPE)], align=True)
assert COPY_DTYPE.itemsize == 64

SYRK_DTYPE = np.dtype([("A", MAT_DTYPE), ("C", MAT_DTYPE), ("D", MAT_DTYPE), ("alpha", "<f8"), ("beta", "<f8")],
                      align=True)
assert SYRK_DTYPE.itemsize == 112

TRSM_DTYPE = np.dtype([("A", MAT_DTYPE), ("B", MAT_DTYPE), ("X", MAT_DTYPE)], align=True)
assert TRSM_DTYPE.itemsize == 96

TRMM_DTYPE = np.dtype([("A", MAT_DTYPE), ("B", MAT_DTYPE), ("C", MAT_DTYPE), ("alpha", "<f8")], align=True)
assert TRMM_DTYPE.itemsize == 104

GER_DTYPE = np.dtype([("x", MAT_DTYPE), ("y", MAT_DTYPE), ("A", MAT_DTYPE), ("B", MAT_DTYPE), ("alpha", "<f8")],
                     align=True)
assert GER_DTYPE.itemsize == 136

LASWP_DTYPE = np.dtype([("A", MAT_DTYPE), ("ipiv", "<u8"), ("k0", "<i4"), ("k1", "<i4")], align=True)
assert LASWP_DTYPE.itemsize == 48

SWAP_DTYPE = np.dtype([("x", MAT_DTYPE), ("y", MAT_DTYPE)], align=True)
assert SWAP_DTYPE.itemsize == 64

GEMM_BWD_DTYPE = np.dtype([("A", MAT_DTYPE), ("B", MAT_DTYPE), ("Dbar", MAT_DTYPE), ("Abar", MAT_DTYPE),
                           ("Bbar", MAT_DTYPE), ("Cbar", MAT_DTYPE), ("alpha", "<f8"), ("beta", "<f8")], align=True)
assert GEMM_BWD_DTYPE.itemsize == 208

TRSM_BWD_DTYPE = np.dtype([("A", MAT_DTYPE), ("X", MAT_DTYPE), ("Xbar", MAT_DTYPE), ("Bbar", MAT_DTYPE),
                           ("Abar", MAT_DTYPE)], align=True)
assert TRSM_BWD_DTYPE.itemsize == 160

POTRF_BWD_DTYPE = np.dtype([("L", MAT_DTYPE), ("Lbar", MAT_DTYPE), ("Abar", MAT_DTYPE)], align=True)
assert POTRF_BWD_DTYPE.itemsize == 96

EMPTY_MAT = (0, 0, 0, 1, 0, 0, 0)


def mat_record(t: torch.Tensor) -> tuple:
    """(data, rows, cols, ld, layout, ps, reserved) for a 2-D float64 CUDA tensor view."""
    from .blast import _as_mat

    if t.dim() != 2:
        raise ValueError("descriptor entries are single matrices (2-D tensors)")
    m = _as_mat(t, "matrix")
    return (m.ptr, m.rows, m.cols, m.ld, m.layout, 0, 0)


def panel_record(buf: torch.Tensor, rows: int, cols: int, ps: int, spacing: int) -> tuple:
    """Descriptor of a panel-layout matrix stored in buf (element (i, j) at
    buf[(i // ps) * spacing + i % ps + j * ps])."""
    if buf.dtype != torch.float64 or not buf.is_cuda:
        raise TypeError("panel storage must be a float64 CUDA tensor")
    return (buf.data_ptr(), rows, cols, spacing, 2, ps, 0)


def upload(records: np.ndarray, device) -> torch.Tensor:
    """Copies a structured descriptor array to device memory (returns the owning uint8 tensor)."""
    raw = torch.from_numpy(records.view(np.uint8).copy())
    return raw.to(device)

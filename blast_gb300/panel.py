"""BLAST's panel storage on the GPU (panel/StaticPanelMatrix.hpp:165-184).

A column-major panel matrix with panel height ps stores rows in groups of ps ("panels"); inside a
panel the ps entries of each column are contiguous, and consecutive panels are `spacing` elements
apart (spacing = ps * cols for BLAST's own panel matrices). Element (i, j) is at
(i // ps) * spacing + i % ps + j * ps.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib, desc


class PanelBatch:
    """`count` panel matrices of shape (rows, cols), panel height ps, one buffer, instance b at
    b * stride elements."""

    def __init__(self, count: int, rows: int, cols: int, ps: int, device="cuda"):
        if ps not in (2, 4):
            raise ValueError("panel height must be 2 (NEON) or 4 (AVX2)")
        self.count, self.rows, self.cols, self.ps = count, rows, cols, ps
        self.spacing = ps * cols
        self.panels = (rows + ps - 1) // ps
        self.stride = self.panels * self.spacing
        self.buf = torch.zeros(max(count * self.stride, 1), dtype=torch.float64, device=device)

    def record(self, b: int) -> tuple:
        ptr = self.buf.data_ptr() + 8 * b * self.stride
        return (ptr, self.rows, self.cols, self.spacing, 2, self.ps, 0)

    def to_numpy(self) -> np.ndarray:
        """(count, rows, cols) dense copy computed on the host from the raw buffer."""
        raw = self.buf.cpu().numpy()[: self.count * self.stride].reshape(self.count, self.panels, self.cols, self.ps)
        dense = np.transpose(raw, (0, 1, 3, 2)).reshape(self.count, self.panels * self.ps, self.cols)
        return dense[:, : self.rows, :]


def copy(src_records: list, dst_records: list, device="cuda") -> torch.Tensor:
    """dst_b = src_b for each pair of blastgpu_mat records (any layouts); returns device status."""
    n = len(src_records)
    recs = np.zeros(n, dtype=desc.COPY_DTYPE)
    for b, (s, d) in enumerate(zip(src_records, dst_records)):
        recs[b] = (s, d)
    d_ = desc.upload(recs, device)
    status = torch.zeros(n, dtype=torch.int32, device=device)
    _lib.call("blastgpu_dcopy_batched", d_.data_ptr(), n, status.data_ptr(),
              torch.cuda.current_stream().cuda_stream)
    torch.cuda.current_stream().synchronize()
    return status


def from_dense(dense: torch.Tensor, ps: int) -> PanelBatch:
    """Panel copy of a (count, rows, cols) float64 CUDA tensor (column- or row-major per matrix)."""
    count, rows, cols = dense.shape
    pb = PanelBatch(count, rows, cols, ps, dense.device)
    copy([desc.mat_record(dense[b]) for b in range(count)], [pb.record(b) for b in range(count)], dense.device)
    return pb


def to_dense(pb: PanelBatch, out: torch.Tensor) -> torch.Tensor:
    copy([pb.record(b) for b in range(pb.count)], [desc.mat_record(out[b]) for b in range(pb.count)], out.device)
    return out


def potrf(A: PanelBatch, L: PanelBatch) -> torch.Tensor:
    """Panel Cholesky L := chol(A) (blast::potrf for panel matrices, panel/Potrf.hpp:59-106)."""
    if (A.count, A.rows, A.cols, A.ps) != (L.count, L.rows, L.cols, L.ps) or A.rows != A.cols:
        raise ValueError("Invalid matrix size")
    recs = np.zeros(A.count, dtype=desc.POTRF_DTYPE)
    for b in range(A.count):
        recs[b] = (A.record(b), L.record(b))
    d_ = desc.upload(recs, A.buf.device)
    info = torch.zeros(A.count, dtype=torch.int32, device=A.buf.device)
    _lib.call("blastgpu_dpotrf_batched", d_.data_ptr(), A.count, 2, A.ps, info.data_ptr(),
              torch.cuda.current_stream().cuda_stream)
    torch.cuda.current_stream().synchronize()
    return info

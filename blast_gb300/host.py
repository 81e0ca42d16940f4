"""Host-resident batches: the public entry for callers whose matrices live in (pinned) host memory,
as BLAST's do.

The batch is cut into chunks that flow through three CUDA streams, so that the host-to-device
copy of chunk i+1, the kernel on chunk i and the device-to-host copy of chunk i-1 overlap (the
GPU's copy engines run both directions concurrently with the SMs). Device buffers are allocated
once per pipeline and reused.
"""
from __future__ import annotations

import torch

from .blast import col_major, posv

_SLOTS = 3


class PosvHostPipeline:
    """Cholesky solves A_b X_b = B_b for host batches of shape (batch, n, n) and (batch, n, nrhs),
    column-major per matrix (a (batch, n, n) tensor whose .mT is contiguous, as made by
    col_major(..., device='cpu'))."""

    def __init__(self, n: int, nrhs: int, chunk: int, device=None):
        self.n, self.nrhs, self.chunk = n, nrhs, chunk
        self.device = torch.device(device or "cuda")
        self.streams = [torch.cuda.Stream(self.device) for _ in range(_SLOTS)]
        self.dA = [col_major((chunk,), n, n, self.device) for _ in range(_SLOTS)]
        self.dL = [col_major((chunk,), n, n, self.device) for _ in range(_SLOTS)]
        self.dB = [col_major((chunk,), n, nrhs, self.device) for _ in range(_SLOTS)]
        self.dX = [col_major((chunk,), n, nrhs, self.device) for _ in range(_SLOTS)]
        self.info = torch.zeros(0, dtype=torch.int32, device=self.device)

    def run(self, hA: torch.Tensor, hB: torch.Tensor, hL: torch.Tensor, hX: torch.Tensor,
            hinfo: torch.Tensor | None = None) -> torch.Tensor:
        """Enqueues the whole batch; returns the device info array (also copied to the pinned
        int32 host tensor hinfo when given). Host outputs are complete once
        torch.cuda.current_stream() has passed the point of return (it waits on the pipeline)."""
        batch = hA.shape[0]
        if self.info.numel() != batch:
            self.info = torch.zeros(batch, dtype=torch.int32, device=self.device)
        cur = torch.cuda.current_stream(self.device)
        start = torch.cuda.Event()
        start.record(cur)
        for s in self.streams:
            s.wait_event(start)
        for c, b0 in enumerate(range(0, batch, self.chunk)):
            b1 = min(batch, b0 + self.chunk)
            k = b1 - b0
            slot = c % _SLOTS
            s = self.streams[slot]
            with torch.cuda.stream(s):
                dA, dB = self.dA[slot][:k], self.dB[slot][:k]
                dL, dX = self.dL[slot][:k], self.dX[slot][:k]
                dA.mT.copy_(hA[b0:b1].mT, non_blocking=True)
                dB.mT.copy_(hB[b0:b1].mT, non_blocking=True)
                info = posv(dA, dL, dB, dX)
                self.info[b0:b1].copy_(info, non_blocking=True)
                if hinfo is not None:
                    hinfo[b0:b1].copy_(info, non_blocking=True)
                hL[b0:b1].mT.copy_(dL.mT, non_blocking=True)
                hX[b0:b1].mT.copy_(dX.mT, non_blocking=True)
        for s in self.streams:
            ev = torch.cuda.Event()
            ev.record(s)
            cur.wait_event(ev)
        return self.info


def pinned_col_major(batch: int, rows: int, cols: int) -> torch.Tensor:
    """A pinned host (batch, rows, cols) float64 tensor, column-major per matrix."""
    t = torch.empty((batch, cols, rows), dtype=torch.float64, pin_memory=True)
    return t.transpose(-1, -2)

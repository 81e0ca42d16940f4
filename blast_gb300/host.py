"""Host-resident batches: the public entry for callers whose matrices live in (pinned) host memory,
as BLAST's do. Three transports:

* ``"copy"``: the batch is cut into chunks that flow through three CUDA streams, so that the
  host-to-device copy of chunk i+1, the kernel on chunk i and the device-to-host copy of chunk i-1
  overlap (the GPU's copy engines run both directions concurrently with the SMs).
* ``"direct"``: the solve kernel reads A and B straight from the pinned host buffers (each element
  once, in the same tile order as from device memory), writes L and X to device slots, and the copy
  engines bring each chunk's results back while the next chunk computes. On GB300 the kernel's
  reads cross NVLink-C2C as it computes, so only the result direction is staged.
* ``"mirror"``: one launch (blastgpu_dposv_mirror_strided); the kernel reads the host inputs
  directly and each warp, once its 32 instances are solved, writes their L and X to the host
  buffers with whole-line stores, while other warps compute. With ``depth`` > 1, up to ``depth``
  batches are in flight at once, each on a stream and a device workspace of its own: the next
  batch's warps start reading their inputs over the host link while the previous batch's warps
  still compute, so the link and the binary64 pipes stay busy together (every warp of one launch
  asks for its next strip at about the same moment, which leaves the link idle while they compute).

Device buffers are allocated once per pipeline and reused.
"""
from __future__ import annotations

import torch

from . import _lib
from .blast import col_major, posv

_SLOTS = 3
TRANSPORTS = ("copy", "direct", "mirror")


def _check_host(n, r, hA, hB, hL, hX):
    for t, name, cols in ((hA, "A", n), (hB, "B", r), (hL, "L", n), (hX, "X", r)):
        if t.is_cuda or (t.numel() and not t.is_pinned()):
            raise ValueError(f"{name} must be a pinned host tensor for this transport")
        if t.dtype != torch.float64 or t.dim() != 3 or t.shape[1:] != (n, cols):
            raise ValueError(f"{name} must be float64 of shape (batch, {n}, {cols})")
        if t.numel() and (t.stride(1) != 1 or t.stride(2) != n or t.stride(0) != n * cols):
            raise ValueError(f"{name} must be column-major per matrix and packed (pinned_col_major)")


class PosvHostPipeline:
    """Cholesky solves A_b X_b = B_b for host batches of shape (batch, n, n) and (batch, n, nrhs),
    column-major per matrix (a (batch, n, n) tensor whose .mT is contiguous, as made by
    pinned_col_major)."""

    def __init__(self, n: int, nrhs: int, chunk: int, device=None, transport: str = "copy", depth: int = 1):
        if transport not in TRANSPORTS:
            raise ValueError(f"transport must be one of {TRANSPORTS}")
        if depth < 1 or (depth > 1 and transport != "mirror"):
            raise ValueError("depth > 1 needs the mirror transport")
        self.n, self.nrhs, self.chunk, self.transport, self.depth = n, nrhs, chunk, transport, depth
        self.device = torch.device(device or "cuda")
        self.info = torch.zeros(0, dtype=torch.int32, device=self.device)
        if transport == "mirror":
            self.work = [(torch.empty((chunk, n, n), dtype=torch.float64, device=self.device),
                          torch.empty((chunk, max(nrhs, 1), n), dtype=torch.float64, device=self.device))
                         for _ in range(depth)]
            self.slot_streams = [torch.cuda.Stream(self.device) for _ in range(depth)] if depth > 1 else []
            self.slot_info = [self.info] * depth
            self.next_slot = 0
            return
        self.streams = [torch.cuda.Stream(self.device) for _ in range(_SLOTS)]
        self.dL = [col_major((chunk,), n, n, self.device) for _ in range(_SLOTS)]
        self.dX = [col_major((chunk,), n, nrhs, self.device) for _ in range(_SLOTS)]
        if transport == "copy":
            self.dA = [col_major((chunk,), n, n, self.device) for _ in range(_SLOTS)]
            self.dB = [col_major((chunk,), n, nrhs, self.device) for _ in range(_SLOTS)]
        else:
            self.out_stream = torch.cuda.Stream(self.device)
            self.slot_free = [None] * _SLOTS

    def run(self, hA: torch.Tensor, hB: torch.Tensor, hL: torch.Tensor, hX: torch.Tensor,
            hinfo: torch.Tensor | None = None) -> torch.Tensor:
        """Enqueues the whole batch; returns the device info array (also copied to the pinned
        int32 host tensor hinfo when given). Host outputs are complete once
        torch.cuda.current_stream() has passed the point of return (it waits on the pipeline).

        With depth > 1 the batch runs on the next of the pipeline's own streams, after the work
        enqueued so far on the current stream, and the current stream does not wait for it: the
        outputs are complete once the current stream has passed a later wait(). Until then the
        batch's host buffers must stay untouched, and batches in flight together need output
        buffers (hL, hX, hinfo) of their own."""
        batch = hA.shape[0]
        if self.transport == "mirror" and self.depth > 1:
            slot = self.next_slot
            self.next_slot = (slot + 1) % self.depth
            stream = self.slot_streams[slot]
            ready = torch.cuda.Event()
            ready.record(torch.cuda.current_stream(self.device))
            stream.wait_event(ready)
            with torch.cuda.stream(stream):
                if self.slot_info[slot].numel() != batch:
                    self.slot_info[slot] = torch.zeros(batch, dtype=torch.int32, device=self.device)
                    self.slot_info[slot].record_stream(stream)
                return self._run_mirror(hA, hB, hL, hX, hinfo, slot)
        if self.info.numel() != batch:
            self.info = torch.zeros(batch, dtype=torch.int32, device=self.device)
        if self.transport == "mirror":
            self.slot_info[0] = self.info
            return self._run_mirror(hA, hB, hL, hX, hinfo, 0)
        if self.transport == "direct":
            return self._run_direct(hA, hB, hL, hX, hinfo)
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

    def _run_direct(self, hA, hB, hL, hX, hinfo):
        n, r = self.n, self.nrhs
        _check_host(n, r, hA, hB, hL, hX)
        batch = hA.shape[0]
        cur = torch.cuda.current_stream(self.device)
        out = self.out_stream
        start = torch.cuda.Event()
        start.record(cur)
        out.wait_event(start)
        for c, b0 in enumerate(range(0, batch, self.chunk)):
            b1 = min(batch, b0 + self.chunk)
            k = b1 - b0
            slot = c % _SLOTS
            if self.slot_free[slot] is not None:  # the slot's previous results have left the GPU
                cur.wait_event(self.slot_free[slot])
            dL, dX = self.dL[slot], self.dX[slot]
            _lib.call("blastgpu_dposv_strided", n, r, hA[b0].data_ptr(), n, n * n, dL.data_ptr(), n, n * n,
                      hB[b0].data_ptr() if r else 0, n, n * r, dX.data_ptr() if r else 0, n, n * r,
                      self.info[b0:].data_ptr(), k, cur.cuda_stream)
            done = torch.cuda.Event()
            done.record(cur)
            out.wait_event(done)
            with torch.cuda.stream(out):
                hL[b0:b1].mT.copy_(dL[:k].mT, non_blocking=True)
                hX[b0:b1].mT.copy_(dX[:k].mT, non_blocking=True)
                free = torch.cuda.Event()
                free.record(out)
            self.slot_free[slot] = free
        if hinfo is not None:
            hinfo.copy_(self.info, non_blocking=True)
        fin = torch.cuda.Event()
        fin.record(out)
        cur.wait_event(fin)
        return self.info

    def wait(self):
        """Makes the current stream wait for every batch in flight (depth > 1; nothing to do
        otherwise, since run() then enqueues on the current stream itself)."""
        cur = torch.cuda.current_stream(self.device)
        for s in getattr(self, "slot_streams", []):
            done = torch.cuda.Event()
            done.record(s)
            cur.wait_event(done)

    def _run_mirror(self, hA, hB, hL, hX, hinfo, slot):
        n, r = self.n, self.nrhs
        _check_host(n, r, hA, hB, hL, hX)
        batch = hA.shape[0]
        stream = torch.cuda.current_stream(self.device)
        wL, wX = self.work[slot]
        info = self.slot_info[slot]
        for b0 in range(0, batch, self.chunk):
            k = min(batch, b0 + self.chunk) - b0
            _lib.call("blastgpu_dposv_mirror_strided", n, r, hA[b0].data_ptr(), n, n * n,
                      hB[b0].data_ptr() if r else 0, n, n * r, hL[b0].data_ptr(), n, n * n,
                      hX[b0].data_ptr() if r else 0, n, n * r, wL.data_ptr(), wX.data_ptr(),
                      info[b0:].data_ptr(), k, stream.cuda_stream)
        if hinfo is not None:
            hinfo.copy_(info, non_blocking=True)
        return info


def pinned_col_major(batch: int, rows: int, cols: int) -> torch.Tensor:
    """A pinned host (batch, rows, cols) float64 tensor, column-major per matrix."""
    t = torch.empty((batch, cols, rows), dtype=torch.float64, pin_memory=True)
    return t.transpose(-1, -2)

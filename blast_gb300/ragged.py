"""Ragged batches: many matrices of different sizes packed in one device buffer, with the
descriptor arrays of the C ABI built once on the host (a "plan") and replayed on a stream.

A plan sorts its instances by decreasing size, so the CTA scheduler starts the longest
factorisations first (longest-processing-time-first ordering of the one launch).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib, desc


class Packed:
    """Column-major n_i x c_i matrices packed back to back (ld = n_i) in one float64 buffer."""

    def __init__(self, rows, cols, device, dtype=torch.float64):
        self.rows = np.asarray(rows, dtype=np.int64)
        self.cols = np.asarray(cols, dtype=np.int64)
        sizes = self.rows * self.cols
        self.offsets = np.zeros(len(sizes), dtype=np.int64)
        if len(sizes):
            self.offsets[1:] = np.cumsum(sizes)[:-1]
        total = int(sizes.sum()) if len(sizes) else 0
        self.buf = torch.zeros(max(total, 1), dtype=dtype, device=device)

    def __len__(self):
        return len(self.rows)

    def ptr(self, i) -> int:
        return self.buf.data_ptr() + int(self.offsets[i]) * self.buf.element_size()

    def view(self, i) -> torch.Tensor:
        """Column-major (rows, cols) view of instance i."""
        r, c, o = int(self.rows[i]), int(self.cols[i]), int(self.offsets[i])
        return self.buf[o:o + r * c].view(c, r).t()

    def record(self, i) -> tuple:
        r, c = int(self.rows[i]), int(self.cols[i])
        return (self.ptr(i), r, c, max(r, 1), 0, 0, 0)

    def fill_from(self, mats):
        """Copies host matrices (numpy, shapes (rows_i, cols_i)) into the buffer."""
        host = np.zeros(self.buf.numel())
        for i, m in enumerate(mats):
            o = int(self.offsets[i])
            host[o:o + m.size] = np.asarray(m, dtype=np.float64).reshape(-1, order="F")
        self.buf.copy_(torch.from_numpy(host))

    def to_list(self):
        host = self.buf.cpu().numpy()
        out = []
        for i in range(len(self)):
            r, c, o = int(self.rows[i]), int(self.cols[i]), int(self.offsets[i])
            out.append(host[o:o + r * c].reshape(c, r).T)
        return out


class PosvPlan:
    """Ragged batch of Cholesky solves A_i X_i = B_i, n_i <= 512.

    mixed=False: binary64 path (factor L_i written to `L`).
    mixed=True : binary32 factor (in an internal workspace) + binary64 refinement to `tol`.
    """

    def __init__(self, A: Packed, B: Packed, X: Packed, L: Packed | None = None, mixed=False,
                 tol=1e-12, max_iter=10):
        n = A.rows
        if np.any(A.cols != n) or np.any(B.rows != n) or np.any(X.rows != n) or np.any(X.cols != B.cols):
            raise ValueError("Invalid argument size")
        if not mixed and L is None:
            raise ValueError("the binary64 path needs L")
        self.count = len(n)
        self.max_n = int(n.max()) if self.count else 0
        if self.max_n > 512:
            raise ValueError("n > 512 is not supported by the ragged Cholesky kernels")
        self.mixed, self.tol, self.max_iter = mixed, float(tol), int(max_iter)
        device = A.buf.device
        self.order = np.argsort(-n, kind="stable")  # largest first
        recs = np.zeros(self.count, dtype=desc.POSV_DTYPE)
        ws_total = 0
        ws_off = np.zeros(self.count, dtype=np.int64)
        if mixed:
            per = np.array([_lib.lib().blastgpu_dposv_mixed_workspace_bytes(int(k)) for k in n], dtype=np.int64)
            ws_off[self.order] = np.concatenate([[0], np.cumsum(per[self.order])[:-1]]) if self.count else []
            ws_total = int(per.sum())
        self.workspace = torch.empty(max(ws_total, 256), dtype=torch.uint8, device=device) if mixed else None
        empty = desc.EMPTY_MAT
        for slot, i in enumerate(self.order):
            recs[slot] = (A.record(i), L.record(i) if L is not None else empty, B.record(i), X.record(i),
                          int(ws_off[i]))
        self.d = desc.upload(recs, device)
        self.info = torch.zeros(self.count, dtype=torch.int32, device=device)
        self.iters = torch.zeros(self.count, dtype=torch.int32, device=device)
        self.berr = torch.zeros(self.count, dtype=torch.float64, device=device)
        self._keep = (A, B, X, L)
        # Size bins (each launched with its own register tiling and shared-memory footprint, on
        # its own stream so that the bins overlap): contiguous slices of the sorted order.
        sorted_n = n[self.order]
        self.bins = []
        for lo, hi in ((257, 512), (129, 256), (65, 128), (0, 64)):
            idx = np.nonzero((sorted_n >= lo) & (sorted_n <= hi))[0]
            if len(idx):
                self.bins.append((int(idx[0]), int(idx[-1]) + 1, int(sorted_n[idx[0]])))
        self.streams = [torch.cuda.Stream(device) for _ in self.bins[1:]]

    def _launch(self, b0, b1, max_n, s):
        cnt = b1 - b0
        dptr = self.d.data_ptr() + b0 * desc.POSV_DTYPE.itemsize
        if self.mixed:
            _lib.call("blastgpu_dposv_mixed_batched", dptr, cnt, max_n, self.workspace.data_ptr(),
                      self.tol, self.max_iter, self.info.data_ptr() + 4 * b0,
                      self.iters.data_ptr() + 4 * b0, self.berr.data_ptr() + 8 * b0, s)
        else:
            _lib.call("blastgpu_dposv_batched", dptr, cnt, max_n, self.info.data_ptr() + 4 * b0, s)

    def run(self, stream=None):
        cur = stream or torch.cuda.current_stream()
        if not self.bins:
            return
        # the largest bin on the caller's stream, the others forked and joined back
        start = torch.cuda.Event()
        start.record(cur)
        for (b0, b1, mx), s in zip(self.bins[1:], self.streams):
            s.wait_event(start)
            self._launch(b0, b1, mx, s.cuda_stream)
        b0, b1, mx = self.bins[0]
        self._launch(b0, b1, mx, cur.cuda_stream)
        for s in self.streams:
            ev = torch.cuda.Event()
            ev.record(s)
            cur.wait_event(ev)

    def capture(self):
        """Records run() into a CUDA graph; returns the torch.cuda.CUDAGraph (call .replay())."""
        return capture_graph(self.run)

    def results(self):
        """(info, iters, berr) as numpy arrays in the caller's instance order."""
        inv = np.empty_like(self.order)
        inv[self.order] = np.arange(self.count)
        info = self.info.cpu().numpy()[inv]
        iters = self.iters.cpu().numpy()[inv]
        berr = self.berr.cpu().numpy()[inv]
        return info, iters, berr


def capture_graph(fn):
    """Captures the stream work of fn() (launches through the C ABI, which neither allocate nor
    synchronise) into a CUDA graph after one warm-up call."""
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        fn()
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        fn()
    return g


class MixedGesvPlan:
    """Ragged batch of mixed-precision LU solves (blastgpu_dgesv_mixed_batched): A_i (n_i x n_i,
    binary64, left untouched) rounded to binary32 and factored with partial pivoting, then
    X_i = A_i^{-1} B_i (written over B_i) refined in binary64 to a normwise backward error <= tol.
    n_i <= 256. Two size bins (n > 64: one CTA per factorisation; n <= 64: one warp) run on forked
    streams; the refinement is one warp per matrix."""

    def __init__(self, A: Packed, B: Packed, tol=1e-12, max_iter=10):
        n = A.rows
        if np.any(A.cols != n) or np.any(B.rows != n):
            raise ValueError("Invalid argument size")
        self.count = len(n)
        if self.count and int(n.max()) > 256:
            raise ValueError("n > 256 is not supported by the mixed-precision LU solve")
        self.tol, self.max_iter = float(tol), int(max_iter)
        device = A.buf.device
        self.order = np.argsort(-n, kind="stable")
        self.ipiv = Packed(n, np.ones_like(n), device, dtype=torch.int32)
        per = np.array([_lib.lib().blastgpu_dgesv_mixed_workspace_bytes(int(k)) for k in n], dtype=np.int64)
        ws_off = np.zeros(self.count, dtype=np.int64)
        if self.count:
            ws_off[self.order] = np.concatenate([[0], np.cumsum(per[self.order])[:-1]])
        self.workspace = torch.empty(max(int(per.sum()), 256), dtype=torch.uint8, device=device)
        recs = np.zeros(self.count, dtype=desc.GESV_MIXED_DTYPE)
        for slot, i in enumerate(self.order):
            recs[slot] = (A.record(i), self.ipiv.ptr(i), B.record(i), int(ws_off[i]))
        self.d = desc.upload(recs, device)
        self.info = torch.zeros(self.count, dtype=torch.int32, device=device)
        self.iters = torch.zeros(self.count, dtype=torch.int32, device=device)
        self.berr = torch.zeros(self.count, dtype=torch.float64, device=device)
        self._keep = (A, B)
        sorted_n = n[self.order]
        big = int(np.sum(sorted_n > 64))
        self.bins = [(b0, b1, int(sorted_n[b0])) for b0, b1 in ((0, big), (big, self.count)) if b1 > b0]
        self.side = torch.cuda.Stream(device)

    def _launch(self, b0, b1, max_n, s):
        _lib.call("blastgpu_dgesv_mixed_batched", self.d.data_ptr() + b0 * desc.GESV_MIXED_DTYPE.itemsize,
                  b1 - b0, max_n, self.workspace.data_ptr(), self.tol, self.max_iter,
                  self.info.data_ptr() + 4 * b0, self.iters.data_ptr() + 4 * b0, self.berr.data_ptr() + 8 * b0, s)

    def run(self, stream=None):
        cur = stream or torch.cuda.current_stream()
        if not self.bins:
            return
        if len(self.bins) == 2:
            start = torch.cuda.Event()
            start.record(cur)
            self.side.wait_event(start)
            self._launch(*self.bins[1], self.side.cuda_stream)
        self._launch(*self.bins[0], cur.cuda_stream)
        if len(self.bins) == 2:
            done = torch.cuda.Event()
            done.record(self.side)
            cur.wait_event(done)

    def capture(self):
        """Records run() into a CUDA graph; returns the torch.cuda.CUDAGraph (call .replay())."""
        return capture_graph(self.run)

    def pivots(self):
        host = self.ipiv.buf.cpu().numpy()
        return [host[int(o):int(o) + int(k)] for o, k in zip(self.ipiv.offsets, self.ipiv.rows)]

    def results(self):
        """(info, corrections, backward error) per instance, in the caller's order."""
        inv = np.empty_like(self.order)
        inv[self.order] = np.arange(self.count)
        return (self.info.cpu().numpy()[inv], self.iters.cpu().numpy()[inv], self.berr.cpu().numpy()[inv])


class GesvPlan:
    """Ragged batch of LU solves (getrf + getrs), column-major A_i (n_i x n_i), B_i (n_i x r_i)."""

    def __init__(self, A: Packed, B: Packed):
        n = A.rows
        if np.any(A.cols != n) or np.any(B.rows != n):
            raise ValueError("Invalid argument size")
        self.count = len(n)
        device = A.buf.device
        self.order = np.argsort(-n, kind="stable")
        self.ipiv = Packed(n, np.ones_like(n), device, dtype=torch.int32)
        recs = np.zeros(self.count, dtype=desc.GETRF_DTYPE)
        for slot, i in enumerate(self.order):
            recs[slot] = (A.record(i), self.ipiv.ptr(i), B.record(i))
        self.d = desc.upload(recs, device)
        self.info = torch.zeros(self.count, dtype=torch.int32, device=device)
        self._keep = (A, B)
        # Two size bins for the factorisation (one CTA per matrix above n = 64, one warp per
        # matrix below), on forked streams; the solves run as one launch afterwards.
        sorted_n = n[self.order]
        big = int(np.sum(sorted_n > 64))
        self.bins = [(b0, b1, int(sorted_n[b0])) for b0, b1 in ((0, big), (big, self.count)) if b1 > b0]
        self.side = torch.cuda.Stream(device)

    def _getrf(self, b0, b1, max_n, s):
        _lib.call("blastgpu_dgetrf_batched", self.d.data_ptr() + b0 * desc.GETRF_DTYPE.itemsize,
                  self.info.data_ptr() + 4 * b0, b1 - b0, max_n, s)

    def run(self, stream=None):
        cur = stream or torch.cuda.current_stream()
        if not self.bins:
            return
        if len(self.bins) == 2:
            start = torch.cuda.Event()
            start.record(cur)
            self.side.wait_event(start)
            self._getrf(*self.bins[1], self.side.cuda_stream)
        self._getrf(*self.bins[0], cur.cuda_stream)
        if len(self.bins) == 2:
            done = torch.cuda.Event()
            done.record(self.side)
            cur.wait_event(done)
        _lib.call("blastgpu_dgetrs_batched", self.d.data_ptr(), self.info.data_ptr(), self.count,
                  self.bins[0][2], cur.cuda_stream)

    def capture(self):
        """Records run() into a CUDA graph; returns the torch.cuda.CUDAGraph (call .replay())."""
        return capture_graph(self.run)

    def pivots(self):
        host = self.ipiv.buf.cpu().numpy()
        return [host[int(o):int(o) + int(k)] for o, k in zip(self.ipiv.offsets, self.ipiv.rows)]

    def info_host(self):
        inv = np.empty_like(self.order)
        inv[self.order] = np.arange(self.count)
        return self.info.cpu().numpy()[inv]

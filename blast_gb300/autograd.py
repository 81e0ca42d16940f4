"""torch.autograd shims over the batched operations and their hand-written adjoints: the Cholesky
solve (below), and gemm, trsm and potrf (at the end of this module).

x = A^{-1} b for SPD A (binary64). Forward: potrf + potrs on the GPU (blastgpu_dposv_* entry
points). Backward: blastgpu_dposv_bwd_batched, which returns dl/db = A^{-1} dl/dx and the
symmetrised dl/dA = -(dl/db x^T + x dl/db^T)/2. The factor L is either kept from the forward
pass (keep_factor=True) or recomputed inside the backward kernel (keep_factor=False), which saves
n^2 doubles per instance between the passes at the price of one more factorisation.

Only the lower triangle of A is read (as by blast::potrf); the gradient is the symmetric matrix
whose lower and upper parts together carry the derivative of the symmetric input.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib, desc
from .blast import LOWER, col_major, gemm, gemm_bwd, posv, potrf, potrf_bwd, trsm, trsm_bwd


def _colmajor_copy(t: torch.Tensor) -> torch.Tensor:
    out = col_major(t.shape[:-2], t.shape[-2], t.shape[-1], t.device)
    out.copy_(t)
    return out


def _bwd_call(records: np.ndarray, count: int, max_n: int, recompute: bool, device) -> torch.Tensor:
    d = desc.upload(records, device)
    info = torch.zeros(count, dtype=torch.int32, device=device)
    _lib.call("blastgpu_dposv_bwd_batched", d.data_ptr(), count, max_n, int(recompute),
              info.data_ptr(), torch.cuda.current_stream().cuda_stream)
    return info, d


class SPDSolve(torch.autograd.Function):
    """Uniform batch: A (batch, n, n) SPD, B (batch, n, nrhs) -> X (batch, n, nrhs)."""

    @staticmethod
    def forward(ctx, A, B, keep_factor=True):
        if A.dtype != torch.float64 or B.dtype != torch.float64:
            raise TypeError("binary64 tensors expected")
        Ac = _colmajor_copy(A)
        Bc = _colmajor_copy(B)
        batch, n = A.shape[0], A.shape[-1]
        L = col_major((batch,), n, n, A.device)
        X = col_major((batch,), n, B.shape[-1], A.device)
        info = posv(Ac, L, Bc, X)
        ctx.keep = keep_factor
        ctx.save_for_backward(Ac, L if keep_factor else torch.empty(0, device=A.device), X, info)
        return X.clone()

    @staticmethod
    def backward(ctx, Xbar):
        Ac, L, X, info = ctx.saved_tensors
        batch, n = Ac.shape[0], Ac.shape[-1]
        nrhs = X.shape[-1]
        dev = Ac.device
        G = _colmajor_copy(Xbar)
        GB = col_major((batch,), n, nrhs, dev)
        GA = col_major((batch,), n, n, dev)
        if not ctx.keep:
            L = col_major((batch,), n, n, dev)
        recs = np.zeros(batch, dtype=desc.POSV_BWD_DTYPE)
        for b in range(batch):
            recs[b] = (desc.mat_record(Ac[b]), desc.mat_record(L[b]), desc.mat_record(X[b]),
                       desc.mat_record(G[b]), desc.mat_record(GB[b]), desc.mat_record(GA[b]))
        info_b, _keep = _bwd_call(recs, batch, n, not ctx.keep, dev)
        torch.cuda.current_stream().synchronize()
        return GA.clone(), GB.clone(), None


def spd_solve(A: torch.Tensor, B: torch.Tensor, keep_factor: bool = True) -> torch.Tensor:
    """X = A^{-1} B, differentiable in A and B (binary64, CUDA)."""
    return SPDSolve.apply(A, B, keep_factor)


class PackedSPDSolve(torch.autograd.Function):
    """Ragged batch in packed buffers: A_flat holds the column-major n_i x n_i matrices back to
    back, B_flat the column-major n_i x r_i right-hand sides; returns X_flat (same packing as B)."""

    @staticmethod
    def forward(ctx, A_flat, B_flat, ns, rs, keep_factor=True):
        from .ragged import Packed, PosvPlan

        dev = A_flat.device
        A = Packed(ns, ns, dev)
        A.buf.copy_(A_flat.detach())
        B = Packed(ns, rs, dev)
        B.buf.copy_(B_flat.detach())
        X = Packed(ns, rs, dev)
        L = Packed(ns, ns, dev)
        plan = PosvPlan(A, B, X, L)
        plan.run()
        ctx.packs = (A, L if keep_factor else None, X)
        ctx.meta = (np.asarray(ns), np.asarray(rs), keep_factor)
        return X.buf.clone()

    @staticmethod
    def backward(ctx, Xbar_flat):
        from .ragged import Packed

        A, L, X = ctx.packs
        ns, rs, keep = ctx.meta
        dev = Xbar_flat.device
        G = Packed(ns, rs, dev)
        G.buf.copy_(Xbar_flat)
        GB = Packed(ns, rs, dev)
        GA = Packed(ns, ns, dev)
        if L is None:
            L = Packed(ns, ns, dev)
        count = len(ns)
        order = np.argsort(-ns, kind="stable")
        recs = np.zeros(count, dtype=desc.POSV_BWD_DTYPE)
        for slot, i in enumerate(order):
            recs[slot] = (A.record(i), L.record(i), X.record(i), G.record(i), GB.record(i), GA.record(i))
        _bwd_call(recs, count, int(ns.max()), not keep, dev)
        torch.cuda.current_stream().synchronize()
        return GA.buf.clone(), GB.buf.clone(), None, None, None


def spd_solve_packed(A_flat, B_flat, ns, rs, keep_factor: bool = True) -> torch.Tensor:
    return PackedSPDSolve.apply(A_flat, B_flat, ns, rs, keep_factor)


def _zeros_col(t: torch.Tensor) -> torch.Tensor:
    return col_major(t.shape[:-2], t.shape[-2], t.shape[-1], t.device).zero_()


class Gemm(torch.autograd.Function):
    """D = alpha*A*B + beta*C (blast.gemm); backward: blastgpu_dgemm_bwd_strided."""

    @staticmethod
    def forward(ctx, A, B, C, alpha=1.0, beta=1.0):
        Ac, Bc, Cc = _colmajor_copy(A), _colmajor_copy(B), _colmajor_copy(C)
        D = col_major(C.shape[:-2], C.shape[-2], C.shape[-1], C.device)
        gemm(float(alpha), Ac, Bc, float(beta), Cc, D)
        ctx.save_for_backward(Ac, Bc)
        ctx.alpha, ctx.beta = float(alpha), float(beta)
        return D.clone()

    @staticmethod
    def backward(ctx, Dbar):
        Ac, Bc = ctx.saved_tensors
        G = _colmajor_copy(Dbar)
        need = ctx.needs_input_grad
        GA = _zeros_col(Ac) if need[0] else None
        GB = _zeros_col(Bc) if need[1] else None
        GC = _zeros_col(G) if need[2] else None
        gemm_bwd(ctx.alpha, Ac, Bc, ctx.beta, G, GA, GB, GC)
        return GA, GB, GC, None, None


class Trsm(torch.autograd.Function):
    """X = A^{-1} B, A triangular (blast.trsm: uplo, unit diagonal); backward:
    blastgpu_dtrsm_bwd_strided. Entries of A outside its triangle (and a unit diagonal) are not
    read, and their gradient is zero."""

    @staticmethod
    def forward(ctx, A, B, uplo=LOWER, unit=False):
        Ac, Bc = _colmajor_copy(A), _colmajor_copy(B)
        X = col_major(B.shape[:-2], B.shape[-2], B.shape[-1], B.device)
        trsm(int(uplo), bool(unit), Ac, Bc, X)
        ctx.save_for_backward(Ac, X)
        ctx.uplo, ctx.unit = int(uplo), bool(unit)
        return X.clone()

    @staticmethod
    def backward(ctx, Xbar):
        Ac, X = ctx.saved_tensors
        G = _colmajor_copy(Xbar)
        GB = _zeros_col(X)
        GA = _zeros_col(Ac) if ctx.needs_input_grad[0] else None
        trsm_bwd(ctx.uplo, ctx.unit, Ac, X, G, GB, GA)
        return GA, GB if ctx.needs_input_grad[1] else None, None, None


class Potrf(torch.autograd.Function):
    """L = chol(A), lower, strictly upper part zero (blast.potrf reads the lower triangle of A);
    backward: blastgpu_dpotrf_bwd_strided, the symmetric dl/dA (as for the solve above)."""

    @staticmethod
    def forward(ctx, A):
        Ac = _colmajor_copy(A)
        L = _zeros_col(Ac)
        potrf(Ac, L)
        ctx.save_for_backward(L)
        return L.clone()

    @staticmethod
    def backward(ctx, Lbar):
        (L,) = ctx.saved_tensors
        G = _colmajor_copy(Lbar)
        GA = col_major(L.shape[:-2], L.shape[-2], L.shape[-1], L.device)
        potrf_bwd(L, G, GA)
        return GA.clone()


def gemm_fn(A, B, C, alpha=1.0, beta=1.0) -> torch.Tensor:
    """Differentiable D = alpha*A*B + beta*C (binary64, CUDA)."""
    return Gemm.apply(A, B, C, alpha, beta)


def trsm_fn(A, B, uplo=LOWER, unit=False) -> torch.Tensor:
    """Differentiable X = A^{-1} B for triangular A (binary64, CUDA)."""
    return Trsm.apply(A, B, uplo, unit)


def potrf_fn(A) -> torch.Tensor:
    """Differentiable lower Cholesky factor (binary64, CUDA)."""
    return Potrf.apply(A)

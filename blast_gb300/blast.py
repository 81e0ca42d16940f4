"""BLAST's hot-path API on batches of device matrices.

Each function keeps the name, argument order and meaning of its BLAST counterpart (cited per
function) and runs the sm_103a kernels of libblastgpu through the C ABI. A matrix is a float64
CUDA tensor of shape (rows, cols) (one instance, BLAST's own call) or (batch, rows, cols)
(a uniform batch). Storage is read from the strides:

* column-major (stride(-2) == 1): BLAST's default dense storage, leading dimension stride(-1);
* row-major (stride(-1) == 1): the storage of BLAST's ``trans()`` view of a column-major matrix,
  so ``A.mT`` of a column-major tensor is BLAST's ``trans(A)``.

Errors follow BLAST's: size mismatches raise ValueError (BLAST: std::invalid_argument "Matrix
sizes do not match"), variants BLAST does not implement raise NotImplementedError (BLAST:
std::logic_error). Calls are asynchronous on torch's current CUDA stream.
"""
from __future__ import annotations

from dataclasses import dataclass

import torch

from . import _lib

COL, ROW, PANEL = 0, 1, 2


@dataclass
class _Mat:
    ptr: int
    rows: int
    cols: int
    ld: int
    layout: int
    batch: int
    bstride: int


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def _as_mat(t: torch.Tensor, name: str) -> _Mat:
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor")
    if t.dtype != torch.float64:
        raise TypeError(f"{name} must be float64 (BLAST's double), got {t.dtype}")
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if t.dim() == 2:
        batch, bstride = 1, 0
    elif t.dim() == 3:
        batch, bstride = t.shape[0], t.stride(0)
    else:
        raise ValueError(f"{name} must have shape (rows, cols) or (batch, rows, cols)")
    rows, cols = t.shape[-2], t.shape[-1]
    s0, s1 = t.stride(-2), t.stride(-1)
    if s0 == 1 and (s1 >= max(rows, 1) or cols <= 1):
        layout, ld = COL, max(s1, rows, 1)
    elif s1 == 1 and (s0 >= max(cols, 1) or rows <= 1):
        layout, ld = ROW, max(s0, cols, 1)
    else:
        raise ValueError(f"{name} must be column-major or row-major per matrix (strides {t.stride()})")
    return _Mat(t.data_ptr(), rows, cols, ld, layout, batch, bstride)


def _batch_of(*mats: _Mat) -> int:
    batches = {m.batch for m in mats}
    if len(batches - {1}) > 1:
        raise ValueError("Batch sizes do not match")
    return max(batches)


def _bstride(m: _Mat, batch: int) -> int:
    return m.bstride if m.batch == batch else 0


def gemm(*args):
    """D = alpha*A*B + beta*C  (blast::gemm, algorithm/Gemm.hpp:80-97);
    gemm(A, B, C, D) is D = A*B + C (algorithm/Gemm.hpp:113-118).

    A and B may be column- or row-major (BLAST's trans() views); C and D are column-major.
    """
    if len(args) == 4:
        alpha, (A, B, C, D), beta = 1.0, args, 1.0
    elif len(args) == 6:
        alpha, A, B, beta, C, D = args
    else:
        raise TypeError("gemm(alpha, A, B, beta, C, D) or gemm(A, B, C, D)")
    a, b, c, d = (_as_mat(x, n) for x, n in ((A, "A"), (B, "B"), (C, "C"), (D, "D")))
    M, N, K = a.rows, b.cols, a.cols
    if b.rows != K or c.rows != M or c.cols != N or d.rows != M or d.cols != N:
        raise ValueError("Matrix sizes do not match")
    if c.layout != COL or d.layout != COL:
        raise NotImplementedError("C and D must be column-major (BLAST's tile() requires it)")
    batch = _batch_of(a, b, c, d)
    if d.batch != batch:
        raise ValueError("D must hold the whole batch")
    _lib.call("blastgpu_dgemm_strided", int(a.layout == ROW), int(b.layout == ROW), M, N, K,
              float(alpha), a.ptr, a.ld, _bstride(a, batch), b.ptr, b.ld, _bstride(b, batch),
              float(beta), c.ptr, c.ld, _bstride(c, batch), d.ptr, d.ld, d.bstride, batch, _stream())
    return D


def _square_col(m: _Mat, name: str):
    if m.layout != COL:
        raise NotImplementedError(f"{name} must be column-major")


def _info_tensor(batch: int, device) -> torch.Tensor:
    return torch.empty(batch, dtype=torch.int32, device=device)


def potrf(A: torch.Tensor, L: torch.Tensor) -> torch.Tensor:
    """Lower Cholesky factor: L := chol(A)  (blast::potrf, dense/Potrf.hpp:66-106).

    Reads the lower triangle of A; writes the lower triangle of L (L may be A). A may be an
    M x N trapezoid with M >= N, as in BLAST (the rows below the top N x N block are solved against
    its factor). Returns the per-instance info (0, or j+1 for the first non-positive pivot).
    """
    a, l = _as_mat(A, "A"), _as_mat(L, "L")
    if a.cols > a.rows:
        raise ValueError("Invalid matrix size")
    if l.rows != a.rows or l.cols != a.cols:
        raise ValueError("Invalid matrix size")
    _square_col(a, "A")
    _square_col(l, "L")
    batch = _batch_of(a, l)
    info = _info_tensor(batch, A.device)
    if a.rows == a.cols:
        _lib.call("blastgpu_dpotrf_strided", a.rows, a.ptr, a.ld, _bstride(a, batch), l.ptr, l.ld,
                  l.bstride, info.data_ptr(), batch, _stream())
    else:
        _lib.call("blastgpu_dpotrf_mn_strided", a.rows, a.cols, a.ptr, a.ld, _bstride(a, batch), l.ptr,
                  l.ld, l.bstride, info.data_ptr(), batch, _stream())
    return info


def posv(A: torch.Tensor, L: torch.Tensor, B: torch.Tensor, X: torch.Tensor) -> torch.Tensor:
    """Cholesky solve A*X = B: potrf(A, L), trsm<Lower>(L, B, X), trsm<Upper>(trans(L), X, X)
    (dense/Potrf.hpp:66-106, dense/Trsm.hpp:17-66), fused in one launch. Returns info."""
    a, l, b, x = (_as_mat(t, n) for t, n in ((A, "A"), (L, "L"), (B, "B"), (X, "X")))
    n = a.rows
    if a.cols != n or l.rows != n or l.cols != n or b.rows != n or x.rows != n or x.cols != b.cols:
        raise ValueError("Invalid argument size")
    for m, nm in ((a, "A"), (l, "L"), (b, "B"), (x, "X")):
        _square_col(m, nm)
    batch = _batch_of(a, l, b, x)
    info = _info_tensor(batch, A.device)
    _lib.call("blastgpu_dposv_strided", n, b.cols, a.ptr, a.ld, _bstride(a, batch), l.ptr, l.ld,
              l.bstride, b.ptr, b.ld, _bstride(b, batch), x.ptr, x.ld, x.bstride, info.data_ptr(),
              batch, _stream())
    return info


def potrs(L: torch.Tensor, B: torch.Tensor, X: torch.Tensor) -> torch.Tensor:
    """X := A^{-1} B from the Cholesky factor L: trsm<Lower>(L, B, X) then
    trsm<Upper>(trans(L), X, X) (dense/Trsm.hpp:17-66)."""
    l, b, x = (_as_mat(t, n) for t, n in ((L, "L"), (B, "B"), (X, "X")))
    n = l.rows
    if l.cols != n or b.rows != n or x.rows != n or x.cols != b.cols:
        raise ValueError("Invalid argument size")
    for m, nm in ((l, "L"), (b, "B"), (x, "X")):
        _square_col(m, nm)
    batch = _batch_of(l, b, x)
    _lib.call("blastgpu_dpotrs_strided", n, b.cols, l.ptr, l.ld, _bstride(l, batch), b.ptr, b.ld,
              _bstride(b, batch), x.ptr, x.ld, x.bstride, batch, _stream())
    return X


def _ipiv_check(ipiv: torch.Tensor, batch: int, k: int, name="ipiv"):
    if ipiv.dtype != torch.int32 or not ipiv.is_cuda:
        raise TypeError(f"{name} must be an int32 CUDA tensor")
    want = (k,) if batch == 1 and ipiv.dim() == 1 else (batch, k)
    if tuple(ipiv.shape) != want or ipiv.stride(-1) != 1:
        raise ValueError(f"{name} must have shape {want} and unit stride")


def getrf(A: torch.Tensor, ipiv: torch.Tensor) -> torch.Tensor:
    """LU with partial pivoting in place: A = P*L*U (blast::getrf, dense/Getrf.hpp:52-119).

    A: column-major (…, m, n); ipiv: int32 (…, min(m, n)) receiving 0-based pivot rows.
    Returns info (0, or k+1 for the first exactly-zero pivot; BLAST throws "Matrix is singular").
    """
    a = _as_mat(A, "A")
    if a.layout != COL:
        raise NotImplementedError("getrf needs column-major storage (BLAST's row-major overload "
                                  "does not pivot)")
    k = min(a.rows, a.cols)
    _ipiv_check(ipiv, a.batch, k)
    info = _info_tensor(a.batch, A.device)
    sp = ipiv.stride(0) if ipiv.dim() == 2 else 0
    _lib.call("blastgpu_dgetrf_strided", a.rows, a.cols, a.ptr, a.ld, a.bstride, ipiv.data_ptr(),
              sp, info.data_ptr(), a.batch, _stream())
    return info


def getrs(LU: torch.Tensor, ipiv: torch.Tensor, X: torch.Tensor, info: torch.Tensor | None = None):
    """X := A^{-1} X from getrf's factors: laswp, trsm<Lower, unit>, trsm<Upper>
    (dense/Laswp.hpp:37-43, dense/Trsm.hpp:17-66). Instances with info != 0 are skipped."""
    lu, x = _as_mat(LU, "LU"), _as_mat(X, "X")
    n = lu.rows
    if lu.cols != n or x.rows != n:
        raise ValueError("Invalid argument size")
    _square_col(lu, "LU")
    _square_col(x, "X")
    batch = _batch_of(lu, x)
    _ipiv_check(ipiv, lu.batch, n)
    sp = ipiv.stride(0) if ipiv.dim() == 2 else 0
    _lib.call("blastgpu_dgetrs_strided", n, x.cols, lu.ptr, lu.ld, _bstride(lu, batch),
              ipiv.data_ptr(), sp, x.ptr, x.ld, x.bstride,
              info.data_ptr() if info is not None else None, batch, _stream())
    return X


LOWER, UPPER = 0, 1
LEFT, RIGHT = 0, 1


def syrk_lower(alpha, A: torch.Tensor, beta, C: torch.Tensor, D: torch.Tensor) -> torch.Tensor:
    """D_lower = alpha*A*A^T + beta*C_lower (blast::syrkLower, dense/Syrk.hpp:15-145)."""
    a, c, d = _as_mat(A, "A"), _as_mat(C, "C"), _as_mat(D, "D")
    m, k = a.rows, a.cols
    if c.rows != m or c.cols != m or d.rows != m or d.cols != m:
        raise ValueError("Matrix sizes do not match")
    for x, nm in ((a, "A"), (c, "C"), (d, "D")):
        _square_col(x, nm)
    batch = _batch_of(a, c, d)
    _lib.call("blastgpu_dsyrk_lower_strided", m, k, float(alpha), a.ptr, a.ld, _bstride(a, batch),
              float(beta), c.ptr, c.ld, _bstride(c, batch), d.ptr, d.ld, d.bstride, batch, _stream())
    return D


def syrk_potrf(alpha, A: torch.Tensor, beta, C: torch.Tensor, D: torch.Tensor) -> torch.Tensor:
    """D = chol(beta*C + alpha*A*A^T), lower, fused (syrkLower then potrf: dense/Syrk.hpp:15-145,
    dense/Potrf.hpp:66-106; BLAST's Riccati benchmark bench/blas/SyrkPotrf.cpp:15-40).

    A is n x k, column-major, or a row-major tensor (BLAST's trans() view: op(A) = A^T of a k x n
    matrix). Reads the lower triangle of C; D may be C. Returns the per-instance info.
    """
    a, c, d = _as_mat(A, "A"), _as_mat(C, "C"), _as_mat(D, "D")
    n, k = a.rows, a.cols
    if c.rows != n or c.cols != n or d.rows != n or d.cols != n:
        raise ValueError("Matrix sizes do not match")
    _square_col(c, "C")
    _square_col(d, "D")
    batch = _batch_of(a, c, d)
    if d.batch != batch:
        raise ValueError("D must hold the whole batch")
    info = _info_tensor(batch, D.device)
    _lib.call("blastgpu_dsyrk_potrf_strided", n, k, int(a.layout == ROW), float(alpha), a.ptr, a.ld,
              _bstride(a, batch), float(beta), c.ptr, c.ld, _bstride(c, batch), d.ptr, d.ld, d.bstride,
              info.data_ptr(), batch, _stream())
    return info


def trsm(uplo: int, unit: bool, A: torch.Tensor, B: torch.Tensor, X: torch.Tensor) -> torch.Tensor:
    """Solve A*X = B, A triangular (blast::trsm<UpLo, UNIT>(A, B, X), dense/Trsm.hpp:17-66).

    A may be a row-major tensor (BLAST's trans() view of a column-major triangle); X may be B.
    """
    a, b, x = _as_mat(A, "A"), _as_mat(B, "B"), _as_mat(X, "X")
    m, n = b.rows, b.cols
    if a.rows != m or a.cols != m:
        raise ValueError("Invalid argument size")
    if x.rows != m or x.cols != n:
        raise ValueError("Invalid argument size")
    _square_col(b, "B")
    _square_col(x, "X")
    trans_a = int(a.layout == ROW)
    batch = _batch_of(a, b, x)
    _lib.call("blastgpu_dtrsm_strided", int(uplo), trans_a, int(bool(unit)), m, n, a.ptr, a.ld,
              _bstride(a, batch), b.ptr, b.ld, _bstride(b, batch), x.ptr, x.ld, x.bstride, batch, _stream())
    return X


def trmm(alpha, *args) -> torch.Tensor:
    """C = alpha*A*B: trmm(alpha, A, uplo, diag, B, C)  (algorithm/Trmm.hpp:260-283), or
    C = alpha*B*A: trmm(alpha, B, A, uplo, diag, C)  (algorithm/Trmm.hpp:287-310).
    BLAST implements A upper for the left product and A lower for the right one, non-unit only
    (std::logic_error otherwise); all (side, uplo, diag) combinations are computed here."""
    if len(args) != 5:
        raise TypeError("trmm(alpha, A, uplo, diag, B, C) or trmm(alpha, B, A, uplo, diag, C)")
    if isinstance(args[1], torch.Tensor):
        B, A, uplo, diag, C = args
        side = RIGHT
    else:
        A, uplo, diag, B, C = args
        side = LEFT
    a, b, c = _as_mat(A, "A"), _as_mat(B, "B"), _as_mat(C, "C")
    m, n = b.rows, b.cols
    ka = m if side == LEFT else n
    if a.rows != ka or a.cols != ka or c.rows != m or c.cols != n:
        raise ValueError("Matrix sizes do not match")
    for x, nm in ((a, "A"), (b, "B"), (c, "C")):
        _square_col(x, nm)
    batch = _batch_of(a, b, c)
    st = _lib.lib().blastgpu_dtrmm_strided(side, int(uplo), int(bool(diag)), m, n, float(alpha), a.ptr,
                                           a.ld, _bstride(a, batch), b.ptr, b.ld, _bstride(b, batch),
                                           c.ptr, c.ld, c.bstride, batch, _stream())
    if st != 0:
        raise _lib.BlastGpuError("blastgpu_dtrmm_strided", st)
    return C


def trsm_right(uplo: int, unit: bool, A: torch.Tensor, B: torch.Tensor, X: torch.Tensor) -> torch.Tensor:
    """Solve X*A = B, A triangular (no BLAST counterpart: RegisterMatrix::trsm leaves the right side
    unimplemented, register_matrix/RegisterMatrix.hpp:592-597). A may be a row-major tensor
    (transposed view); X may be B."""
    a, b, x = _as_mat(A, "A"), _as_mat(B, "B"), _as_mat(X, "X")
    m, n = b.rows, b.cols
    if a.rows != n or a.cols != n or x.rows != m or x.cols != n:
        raise ValueError("Invalid argument size")
    _square_col(b, "B")
    _square_col(x, "X")
    batch = _batch_of(a, b, x)
    _lib.call("blastgpu_dtrsm_right_strided", int(uplo), int(a.layout == ROW), int(bool(unit)), m, n, a.ptr,
              a.ld, _bstride(a, batch), b.ptr, b.ld, _bstride(b, batch), x.ptr, x.ld, x.bstride, batch,
              _stream())
    return X


def _out(t, name: str, rows: int, cols: int, layout: int, batch: int):
    """Pointer, ld and batch stride of an optional gradient output with the given shape and
    storage orientation, holding the whole batch."""
    if t is None:
        return 0, 1, 0
    o = _as_mat(t, name)
    if o.rows != rows or o.cols != cols:
        raise ValueError(f"{name} must have shape ({rows}, {cols})")
    if o.layout != layout:
        raise ValueError(f"{name} must have the storage order of its forward operand")
    if o.batch != batch or (batch > 1 and o.bstride == 0):
        raise ValueError(f"{name} must hold the whole batch")
    return o.ptr, o.ld, o.bstride


def gemm_bwd(alpha, A: torch.Tensor, B: torch.Tensor, beta, Dbar: torch.Tensor, Abar=None, Bbar=None,
             Cbar=None):
    """Adjoint of D = alpha*A*B + beta*C (gemm above): ACCUMULATES dl/dA into Abar, dl/dB into Bbar
    and dl/dC into Cbar (each optional; same shape and storage order as A, B and C; zero them
    first for plain gradients). A and B are the forward operands (row-major = BLAST's trans())."""
    a, b, db = _as_mat(A, "A"), _as_mat(B, "B"), _as_mat(Dbar, "Dbar")
    M, N, K = a.rows, b.cols, a.cols
    if b.rows != K or db.rows != M or db.cols != N:
        raise ValueError("Matrix sizes do not match")
    _square_col(db, "Dbar")
    batch = _batch_of(a, b, db)
    oa = _out(Abar, "Abar", M, K, a.layout, batch)
    ob = _out(Bbar, "Bbar", K, N, b.layout, batch)
    oc = _out(Cbar, "Cbar", M, N, COL, batch)
    _lib.call("blastgpu_dgemm_bwd_strided", int(a.layout == ROW), int(b.layout == ROW), M, N, K, float(alpha),
              a.ptr, a.ld, _bstride(a, batch), b.ptr, b.ld, _bstride(b, batch), float(beta), db.ptr, db.ld,
              _bstride(db, batch), *oa, *ob, *oc, batch, _stream())


def trsm_bwd(uplo: int, unit: bool, A: torch.Tensor, X: torch.Tensor, Xbar: torch.Tensor, Bbar: torch.Tensor,
             Abar=None) -> torch.Tensor:
    """Adjoint of trsm(uplo, unit, A, B, X) (A*X = B, uplo of A as passed; a row-major A is
    BLAST's trans() view): WRITES Bbar = A^{-T} Xbar (Bbar may be Xbar) and, if given,
    ACCUMULATES -Bbar X^T on A's triangle (strictly, when unit) into Abar (A's shape and order)."""
    a, x, xb = _as_mat(A, "A"), _as_mat(X, "X"), _as_mat(Xbar, "Xbar")
    bb = _as_mat(Bbar, "Bbar")
    m, n = x.rows, x.cols
    if a.rows != m or a.cols != m or xb.rows != m or xb.cols != n or bb.rows != m or bb.cols != n:
        raise ValueError("Invalid argument size")
    for t, nm in ((x, "X"), (xb, "Xbar"), (bb, "Bbar")):
        _square_col(t, nm)
    batch = _batch_of(a, x, xb, bb)
    if bb.batch != batch or (batch > 1 and bb.bstride == 0):
        raise ValueError("Bbar must hold the whole batch")
    oa = _out(Abar, "Abar", m, m, a.layout, batch)
    _lib.call("blastgpu_dtrsm_bwd_strided", int(uplo), int(a.layout == ROW), int(bool(unit)), m, n, a.ptr, a.ld,
              _bstride(a, batch), x.ptr, x.ld, _bstride(x, batch), xb.ptr, xb.ld, _bstride(xb, batch), bb.ptr, bb.ld,
              bb.bstride, *oa, batch, _stream())
    return Bbar


def potrf_bwd(L: torch.Tensor, Lbar: torch.Tensor, Abar: torch.Tensor) -> torch.Tensor:
    """Adjoint of L = chol(A) (potrf above): WRITES the symmetric dl/dA into Abar, in full, from L
    and Lbar = dl/dL (lower triangles read)."""
    lm, lb = _as_mat(L, "L"), _as_mat(Lbar, "Lbar")
    n = lm.rows
    if lm.cols != n or lb.rows != n or lb.cols != n:
        raise ValueError("Invalid argument size")
    _square_col(lm, "L")
    _square_col(lb, "Lbar")
    batch = _batch_of(lm, lb)
    oa = _out(Abar, "Abar", n, n, COL, batch)
    _lib.call("blastgpu_dpotrf_bwd_strided", n, lm.ptr, lm.ld, _bstride(lm, batch), lb.ptr, lb.ld,
              _bstride(lb, batch), *oa, batch, _stream())
    return Abar


def _vec(v: torch.Tensor, name: str):
    """(batch, n) or (n,) float64 CUDA tensor -> (ptr, n, inc, batch, batch stride)."""
    if v.dtype != torch.float64 or not v.is_cuda:
        raise TypeError(f"{name} must be a float64 CUDA tensor")
    if v.dim() == 1:
        return v.data_ptr(), v.shape[0], v.stride(0), 1, 0
    if v.dim() == 2:
        return v.data_ptr(), v.shape[1], v.stride(1), v.shape[0], v.stride(0)
    raise ValueError(f"{name} must have shape (n,) or (batch, n)")


def ger(alpha, x: torch.Tensor, y: torch.Tensor, A: torch.Tensor, B: torch.Tensor) -> torch.Tensor:
    """B = A + alpha*x*y^T (blast::ger, dense/Ger.hpp:40-135); B may be A."""
    xp, m, incx, bx, sx = _vec(x, "x")
    yp, n, incy, by, sy = _vec(y, "y")
    a, bm = _as_mat(A, "A"), _as_mat(B, "B")
    if a.rows != m or a.cols != n or bm.rows != m or bm.cols != n:
        raise ValueError("Matrix sizes do not match")
    _square_col(a, "A")
    _square_col(bm, "B")
    batch = max(bx, by, a.batch, bm.batch)
    for cnt in (bx, by, a.batch):
        if cnt not in (1, batch):
            raise ValueError("Batch sizes do not match")
    if bm.batch != batch:
        raise ValueError("B must hold the whole batch")
    _lib.call("blastgpu_dger_strided", m, n, float(alpha), xp, incx, sx if bx == batch else 0, yp, incy,
              sy if by == batch else 0, a.ptr, a.ld, _bstride(a, batch), bm.ptr, bm.ld, bm.bstride, batch,
              _stream())
    return B


def iamax(x: torch.Tensor) -> torch.Tensor:
    """First index of the largest |x_i| per vector (blast::iamax, dense/Iamax.hpp:66-96)."""
    xp, n, inc, batch, sx = _vec(x, "x")
    if n == 0:
        raise ValueError("Vector must be non-empty")
    out = torch.empty(batch, dtype=torch.int32, device=x.device)
    _lib.call("blastgpu_idamax_strided", n, xp, inc, sx, out.data_ptr(), batch, _stream())
    return out


def laswp(A: torch.Tensor, k0: int, k1: int, ipiv: torch.Tensor) -> torch.Tensor:
    """Row interchanges k = k0..k1-1 with ipiv (blast::laswp, dense/Laswp.hpp:37-43), in place."""
    a = _as_mat(A, "A")
    _square_col(a, "A")
    if ipiv.dtype != torch.int32 or not ipiv.is_cuda:
        raise TypeError("ipiv must be an int32 CUDA tensor")
    if ipiv.dim() == 2 and ipiv.shape[0] != a.batch:
        raise ValueError("Batch sizes do not match")
    if ipiv.shape[-1] < k1 or ipiv.stride(-1) != 1:
        raise ValueError("ipiv must be contiguous and hold k1 pivots")
    sp = ipiv.stride(0) if ipiv.dim() == 2 else 0
    _lib.call("blastgpu_dlaswp_strided", a.cols, a.ptr, a.ld, a.bstride, int(k0), int(k1), ipiv.data_ptr(),
              sp, a.batch, _stream())
    return A


def swap(x: torch.Tensor, y: torch.Tensor):
    """Exchange two vectors (blast::swap, dense/Swap.hpp:35-44)."""
    xp, n, incx, bx, sx = _vec(x, "x")
    yp, n2, incy, by, sy = _vec(y, "y")
    if n != n2 or bx != by:
        raise ValueError("Vector sizes must be equal")
    _lib.call("blastgpu_dswap_strided", n, xp, incx, sx, yp, incy, sy, bx, _stream())


def trsv_left_lower(A: torch.Tensor, b: torch.Tensor, x: torch.Tensor) -> torch.Tensor:
    """Solve A*x = b, A lower triangular (blast::trsvLeftLower, dense/Trsv.hpp:15-38)."""
    return trsm(LOWER, False, A, b.unsqueeze(-1), x.unsqueeze(-1)).squeeze(-1)


def trsv_left_upper(A: torch.Tensor, b: torch.Tensor, x: torch.Tensor) -> torch.Tensor:
    """Solve A*x = b, A upper triangular (blast::trsvLeftUpper, dense/Trsv.hpp:41-68)."""
    return trsm(UPPER, False, A, b.unsqueeze(-1), x.unsqueeze(-1)).squeeze(-1)


def col_major(batch_shape, rows: int, cols: int, device="cuda", ld: int | None = None) -> torch.Tensor:
    """An uninitialised column-major float64 tensor (…, rows, cols) with leading dimension ld."""
    ld = rows if ld is None else ld
    if ld < rows:
        raise ValueError("ld < rows")
    shape = tuple(batch_shape) + (cols, ld)
    t = torch.empty(shape, dtype=torch.float64, device=device)
    return t[..., :rows].transpose(-1, -2)

"""GPU parity of batched syrkLower, trsm and trmm against the oracle (bit for bit), over the
reference's own size sweeps (dense/SyrkTest.cpp, TrsmTest.cpp, TrmmTest.cpp)."""
import numpy as np
import pytest

from helpers import approx_equal, to_dev

pytestmark = pytest.mark.gpu


def F(a):
    return np.asfortranarray(a)


def test_syrk_lower_sweep_bitexact(gpu, oracle_lib):
    import torch

    rng = np.random.default_rng(1)
    for m in (1, 2, 5, 12, 13, 20, 33):
        for k in (1, 4, 20, 31):
            batch = 3
            A = rng.random((batch, m, k))
            C = rng.random((batch, m, m))
            C = C + np.swapaxes(C, 1, 2)
            alpha, beta = (1.0 if k % 2 == 0 else 0.75), -1.25  # alpha = 1 takes its own code path
            dA, dC = to_dev(A), to_dev(C)
            dD = to_dev(np.full((batch, m, m), 3.0))
            gpu.syrk_lower(alpha, dA, beta, dC, dD)
            torch.cuda.synchronize()
            D = dD.cpu().numpy()
            for b in range(batch):
                Dr = F(np.full((m, m), 3.0))
                oracle_lib.syrk_lower(alpha, F(A[b]), beta, F(C[b]), Dr)
                assert np.array_equal(D[b], Dr), (m, k)  # upper triangle untouched too


@pytest.mark.parametrize("uplo,unit", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_trsm_sweep_bitexact(gpu, oracle_lib, uplo, unit):
    import torch

    rng = np.random.default_rng(10 + 2 * uplo + unit)
    for m in (1, 4, 9, 17, 50):
        for n in (1, 3, 8, 50):
            batch = 4
            A = rng.random((batch, m, m)) + np.eye(m)
            B = rng.random((batch, m, n))
            dA, dB = to_dev(A), to_dev(B)
            dX = gpu.col_major((batch,), m, n, "cuda")
            gpu.trsm(uplo, unit, dA, dB, dX)
            gpu.trsm(uplo, unit, dA, dB, dB)  # X aliasing B
            torch.cuda.synchronize()
            X, Xa = dX.cpu().numpy(), dB.cpu().numpy()
            for b in range(batch):
                Xr = F(np.zeros((m, n)))
                oracle_lib.trsm(uplo, unit, F(A[b]), F(B[b]), Xr)
                assert np.array_equal(X[b], Xr), (m, n)
                assert np.array_equal(Xa[b], Xr), (m, n)
                At = np.tril(A[b]) if uplo == 0 else np.triu(A[b])
                if unit:
                    np.fill_diagonal(At, 1.0)
                assert approx_equal(At @ X[b], B[b], 1e-10, 1e-10)


def test_trsm_transposed_view(gpu, oracle_lib):
    """trsm<Upper>(trans(L), Y, X): A given as a row-major tensor (BLAST's trans() view)."""
    import torch

    rng = np.random.default_rng(4)
    m, n, batch = 23, 5, 3
    Lh = np.tril(rng.random((batch, m, m))) + np.eye(m)
    Y = rng.random((batch, m, n))
    dL = to_dev(Lh)
    dX = to_dev(Y)
    gpu.trsm(1, 0, dL.mT, dX, dX)
    torch.cuda.synchronize()
    X = dX.cpu().numpy()
    for b in range(batch):
        Xr = F(Y[b].copy())
        oracle_lib.trsm(1, 0, F(Lh[b]), Xr, Xr, trans_a=1)
        assert np.array_equal(X[b], Xr)


def test_trmm_sweep_bitexact(gpu, oracle_lib):
    import torch

    rng = np.random.default_rng(5)
    for m in (1, 3, 8, 13, 20):
        for n in (1, 4, 7, 20):
            batch = 2
            alpha = 0.625
            A = rng.random((batch, m, m))  # strictly lower part non-zero: must not be read
            B = rng.random((batch, m, n))
            dC = gpu.col_major((batch,), m, n, "cuda")
            gpu.trmm(alpha, to_dev(A), gpu.UPPER, False, to_dev(B), dC)
            A2 = rng.random((batch, n, n))
            B2 = rng.random((batch, m, n))
            dC2 = gpu.col_major((batch,), m, n, "cuda")
            gpu.trmm(alpha, to_dev(B2), to_dev(A2), gpu.LOWER, False, dC2)
            torch.cuda.synchronize()
            C, C2 = dC.cpu().numpy(), dC2.cpu().numpy()
            for b in range(batch):
                Cr = F(np.zeros((m, n)))
                assert oracle_lib.trmm(0, 1, 0, alpha, F(A[b]), F(B[b]), Cr) == 0
                assert np.array_equal(C[b], Cr)
                Cr2 = F(np.zeros((m, n)))
                assert oracle_lib.trmm(1, 0, 0, alpha, F(A2[b]), F(B2[b]), Cr2) == 0
                assert np.array_equal(C2[b], Cr2)


@pytest.mark.parametrize("side,uplo,unit", [(0, 0, 0), (0, 0, 1), (0, 1, 1), (1, 1, 0), (1, 1, 1), (1, 0, 1)])
def test_trmm_variants_blast_leaves_out(gpu, oracle_lib, side, uplo, unit):
    """The (side, uplo, unit) combinations BLAST throws for (algorithm/Trmm.hpp:101-124, 240):
    bit for bit against the oracle's extension of the implemented pattern, and against numpy."""
    import torch

    rng = np.random.default_rng(40 + 4 * side + 2 * uplo + unit)
    for m in (1, 3, 8, 13, 20):
        for n in (1, 5, 12, 20):
            batch = 3
            k = m if side == 0 else n
            A = rng.random((batch, k, k))
            B = rng.random((batch, m, n))
            alpha = 1.0 if n % 2 == 0 else 0.625
            dA, dB = to_dev(A), to_dev(B)
            dC = gpu.col_major((batch,), m, n, "cuda")
            if side == 0:
                gpu.trmm(alpha, dA, uplo, bool(unit), dB, dC)
            else:
                gpu.trmm(alpha, dB, dA, uplo, bool(unit), dC)
            torch.cuda.synchronize()
            C = dC.cpu().numpy()
            for b in range(batch):
                Cr = F(np.zeros((m, n)))
                assert oracle_lib.trmm_any(side, uplo, unit, alpha, F(A[b]), F(B[b]), Cr) == 0
                assert np.array_equal(C[b], Cr), (m, n)
                T = np.triu(A[b]) if uplo == 1 else np.tril(A[b])
                if unit:
                    np.fill_diagonal(T, 1.0)
                ref = alpha * (T @ B[b] if side == 0 else B[b] @ T)
                assert approx_equal(C[b], ref, 1e-10, 1e-10)


@pytest.mark.parametrize("uplo,unit,trans", [(0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 1), (1, 0, 1)])
def test_trsm_right_side(gpu, oracle_lib, uplo, unit, trans):
    """X op(A) = B (no BLAST counterpart), bit for bit against the oracle, residual against numpy."""
    import torch

    rng = np.random.default_rng(60 + 4 * uplo + 2 * unit + trans)
    for m in (1, 4, 9, 17):
        for n in (1, 3, 8, 30):
            batch = 3
            A = rng.random((batch, n, n)) + n * np.eye(n)
            B = rng.random((batch, m, n))
            dA = to_dev(np.swapaxes(A, 1, 2)).mT if trans else to_dev(A)
            dB = to_dev(B)
            dX = gpu.col_major((batch,), m, n, "cuda")
            gpu.trsm_right(uplo, unit, dA, dB, dX)
            gpu.trsm_right(uplo, unit, dA, dB, dB)  # X aliasing B
            torch.cuda.synchronize()
            X, Xa = dX.cpu().numpy(), dB.cpu().numpy()
            for b in range(batch):
                Xr = F(np.zeros((m, n)))
                At = np.ascontiguousarray(A[b].T) if trans else F(A[b])
                assert oracle_lib.trsm_right(uplo, unit, At, F(B[b]), Xr, trans) == 0
                assert np.array_equal(X[b], Xr), (m, n)
                assert np.array_equal(Xa[b], Xr), (m, n)
                opA = A[b]
                T = np.triu(opA) if uplo == 1 else np.tril(opA)
                if unit:
                    np.fill_diagonal(T, 1.0)
                assert approx_equal(X[b] @ T, B[b], 1e-10, 1e-10)

"""GPU parity of batched potrf / potrs / posv against the oracle.

Reference: blast::potrf (dense/Potrf.hpp:66-106) and the trsm solves (dense/Trsm.hpp:17-66).
Bar: normwise relative error <= 10*n*eps against the oracle's BLAST restatement on the same
inputs (the kernel multiplies by reciprocal pivots where BLAST divides), plus BLAST's own test
checks (L*L^T == A at 1e-11, dense/PotrfTest.cpp:26-88).
"""
import numpy as np
import pytest

from helpers import EPS, approx_equal, normwise, spd, spd_batch, to_dev

pytestmark = pytest.mark.gpu


def test_recip_helpers_accuracy(gpu):
    """The Newton-Raphson reciprocal square root / reciprocal match IEEE 1/sqrt(x), 1/x to 2 ulp."""
    import torch

    from blast_gb300 import _lib

    rng = np.random.default_rng(0)
    x = np.concatenate([10.0 ** rng.uniform(-300, 300, 4000), rng.uniform(0.5, 2, 4000),
                        10.0 ** rng.uniform(-40, 40, 4000)])
    dx = torch.from_numpy(x).cuda()
    for which, ref in ((0, 1.0 / np.sqrt(x)), (1, 1.0 / x)):
        dy = torch.empty_like(dx)
        _lib.call("blastgpu_selftest_recip", which, dx.data_ptr(), dy.data_ptr(), len(x),
                  torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        y = dy.cpu().numpy()
        ulps = np.abs(y - ref) / np.spacing(ref)
        assert ulps.max() <= 2.0, (which, ulps.max())


def test_posv_n48_batch(gpu, oracle_lib):
    """The Cholesky-solve workload's shape: n = 48, 8 right-hand sides."""
    import torch

    rng = np.random.default_rng(42)
    batch, n, nrhs = 512, 48, 8
    A = spd_batch(rng, batch, n)
    B = rng.standard_normal((batch, n, nrhs))
    Lr, Xr, infor = oracle_lib.posv_batch(A, B)
    dA, dB = to_dev(A), to_dev(B)
    dL = gpu.col_major((batch,), n, n, "cuda")
    dL.zero_()
    dX = gpu.col_major((batch,), n, nrhs, "cuda")
    info = gpu.posv(dA, dL, dB, dX)
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0 and int(np.abs(infor).sum()) == 0
    L, X = np.tril(dL.cpu().numpy()), dX.cpu().numpy()
    tol = 10 * n * EPS
    for b in range(batch):
        assert normwise(L[b], np.tril(Lr[b])) <= tol
        assert normwise(X[b], Xr[b]) <= tol * 10  # two solves amplify by cond(L)
    # the strict upper triangle of L is not written
    assert np.all(np.triu(dL.cpu().numpy(), 1) == 0)


def test_potrf_sizes_0_to_50(gpu, oracle_lib):
    """BLAST's sweep M = 0..50 (dense/PotrfTest.cpp:26-45): L*L^T == A, and parity."""
    import torch

    rng = np.random.default_rng(1)
    for n in range(0, 51):
        batch = 3
        A = spd_batch(rng, batch, n) if n else np.zeros((batch, 0, 0))
        dA = to_dev(A)
        dL = gpu.col_major((batch,), n, n, "cuda")
        dL.zero_()
        info = gpu.potrf(dA, dL)
        torch.cuda.synchronize()
        assert int(info.abs().sum()) == 0
        L = dL.cpu().numpy()
        for b in range(batch):
            Lr = np.zeros((n, n), order="F")
            oracle_lib.potrf(np.asfortranarray(A[b]), Lr)
            assert normwise(L[b], Lr) <= 10 * max(n, 1) * EPS, n
            assert approx_equal(L[b] @ L[b].T, A[b]), n


def test_potrf_in_place_keeps_upper(gpu):
    """potrf(A, A) (dense/PotrfTest.cpp:67-88): the strict upper triangle is left untouched."""
    import torch

    rng = np.random.default_rng(2)
    n = 20
    A = np.stack([spd(rng, n) for _ in range(4)])
    marker = np.triu(np.full((n, n), 7.0), 1)
    Ain = np.tril(A) + marker
    dA = to_dev(Ain)
    info = gpu.potrf(dA, dA)
    torch.cuda.synchronize()
    out = dA.cpu().numpy()
    assert int(info.abs().sum()) == 0
    assert np.all(np.triu(out, 1) == marker)
    for b in range(4):
        L = np.tril(out[b])
        assert approx_equal(L @ L.T, A[b])


def test_potrf_not_positive_definite_info(gpu, oracle_lib):
    import torch

    rng = np.random.default_rng(3)
    n = 13
    A = spd_batch(rng, 6, n)
    A[1, 5, 5] = -100.0  # pivot 5 becomes negative
    A[3] = -np.eye(n)    # first pivot negative
    dA = to_dev(A)
    dL = gpu.col_major((6,), n, n, "cuda")
    info = gpu.potrf(dA, dL).cpu().numpy()
    ref = []
    for b in range(6):
        Lr = np.zeros((n, n), order="F")
        ref.append(oracle_lib.potrf(np.asfortranarray(A[b]), Lr))
    assert list(info) == ref
    assert info[1] == 6 and info[3] == 1 and info[0] == 0


def test_potrs_standalone_and_aliasing(gpu, oracle_lib):
    import torch

    rng = np.random.default_rng(4)
    for n, nrhs in [(1, 1), (7, 3), (48, 8), (61, 13)]:
        batch = 4
        A = spd_batch(rng, batch, n)
        B = rng.standard_normal((batch, n, nrhs))
        Lr, Xr, _ = oracle_lib.posv_batch(A, B)
        dL = to_dev(Lr)
        dX = to_dev(B)
        gpu.potrs(dL, dX, dX)  # X aliases B
        torch.cuda.synchronize()
        X = dX.cpu().numpy()
        for b in range(batch):
            assert normwise(X[b], Xr[b]) <= 100 * n * EPS, (n, nrhs)
            assert normwise(A[b] @ X[b], B[b]) <= 1e-12 * n


def test_potrf_size_errors(gpu):
    dA = to_dev(np.eye(4)[None].repeat(2, 0))
    dL = gpu.col_major((2,), 3, 3, "cuda")
    with pytest.raises(ValueError):
        gpu.potrf(dA, dL)


@pytest.mark.parametrize("n,nrhs,batch", [(48, 8, 20_000), (48, 8, 2_000), (13, 3, 777), (61, 13, 1_000),
                                          (100, 8, 300), (1, 1, 50), (4, 2, 40)])
def test_posv_quad_kernel_bit_identical(gpu, n, nrhs, batch):
    """The quad kernel (4 lanes per matrix, rows interleaved over the lanes, right-hand sides split
    between them; ``posv.quad.n<bin>`` chooses it by batch size) gives the thread-per-matrix
    kernel's L, X and info bit for bit, for posv, potrf and potrs: every element sees the same
    operations in the same order. n = 61 and 100 take more than one tile of rows per lane."""
    import torch

    from blast_gb300 import _lib
    from blast_gb300.tune import size_bin

    rng = np.random.default_rng(n * 1000 + nrhs)
    A = spd_batch(rng, batch, n)
    A[batch // 2, n // 2, n // 2] = -1.0  # one matrix not positive definite: info and NaNs agree
    B = rng.standard_normal((batch, n, nrhs))
    key = f"posv.quad.n{size_bin(n)}"
    old = _lib.tune_get(key)
    outs = {}
    try:
        for q in (0, 1_000_000):  # never / always quads
            _lib.tune_set(key, q)
            dA, dB = to_dev(A), to_dev(B)
            dL = gpu.col_major((batch,), n, n, "cuda")
            dL.zero_()
            dX = gpu.col_major((batch,), n, nrhs, "cuda")
            info = gpu.posv(dA, dL, dB, dX)
            dL2 = gpu.col_major((batch,), n, n, "cuda")
            dL2.zero_()
            info2 = gpu.potrf(dA, dL2)
            dY = to_dev(B)
            gpu.potrs(dL2, dY, dY)
            torch.cuda.synchronize()
            outs[q] = [t.cpu().numpy() for t in (dL, dX, info, dL2, info2, dY)]
    finally:
        if old is not None:
            _lib.tune_set(key, old)
        else:
            _lib.tune_set(key, 0 if n <= 8 else 50 if n <= 16 else 150)
    assert outs[0][2][batch // 2] != 0
    for a, b in zip(outs[0], outs[1_000_000]):
        assert np.array_equal(a, b, equal_nan=True)

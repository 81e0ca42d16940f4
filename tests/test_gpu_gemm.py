"""GPU parity of the batched gemm against the oracle (blast::gemm, algorithm/Gemm.hpp:41-118).

The kernel performs BLAST's per-element sequence of fused multiply-adds, so results are compared
bit for bit; the reference's own tolerance (test/blast/math/dense/GemmTest.cpp, 1e-11) is implied.
"""
import numpy as np
import pytest

from helpers import to_dev

pytestmark = pytest.mark.gpu


def _oracle_gemm(orc, alpha, A, B, beta, C):
    D = np.zeros((A.shape[0], B.shape[1]), order="F")
    orc.gemm(alpha, np.asfortranarray(A), np.asfortranarray(B), beta, np.asfortranarray(C), D)
    return D


@pytest.mark.parametrize("alpha,beta", [(1.0, 1.0), (0.7, -1.3), (-1.0, 0.0)])
def test_gemm_24_batch_bitexact(gpu, oracle_lib, alpha, beta):
    import torch

    rng = np.random.default_rng(11)
    batch, m = 1000, 24
    A, B, C = (rng.uniform(-1, 1, (batch, m, m)) for _ in range(3))
    ref = oracle_lib.gemm_batch(alpha, A, B, beta, C)
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
    dD = gpu.col_major((batch,), m, m, "cuda")
    gpu.gemm(alpha, dA, dB, beta, dC, dD)
    torch.cuda.synchronize()
    assert np.array_equal(dD.cpu().numpy(), ref)


def test_gemm_sweep_ragged_descriptors(gpu, oracle_lib):
    """BLAST's sweep m, n, k in 1..20 (GemmTest.cpp:30-32), all in one ragged launch, with B both
    column-major and row-major (trans view, Cr variant) and as unaligned submatrix views taken at
    the bottom-right corner of a 20 x 20 parent (GemmTest.cpp:56-88)."""
    import torch

    from blast_gb300 import _lib, desc

    rng = np.random.default_rng(5)
    sizes = [(m, n, k) for m in range(1, 21) for n in range(1, 21) for k in range(1, 21, 3)]
    recs = np.zeros(len(sizes), dtype=desc.GEMM_DTYPE)
    keep, refs, outs = [], [], []
    for idx, (m, n, k) in enumerate(sizes):
        A = rng.uniform(-1, 1, (m, k))
        B = rng.uniform(-1, 1, (k, n))
        C = rng.uniform(-1, 1, (m, n))
        alpha, beta = rng.uniform(-1, 1), rng.uniform(-1, 1)
        refs.append(_oracle_gemm(oracle_lib, alpha, A, B, beta, C))
        dA = to_dev(A)
        if idx % 2:  # row-major B (BLAST's trans() of a column-major n x k)
            dB = torch.from_numpy(np.ascontiguousarray(B)).cuda()
        else:
            dB = to_dev(B)
        # C and D as views at the bottom-right corner of 20 x 20 parents (unaligned pointers).
        pc = to_dev(rng.uniform(-1, 1, (20, 20)))
        pc[20 - m:, 20 - n:] = torch.from_numpy(C).cuda()
        dC = pc[20 - m:, 20 - n:]
        pd = to_dev(np.zeros((20, 20)))
        dD = pd[20 - m:, 20 - n:]
        recs[idx] = (desc.mat_record(dA), desc.mat_record(dB), desc.mat_record(dC),
                     desc.mat_record(dD), alpha, beta)
        keep += [dA, dB, pc, pd]
        outs.append(dD)
    d = desc.upload(recs, "cuda")
    _lib.call("blastgpu_dgemm_batched", d.data_ptr(), len(sizes), 20, 20, 20,
              torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    for (m, n, k), ref, dD in zip(sizes, refs, outs):
        assert np.array_equal(dD.cpu().numpy(), ref), (m, n, k)


def test_gemm_larger_and_transposed(gpu, oracle_lib):
    import torch

    rng = np.random.default_rng(7)
    for (m, n, k) in [(33, 65, 17), (64, 64, 64), (100, 3, 129)]:
        batch = 5
        A = rng.uniform(-1, 1, (batch, m, k))
        B = rng.uniform(-1, 1, (batch, k, n))
        C = rng.uniform(-1, 1, (batch, m, n))
        ref = oracle_lib.gemm_batch(1.5, A, B, 0.5, C)
        dA = torch.from_numpy(A).cuda()  # row-major A (trans view)
        dB = to_dev(B, ld=k + 3)
        dC, dD = to_dev(C), gpu.col_major((batch,), m, n, "cuda", ld=m + 1)
        gpu.gemm(1.5, dA, dB, 0.5, dC, dD)
        torch.cuda.synchronize()
        assert np.array_equal(dD.cpu().numpy(), ref), (m, n, k)


def test_gemm_in_place_and_errors(gpu, oracle_lib):
    import torch

    rng = np.random.default_rng(3)
    A, B, C = (rng.uniform(-1, 1, (4, 24, 24)) for _ in range(3))
    ref = oracle_lib.gemm_batch(-1.0, A, B, 1.0, C)
    dC = to_dev(C)
    gpu.gemm(-1.0, to_dev(A), to_dev(B), 1.0, dC, dC)  # C == D, as getrf's trailing update
    torch.cuda.synchronize()
    assert np.array_equal(dC.cpu().numpy(), ref)
    with pytest.raises(ValueError, match="Matrix sizes do not match"):
        gpu.gemm(to_dev(A[:, :, :5]), to_dev(B), dC, dC)

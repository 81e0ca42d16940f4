"""GPU parity of the batched BLAS-2 building blocks (ger, iamax, laswp, swap, trsv) against the
oracle, bit for bit, over the reference's own size sweeps (dense/GerTest.cpp: m, n in 1..20;
dense/Iamax.cpp: n in 1..49; dense/TrsvTest.cpp: n in 1..20)."""
import numpy as np
import pytest

from helpers import approx_equal, to_dev

pytestmark = pytest.mark.gpu


def F(a):
    return np.asfortranarray(a)


def test_ger_sweep_bitexact(gpu, oracle_lib):
    import torch

    rng = np.random.default_rng(21)
    batch = 3
    for m in range(1, 21):
        for n in range(1, 21, 3):
            x, y = rng.random((batch, m)), rng.random((batch, n))
            A = rng.random((batch, m, n))
            alpha = float(rng.random())
            dx, dy = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
            dA = to_dev(A)
            dB = gpu.col_major((batch,), m, n, "cuda")
            gpu.ger(alpha, dx, dy, dA, dB)
            gpu.ger(alpha, dx, dy, dA, dA)  # B aliasing A
            torch.cuda.synchronize()
            B, Ba = dB.cpu().numpy(), dA.cpu().numpy()
            for b in range(batch):
                Br = F(np.zeros((m, n)))
                oracle_lib.ger(alpha, x[b], y[b], F(A[b]), Br)
                assert np.array_equal(B[b], Br), (m, n)
                assert np.array_equal(Ba[b], Br), (m, n)
                assert approx_equal(Br, A[b] + alpha * np.outer(x[b], y[b]), 1e-10, 1e-10)


def test_ger_strided_vectors(gpu, oracle_lib):
    """x and y with increments (rows of a matrix), one shared y for the whole batch."""
    import torch

    rng = np.random.default_rng(22)
    batch, m, n = 5, 37, 9
    X = torch.from_numpy(rng.random((batch, 3, m))).cuda()
    y = torch.from_numpy(rng.random(2 * n)).cuda()[::2]
    A = rng.random((batch, m, n))
    dA = to_dev(A)
    x = X[:, 1, :]
    gpu.ger(-1.0, x, y, dA, dA)
    torch.cuda.synchronize()
    out = dA.cpu().numpy()
    for b in range(batch):
        Br = F(np.zeros((m, n)))
        oracle_lib.ger(-1.0, x[b].cpu().numpy(), y.cpu().numpy(), F(A[b]), Br)
        assert np.array_equal(out[b], Br)


def test_iamax_sweep(gpu, oracle_lib):
    import torch

    rng = np.random.default_rng(23)
    for n in range(1, 50):
        x = rng.standard_normal((7, n))
        got = gpu.iamax(torch.from_numpy(x).cuda()).cpu().numpy()
        for b in range(7):
            assert got[b] == oracle_lib.idamax(x[b]), n
    # long vectors, strided, ties (first index wins), NaN rules of the strict '>' scan
    n = 1000
    x = rng.standard_normal((6, n))
    x[1, [17, 400, 901]] = 50.0
    x[2, 0] = np.nan
    x[3, 5] = np.nan
    x[4, :] = 0.0
    x[5, [3, 999]] = -np.inf
    dx = torch.from_numpy(np.repeat(x, 2, axis=1)).cuda()[:, ::2]
    got = gpu.iamax(dx).cpu().numpy()
    want = [oracle_lib.idamax(x[b]) for b in range(6)]
    assert list(got) == want
    assert want[1] == 17 and want[2] == 0 and want[4] == 0 and want[5] == 3


def test_laswp_matches_oracle(gpu, oracle_lib):
    import torch

    rng = np.random.default_rng(24)
    batch, m, ncols = 4, 30, 11
    A = rng.random((batch, m, ncols))
    ipiv = np.stack([np.array([rng.integers(k, m) for k in range(m)], dtype=np.int32) for _ in range(batch)])
    dA = to_dev(A)
    gpu.laswp(dA, 3, 25, torch.from_numpy(ipiv).cuda())
    torch.cuda.synchronize()
    out = dA.cpu().numpy()
    for b in range(batch):
        Ar = F(A[b].copy())
        oracle_lib.laswp(Ar, 3, 25, ipiv[b])
        assert np.array_equal(out[b], Ar)


def test_swap(gpu):
    import torch

    rng = np.random.default_rng(25)
    x, y = rng.random((3, 40)), rng.random((3, 40))
    dx, dy = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    gpu.swap(dx, dy)
    assert np.array_equal(dx.cpu().numpy(), y) and np.array_equal(dy.cpu().numpy(), x)


@pytest.mark.parametrize("upper", [False, True])
def test_trsv_sweep_bitexact(gpu, oracle_lib, upper):
    import torch

    rng = np.random.default_rng(26 + upper)
    batch = 3
    for n in range(1, 21):
        A = rng.random((batch, n, n))
        A = (np.triu(A) if upper else np.tril(A)) + np.eye(n)
        b = rng.random((batch, n))
        dA, db = to_dev(A), torch.from_numpy(b).cuda()
        dx = torch.zeros((batch, n), dtype=torch.float64, device="cuda")
        (gpu.trsv_left_upper if upper else gpu.trsv_left_lower)(dA, db, dx)
        torch.cuda.synchronize()
        x = dx.cpu().numpy()
        for k in range(batch):
            Xr = F(np.zeros((n, 1)))
            oracle_lib.trsm(int(upper), 0, F(A[k]), F(b[k][:, None]), Xr)
            assert np.array_equal(x[k], Xr[:, 0]), n
            assert approx_equal(A[k] @ x[k], b[k], 1e-10, 1e-10)


def test_blas2_argument_errors(gpu):
    import torch

    from blast_gb300 import _lib

    x = torch.zeros((2, 4), dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        gpu.iamax(torch.zeros((2, 0), dtype=torch.float64, device="cuda"))
    with pytest.raises(ValueError):
        gpu.swap(x, torch.zeros((2, 5), dtype=torch.float64, device="cuda"))
    assert _lib.lib().blastgpu_idamax_strided(0, x.data_ptr(), 1, 4, x.data_ptr(), 2, None) == -1
    assert _lib.lib().blastgpu_dlaswp_strided(4, x.data_ptr(), 4, 16, 3, 2, None, 0, 1, None) == -6

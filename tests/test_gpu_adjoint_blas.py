"""Adjoints of gemm, trsm and potrf (blastgpu_dgemm_bwd_strided, blastgpu_dtrsm_bwd_strided,
blastgpu_dpotrf_bwd_strided): against CPU binary64 reference gradients (numpy, the formulas
written out independently), and against central finite differences (h = 1e-6) of the forward
operations run on the GPU."""
import numpy as np
import pytest

from helpers import spd, to_dev

pytestmark = pytest.mark.gpu


def _tensor(vals, row_major):
    """CUDA tensor holding vals (…, r, c): column-major, or the row-major view BLAST's trans() gives."""
    return to_dev(np.swapaxes(vals, -1, -2)).mT if row_major else to_dev(vals)


@pytest.mark.parametrize("ta,tb", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_gemm_bwd_matches_reference(gpu, ta, tb):
    import torch

    rng = np.random.default_rng(70 + 2 * ta + tb)
    batch, m, n, k = 5, 7, 4, 6
    alpha, beta = 0.7, -1.3
    opA, opB = rng.standard_normal((batch, m, k)), rng.standard_normal((batch, k, n))
    Dbar = rng.standard_normal((batch, m, n))
    A0, B0, C0 = (rng.standard_normal(s) for s in ((batch, m, k), (batch, k, n), (batch, m, n)))
    dA, dB, dD = _tensor(opA, ta), _tensor(opB, tb), to_dev(Dbar)
    Abar, Bbar, Cbar = _tensor(A0, ta), _tensor(B0, tb), to_dev(C0)
    gpu.gemm_bwd(alpha, dA, dB, beta, dD, Abar, Bbar, Cbar)
    torch.cuda.synchronize()
    want_A = A0 + alpha * Dbar @ np.swapaxes(opB, 1, 2)
    want_B = B0 + alpha * np.swapaxes(opA, 1, 2) @ Dbar
    want_C = C0 + beta * Dbar
    assert np.allclose(Abar.cpu().numpy(), want_A, rtol=1e-12, atol=1e-12)
    assert np.allclose(Bbar.cpu().numpy(), want_B, rtol=1e-12, atol=1e-12)
    assert np.allclose(Cbar.cpu().numpy(), want_C, rtol=1e-12, atol=1e-12)
    # outputs are optional: only dl/dC
    C1 = to_dev(np.zeros((batch, m, n)))
    gpu.gemm_bwd(alpha, dA, dB, beta, dD, None, None, C1)
    torch.cuda.synchronize()
    assert np.array_equal(C1.cpu().numpy(), beta * Dbar)


def test_gemm_bwd_finite_differences(gpu):
    import torch

    rng = np.random.default_rng(75)
    m, n, k = 5, 3, 4
    A, B = rng.standard_normal((m, k)), rng.standard_normal((k, n))
    C, W = rng.standard_normal((m, n)), rng.standard_normal((m, n))
    alpha, beta = 1.1, 0.4

    def loss(Ah, Bh, Ch):
        D = to_dev(np.zeros((m, n)))
        gpu.gemm(alpha, to_dev(Ah), to_dev(Bh), beta, to_dev(Ch), D)
        torch.cuda.synchronize()
        return float(np.sum(W * D.cpu().numpy()))

    gA, gB, gC = (to_dev(np.zeros(s)) for s in ((m, k), (k, n), (m, n)))
    gpu.gemm_bwd(alpha, to_dev(A), to_dev(B), beta, to_dev(W), gA, gB, gC)
    torch.cuda.synchronize()
    h = 1e-6
    for X, g, idx in ((A, gA, (2, 1)), (B, gB, (3, 2)), (C, gC, (0, 2))):
        E = np.zeros_like(X)
        E[idx] = h
        args_p = [A, B, C]
        args_m = [A, B, C]
        pos = 0 if X is A else (1 if X is B else 2)
        args_p[pos], args_m[pos] = X + E, X - E
        fd = (loss(*args_p) - loss(*args_m)) / (2 * h)
        assert abs(fd - g.cpu().numpy()[idx]) <= 1e-6 * max(1.0, abs(fd)), (idx, fd)


def _tri(T, uplo, unit):
    out = np.triu(T) if uplo == 1 else np.tril(T)
    if unit:
        np.fill_diagonal(out, 1.0)
    return out


@pytest.mark.parametrize("uplo", [0, 1])
@pytest.mark.parametrize("unit", [0, 1])
@pytest.mark.parametrize("trans", [0, 1])
def test_trsm_bwd_matches_reference(gpu, uplo, unit, trans):
    import torch

    rng = np.random.default_rng(80 + 4 * uplo + 2 * unit + trans)
    batch, m, r = 4, 9, 3
    T = rng.standard_normal((batch, m, m)) + 6.0 * np.eye(m)  # the values of op(A) as passed
    B = rng.standard_normal((batch, m, r))
    Xbar = rng.standard_normal((batch, m, r))
    G0 = rng.standard_normal((batch, m, m))
    dA = _tensor(T, trans)
    dX = to_dev(np.zeros((batch, m, r)))
    gpu.trsm(uplo, unit, dA, to_dev(B), dX)
    dBbar = to_dev(np.zeros((batch, m, r)))
    dAbar = _tensor(G0, trans)
    gpu.trsm_bwd(uplo, unit, dA, dX, to_dev(Xbar), dBbar, dAbar)
    torch.cuda.synchronize()
    X, Bbar, Abar = dX.cpu().numpy(), dBbar.cpu().numpy(), dAbar.cpu().numpy()
    for b in range(batch):
        Tt = _tri(T[b], uplo, unit)
        br = np.linalg.solve(Tt.T, Xbar[b])
        G = -br @ X[b].T
        mask = np.triu(np.ones((m, m)), 1 if unit else 0) if uplo == 1 else np.tril(np.ones((m, m)), -1 if unit else 0)
        assert np.allclose(Bbar[b], br, rtol=1e-11, atol=1e-12), b
        assert np.allclose(Abar[b], G0[b] + mask * G, rtol=1e-11, atol=1e-12), b
    # Bbar may be Xbar (in place); Abar is optional
    dXb = to_dev(Xbar)
    gpu.trsm_bwd(uplo, unit, dA, dX, dXb, dXb)
    torch.cuda.synchronize()
    assert np.array_equal(dXb.cpu().numpy(), Bbar)


def test_trsm_bwd_finite_differences(gpu):
    import torch

    rng = np.random.default_rng(88)
    m, r = 6, 2
    T = rng.standard_normal((m, m)) + 5.0 * np.eye(m)
    B, W = rng.standard_normal((m, r)), rng.standard_normal((m, r))

    def loss(Th, Bh):
        X = to_dev(np.zeros((m, r)))
        gpu.trsm(0, False, to_dev(Th), to_dev(Bh), X)
        torch.cuda.synchronize()
        return float(np.sum(W * X.cpu().numpy()))

    X = to_dev(np.zeros((m, r)))
    gpu.trsm(0, False, to_dev(T), to_dev(B), X)
    gB, gT = to_dev(np.zeros((m, r))), to_dev(np.zeros((m, m)))
    gpu.trsm_bwd(0, False, to_dev(T), X, to_dev(W), gB, gT)
    torch.cuda.synchronize()
    h = 1e-6
    for i, j in ((0, 0), (3, 1), (5, 5), (4, 2)):
        E = np.zeros((m, m))
        E[i, j] = h
        fd = (loss(T + E, B) - loss(T - E, B)) / (2 * h)
        assert abs(fd - gT.cpu().numpy()[i, j]) <= 1e-6 * max(1.0, abs(fd)), (i, j)
    for i, j in ((0, 0), (5, 1)):
        E = np.zeros((m, r))
        E[i, j] = h
        fd = (loss(T, B + E) - loss(T, B - E)) / (2 * h)
        assert abs(fd - gB.cpu().numpy()[i, j]) <= 1e-6 * max(1.0, abs(fd)), (i, j)


@pytest.mark.parametrize("n", [1, 2, 5, 17, 48])
def test_potrf_bwd_matches_reference(gpu, n):
    import torch

    rng = np.random.default_rng(90 + n)
    batch = 3
    A = np.stack([spd(rng, n) for _ in range(batch)])
    Lbar = np.tril(rng.standard_normal((batch, n, n)))
    dL = to_dev(np.full((batch, n, n), np.nan))  # the strict upper parts are never read
    info = gpu.potrf(to_dev(A), dL)
    Lb = Lbar + np.triu(np.full((n, n), np.nan), 1)
    dAbar = to_dev(np.zeros((batch, n, n)))
    gpu.potrf_bwd(dL, to_dev(Lb), dAbar)
    torch.cuda.synchronize()
    assert not info.any()
    L, Abar = np.tril(np.nan_to_num(dL.cpu().numpy())), dAbar.cpu().numpy()
    for b in range(batch):
        P = L[b].T @ Lbar[b]
        Phi = np.tril(P)
        Phi[np.diag_indices(n)] *= 0.5
        Li = np.linalg.inv(L[b])
        S = Li.T @ Phi @ Li
        want = 0.5 * (S + S.T)
        assert np.allclose(Abar[b], want, rtol=1e-10, atol=1e-12 * np.abs(want).max()), b
        assert np.array_equal(Abar[b], Abar[b].T)


def test_potrf_bwd_finite_differences(gpu):
    import torch

    rng = np.random.default_rng(95)
    n = 6
    A = spd(rng, n)
    W = np.tril(rng.standard_normal((n, n)))

    def loss(Ah):
        L = to_dev(np.zeros((n, n)))
        gpu.potrf(to_dev(Ah), L)
        torch.cuda.synchronize()
        return float(np.sum(W * np.tril(L.cpu().numpy())))

    L = to_dev(np.zeros((n, n)))
    gpu.potrf(to_dev(A), L)
    G = to_dev(np.zeros((n, n)))
    gpu.potrf_bwd(L, to_dev(W), G)
    torch.cuda.synchronize()
    g = G.cpu().numpy()
    h = 1e-6
    for i, j in ((0, 0), (3, 1), (5, 5), (4, 2), (5, 0)):
        E = np.zeros((n, n))
        E[i, j] = E[j, i] = h  # symmetric direction: the gradient pairs (i, j) with (j, i)
        fd = (loss(A + E) - loss(A - E)) / (2 * h)
        assert abs(fd - np.sum(g * E) / h) <= 1e-6 * max(1.0, abs(fd)), (i, j)


def test_adjoint_argument_errors(gpu):
    import torch

    from blast_gb300 import _lib

    x = torch.zeros(64, dtype=torch.float64, device="cuda")
    p = x.data_ptr()
    lib = _lib.lib()
    # a shared (stride 0) output for a batch of 2 would race
    assert lib.blastgpu_dpotrf_bwd_strided(4, p, 4, 16, p, 4, 16, p, 4, 0, 2, None) == -10
    assert lib.blastgpu_dtrsm_bwd_strided(0, 0, 0, 4, 1, p, 4, 16, p, 4, 4, p, 4, 4, p, 4, 0, None, 4, 0, 2,
                                          None) == -17
    assert lib.blastgpu_dgemm_bwd_strided(0, 0, 2, 2, 2, 1.0, p, 2, 4, p, 2, 4, 1.0, p, 2, 4, p, 2, 0, None, 2, 0,
                                          None, 2, 0, 2, None) == -19
    with pytest.raises(ValueError):
        gpu.potrf_bwd(to_dev(np.eye(3)), to_dev(np.eye(3)), to_dev(np.zeros((3, 4))))


def test_autograd_shims_gradcheck(gpu):
    """The torch.autograd shims over the three adjoints (blast_gb300.autograd: gemm_fn, trsm_fn,
    potrf_fn) pass torch.autograd.gradcheck (central differences of the GPU forward operations)."""
    import torch

    from blast_gb300.autograd import gemm_fn, potrf_fn, trsm_fn

    rng = np.random.default_rng(99)
    dev = "cuda"
    A = torch.tensor(rng.standard_normal((2, 3, 4)), device=dev, requires_grad=True)
    B = torch.tensor(rng.standard_normal((2, 4, 2)), device=dev, requires_grad=True)
    C = torch.tensor(rng.standard_normal((2, 3, 2)), device=dev, requires_grad=True)
    assert torch.autograd.gradcheck(lambda a, b, c: gemm_fn(a, b, c, 0.8, -0.5), (A, B, C))
    T = torch.tensor(rng.standard_normal((2, 4, 4)) + 4.0 * np.eye(4), device=dev, requires_grad=True)
    R = torch.tensor(rng.standard_normal((2, 4, 3)), device=dev, requires_grad=True)
    for uplo in (0, 1):
        for unit in (False, True):
            assert torch.autograd.gradcheck(lambda t, r: trsm_fn(t, r, uplo, unit), (T, R))
    G = rng.standard_normal((2, 5, 5))
    S = torch.tensor(G @ np.swapaxes(G, 1, 2) + 5.0 * np.eye(5), device=dev, requires_grad=True)
    # potrf reads the lower triangle of a symmetric input: checked through a symmetrising wrapper
    assert torch.autograd.gradcheck(lambda a: potrf_fn(0.5 * (a + a.mT)), (S,))

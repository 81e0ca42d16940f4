"""GPU parity of the fused syrk + potrf, D = chol(beta*C + alpha*op(A)*op(A)^T): bit for bit against
the two-launch composition (syrkLower then potrf) on the GPU, and within 10*n*eps normwise of the
oracle's syrkLower then potrf. Shapes include BLAST's Riccati benchmark (bench/blas/SyrkPotrf.cpp:
M x N = 4 x 5 and 30 x 60, D = C + A^T*A)."""
import numpy as np
import pytest

from helpers import EPS, normwise, to_dev

pytestmark = pytest.mark.gpu


def F(a):
    return np.asfortranarray(a)


@pytest.fixture(params=["fused", "two_launch"])
def path(request, gpu):
    """Both code paths of blastgpu_dsyrk_potrf_strided: the fused kernel and syrkLower then potrf
    (the default), forced through the tuning key that separates them."""
    from blast_gb300 import _lib

    old = _lib.tune_get("syrk_potrf.fused_min_batch")
    _lib.tune_set("syrk_potrf.fused_min_batch", 0 if request.param == "fused" else 1 << 30)
    yield request.param
    _lib.tune_set("syrk_potrf.fused_min_batch", old if old is not None else 0x7FFFFFFF)  # default: pair


def _case(rng, batch, n, k):
    A = rng.uniform(-1, 1, (batch, n, k))
    G = rng.uniform(-1, 1, (batch, n, n))
    C = G @ np.swapaxes(G, 1, 2) + n * np.eye(n)
    return A, C


@pytest.mark.parametrize("trans", [False, True])
def test_syrk_potrf_matches_composition(gpu, oracle_lib, trans, path):
    import torch

    rng = np.random.default_rng(31 + trans)
    shapes = [(n, k) for n in (1, 2, 3, 5, 8, 13, 20) for k in (1, 4, 11, 20)] + [(48, 16), (60, 30), (64, 7)]
    for n, k in shapes:
        batch = 6
        A, C = _case(rng, batch, n, k)
        alpha, beta = (1.0 if n % 2 else 0.75), (1.0 if k % 2 else 0.5)  # alpha = 1: own code path
        # op(A) = A (n x k, column-major) or the row-major view of a k x n column-major matrix
        dA = to_dev(np.swapaxes(A, 1, 2)).mT if trans else to_dev(A)
        dC = to_dev(C)
        dD = to_dev(np.full((batch, n, n), 7.0))
        info = gpu.syrk_potrf(alpha, dA, beta, dC, dD)
        # composition on the GPU: syrkLower into S, then potrf(S, S)
        dS = to_dev(np.full((batch, n, n), 7.0))
        gpu.syrk_lower(alpha, to_dev(A), beta, dC, dS)
        info2 = gpu.potrf(dS, dS)
        torch.cuda.synchronize()
        D, S = dD.cpu().numpy(), dS.cpu().numpy()
        assert not info.any() and not info2.any(), (n, k)
        assert np.array_equal(D, S), (n, k)
        assert np.all(np.triu(D, 1) == np.triu(np.full((n, n), 7.0), 1)), (n, k)  # upper untouched
        for b in range(batch):
            Sr, Lr = F(np.zeros((n, n))), F(np.zeros((n, n)))
            oracle_lib.syrk_lower(alpha, F(A[b]), beta, F(C[b]), Sr)
            assert oracle_lib.potrf(Sr, Lr) == 0
            assert normwise(np.tril(D[b]), np.tril(Lr)) <= 10 * n * EPS, (n, k)


def test_syrk_potrf_in_place_and_info(gpu, path):
    import torch

    rng = np.random.default_rng(33)
    batch, n, k = 64, 30, 60
    A, C = _case(rng, batch, n, k)
    dA, dC = to_dev(A), to_dev(C)
    dD = to_dev(np.zeros((batch, n, n)))
    gpu.syrk_potrf(1.0, dA, 1.0, dC, dD)
    info = gpu.syrk_potrf(1.0, dA, 1.0, dC, dC)  # D aliasing C
    torch.cuda.synchronize()
    assert not info.any()
    assert np.array_equal(np.tril(dC.cpu().numpy()), np.tril(dD.cpu().numpy()))
    # beta*C + alpha*A*A^T indefinite in instance 3 (C = -10 I, alpha tiny): first pivot fails
    C2 = C.copy()
    C2[3] = -10.0 * np.eye(n)
    info = gpu.syrk_potrf(1e-3, to_dev(A), 1.0, to_dev(C2), dD)
    torch.cuda.synchronize()
    got = info.cpu().numpy()
    assert got[3] == 1 and np.count_nonzero(got) == 1


def test_syrk_potrf_argument_errors(gpu):
    import torch

    from blast_gb300 import _lib

    x = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = x.data_ptr()
    assert _lib.lib().blastgpu_dsyrk_potrf_strided(4, 2, 2, 1.0, p, 4, 0, 1.0, p, 4, 0, p, 4, 0, None, 1,
                                                   None) == -3
    assert _lib.lib().blastgpu_dsyrk_potrf_strided(4, 2, 1, 1.0, p, 1, 0, 1.0, p, 4, 0, p, 4, 0, None, 1,
                                                   None) == -6
    assert _lib.lib().blastgpu_dsyrk_potrf_strided(4, 2, 0, 1.0, p, 4, 0, 1.0, p, 3, 0, p, 4, 0, None, 1,
                                                   None) == -10
    with pytest.raises(ValueError):
        gpu.syrk_potrf(1.0, to_dev(np.zeros((2, 4, 3))), 1.0, to_dev(np.zeros((2, 5, 5))),
                       to_dev(np.zeros((2, 5, 5))))


def test_syrk_potrf_k0_is_potrf(gpu, path):
    """k = 0 leaves D = chol(beta*C); with beta = 1 it is potrf(C) bit for bit."""
    import torch

    rng = np.random.default_rng(34)
    batch, n = 40, 24
    _, C = _case(rng, batch, n, 1)
    dC = to_dev(C)
    dA = torch.zeros((batch, n, 0), dtype=torch.float64, device="cuda")
    dD = to_dev(np.zeros((batch, n, n)))
    info = gpu.syrk_potrf(1.0, dA, 1.0, dC, dD)
    dL = to_dev(np.zeros((batch, n, n)))
    info2 = gpu.potrf(dC, dL)
    torch.cuda.synchronize()
    assert not info.any() and not info2.any()
    assert torch.equal(torch.tril(dD), torch.tril(dL))

"""Hand-written adjoint of the batched SPD solve, through the torch.autograd shim, checked against
central finite differences (h = 1e-6) and a CPU binary64 reference gradient, with the factor kept
or recomputed in the backward pass."""
import numpy as np
import pytest

from helpers import spd

pytestmark = pytest.mark.gpu


def _ref_grads(A, b, t):
    """CPU binary64: l = |x - t|^2 / 2, x = A^{-1} b."""
    x = np.linalg.solve(A, b)
    bbar = np.linalg.solve(A, x - t)
    Abar = -0.5 * (bbar @ x.T + x @ bbar.T)
    return x, Abar, bbar


@pytest.mark.parametrize("keep", [True, False])
def test_spd_solve_uniform_grad(gpu, keep):
    import torch

    from blast_gb300.autograd import spd_solve

    rng = np.random.default_rng(5)
    batch, n, nrhs = 6, 17, 2
    A = np.stack([spd(rng, n) for _ in range(batch)])
    b = rng.standard_normal((batch, n, nrhs))
    t = rng.standard_normal((batch, n, nrhs))
    tA = torch.tensor(A, device="cuda", requires_grad=True)
    tb = torch.tensor(b, device="cuda", requires_grad=True)
    tt = torch.tensor(t, device="cuda")
    x = spd_solve(tA, tb, keep_factor=keep)
    loss = 0.5 * ((x - tt) ** 2).sum()
    loss.backward()
    gA, gb = tA.grad.cpu().numpy(), tb.grad.cpu().numpy()
    for k in range(batch):
        xr, Ar, br = _ref_grads(A[k], b[k], t[k])
        assert np.allclose(x[k].detach().cpu().numpy(), xr, rtol=1e-12, atol=1e-13)
        assert np.allclose(gA[k], Ar, rtol=1e-10, atol=1e-12)
        assert np.allclose(gb[k], br, rtol=1e-10, atol=1e-12)
        assert np.allclose(gA[k], gA[k].T)


def test_spd_solve_finite_differences(gpu):
    import torch

    from blast_gb300.autograd import spd_solve

    rng = np.random.default_rng(6)
    batch, n, nrhs = 2, 9, 1
    A = np.stack([spd(rng, n) for _ in range(batch)])
    b = rng.standard_normal((batch, n, nrhs))
    t = rng.standard_normal((batch, n, nrhs))
    tA = torch.tensor(A, device="cuda", requires_grad=True)
    tb = torch.tensor(b, device="cuda", requires_grad=True)
    tt = torch.tensor(t, device="cuda")

    def loss_of(Ah, bh):
        with torch.no_grad():
            x = spd_solve(torch.tensor(Ah, device="cuda"), torch.tensor(bh, device="cuda"))
            return float(0.5 * ((x - tt) ** 2).sum())

    x = spd_solve(tA, tb)
    (0.5 * ((x - tt) ** 2).sum()).backward()
    gA, gb = tA.grad.cpu().numpy(), tb.grad.cpu().numpy()
    h = 1e-6
    for _ in range(4):
        V = rng.standard_normal(A.shape)
        V = V + np.swapaxes(V, 1, 2)  # symmetric direction
        fd = (loss_of(A + h * V, b) - loss_of(A - h * V, b)) / (2 * h)
        assert abs(fd - np.sum(gA * V)) <= 1e-6 * max(1.0, abs(fd))
        W = rng.standard_normal(b.shape)
        fd = (loss_of(A, b + h * W) - loss_of(A, b - h * W)) / (2 * h)
        assert abs(fd - np.sum(gb * W)) <= 1e-6 * max(1.0, abs(fd))


@pytest.mark.parametrize("warp", [1, 0])
@pytest.mark.parametrize("keep", [True, False])
def test_spd_solve_packed_ragged_grad(gpu, keep, warp):
    """The differentiable workload's shape: ragged n in [32, 128], one right-hand side, with the
    forward solve and the adjoint one warp per matrix ("posv.warp.n<bin>", "posv.warp_bwd.n<bin>"
    = 1) or one CTA per matrix (0)."""
    import torch

    from blast_gb300 import _lib
    from blast_gb300.autograd import spd_solve_packed

    keys = [f"posv.{p}.n{b}" for p in ("warp", "warp_bwd") for b in (8, 16, 32, 64, 128)]
    old = {k: _lib.tune_get(k) for k in keys}
    for k in keys:
        _lib.tune_set(k, warp)
    try:
        _packed_ragged_grad(keep)
    finally:
        for k, v in old.items():
            _lib.tune_set(k, v if v is not None else 1)


def _packed_ragged_grad(keep):
    import torch

    from blast_gb300.autograd import spd_solve_packed

    rng = np.random.default_rng(7)
    ns = np.array([32, 77, 128, 45, 100, 33])
    rs = np.ones_like(ns)
    As = [spd(rng, n) for n in ns]
    bs = [rng.standard_normal((n, 1)) for n in ns]
    ts = [rng.standard_normal((n, 1)) for n in ns]
    A_flat = torch.tensor(np.concatenate([a.reshape(-1, order="F") for a in As]), device="cuda",
                          requires_grad=True)
    b_flat = torch.tensor(np.concatenate([v.ravel() for v in bs]), device="cuda", requires_grad=True)
    t_flat = torch.tensor(np.concatenate([v.ravel() for v in ts]), device="cuda")
    x = spd_solve_packed(A_flat, b_flat, ns, rs, keep_factor=keep)
    (0.5 * ((x - t_flat) ** 2).sum()).backward()
    gA, gb = A_flat.grad.cpu().numpy(), b_flat.grad.cpu().numpy()
    oa = ob = 0
    for n, A, b, t in zip(ns, As, bs, ts):
        xr, Ar, br = _ref_grads(A, b, t)
        assert np.allclose(gA[oa:oa + n * n].reshape(n, n, order="F"), Ar, rtol=1e-10, atol=1e-12)
        assert np.allclose(gb[ob:ob + n], br.ravel(), rtol=1e-10, atol=1e-12)
        oa += n * n
        ob += n

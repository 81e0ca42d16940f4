"""Ragged Cholesky solves (one CTA per matrix; one warp per matrix for small n): the binary64 path
against the oracle and the
mixed-precision path (binary32 factor + binary64 refinement) against the 1e-12 backward-error bar.
"""
import numpy as np
import pytest

from helpers import EPS, normwise

pytestmark = pytest.mark.gpu


def _spd_cond(rng, n, cond):
    """A = Q diag(lambda) Q^T with lambda log-spaced from 1 to 1/cond (the mixed workload's matrices)."""
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    lam = np.logspace(0, -np.log10(cond), n)
    A = (Q * lam) @ Q.T
    return (A + A.T) / 2


def _fwd_inf(x, ref) -> float:
    """Normwise forward error in the infinity norm."""
    return float(np.abs(np.asarray(x) - ref).max() / np.abs(ref).max())


def test_ragged_posv_fp64_matches_oracle(gpu, oracle_lib):
    import torch

    from blast_gb300.ragged import Packed, PosvPlan

    rng = np.random.default_rng(0)
    ns = [65, 1, 7, 32, 33, 64, 100, 128, 129, 200, 256, 257, 300, 511, 512, 31]
    nrhs = [1, 2, 1, 3, 1, 1, 2, 1, 1, 1, 1, 1, 2, 1, 1, 4]
    As = [np.tril(rng.standard_normal((n, n))) for n in ns]
    As = [G @ G.T + n * np.eye(n) for G, n in zip(As, ns)]
    Bs = [rng.standard_normal((n, r)) for n, r in zip(ns, nrhs)]
    dev = "cuda"
    A = Packed(ns, ns, dev)
    A.fill_from(As)
    B = Packed(ns, nrhs, dev)
    B.fill_from(Bs)
    X = Packed(ns, nrhs, dev)
    L = Packed(ns, ns, dev)
    plan = PosvPlan(A, B, X, L)
    plan.run()
    torch.cuda.synchronize()
    info, _, _ = plan.results()
    assert not info.any()
    Ls, Xs = L.to_list(), X.to_list()
    for n, Ah, Bh, Lg, Xg in zip(ns, As, Bs, Ls, Xs):
        Lr = np.zeros((n, n), order="F")
        assert oracle_lib.potrf(np.asfortranarray(Ah), Lr) == 0
        Xr = np.zeros_like(Bh, order="F")
        oracle_lib.potrs(Lr, np.asfortranarray(Bh), Xr)
        assert normwise(np.tril(Lg), Lr) <= 10 * n * EPS, n
        assert normwise(Xg, Xr) <= 100 * n * EPS, n


@pytest.mark.parametrize("ns", [[1, 2, 3, 4, 5, 7, 8, 9, 16, 17, 31, 32],
                                [33, 40, 63, 64, 1, 12, 48, 57],
                                [65, 100, 127, 128, 1, 4, 31, 64, 97, 120, 66, 5]])
def test_ragged_posv_small_warp_kernel(gpu, ns):
    """Ragged binary64 batches with every n <= 128 run one warp per matrix ("posv.warp.n<bin>").
    Its fused multiply-adds are the thread-per-matrix kernel's, in the same order, so L and X are
    the same bits as the uniform thread kernel's on each instance. They also agree with the CTA
    kernel, the other choice for the same bins, within 10 n eps, and a non-positive-definite
    instance reports the same info as the thread kernel."""
    import torch

    from blast_gb300 import _lib
    from blast_gb300.ragged import Packed, PosvPlan

    rng = np.random.default_rng(sum(ns))
    nrhs = [1 + (i % 3) for i in range(len(ns))]
    As = [G @ G.T + n * np.eye(n) for G, n in ((rng.standard_normal((n, n)), n) for n in ns)]
    bad = len(ns) // 2
    if ns[bad] > 2:
        As[bad] = As[bad].copy()
        As[bad][2, 2] = -1.0  # not positive definite: the third pivot fails
    Bs = [rng.standard_normal((n, r)) for n, r in zip(ns, nrhs)]

    def solve(warp):
        A = Packed(ns, ns, "cuda")
        A.fill_from(As)
        B = Packed(ns, nrhs, "cuda")
        B.fill_from(Bs)
        X, L = Packed(ns, nrhs, "cuda"), Packed(ns, ns, "cuda")
        keys = [f"posv.warp.n{b}" for b in (8, 16, 32, 64, 128)]
        old = {k: _lib.tune_get(k) for k in keys}
        try:
            for k in keys:
                _lib.tune_set(k, warp)
            plan = PosvPlan(A, B, X, L)
            plan.run()
            torch.cuda.synchronize()
        finally:
            for k, v in old.items():
                _lib.tune_set(k, v if v is not None else 1)
        return [np.tril(m) for m in L.to_list()], X.to_list(), plan.results()[0]

    Lw, Xw, infow = solve(1)
    Lc, Xc, infoc = solve(0)
    old_min = _lib.tune_get("posv.cta_min_n")
    _lib.tune_set("posv.cta_min_n", 513)  # uniform batches on the thread-per-matrix kernel
    try:
        for i, (n, Ah, Bh) in enumerate(zip(ns, As, Bs)):
            dA = gpu.col_major((1,), n, n, "cuda")
            dA.copy_(torch.from_numpy(Ah[None]))
            dB = gpu.col_major((1,), n, nrhs[i], "cuda")
            dB.copy_(torch.from_numpy(Bh[None]))
            dL, dX = gpu.col_major((1,), n, n, "cuda"), gpu.col_major((1,), n, nrhs[i], "cuda")
            dL.zero_()
            info_t = gpu.posv(dA, dL, dB, dX)
            torch.cuda.synchronize()
            assert int(info_t[0]) == int(infow[i]) == int(infoc[i]), (n, int(info_t[0]), int(infow[i]), int(infoc[i]))
            if infow[i] != 0:
                continue
            assert np.array_equal(Lw[i], np.tril(dL.cpu().numpy()[0])), n
            assert np.array_equal(Xw[i], dX.cpu().numpy()[0]), n
            assert normwise(Lw[i], Lc[i]) <= 10 * n * EPS, n
            assert normwise(Xw[i], Xc[i]) <= 100 * n * EPS, n
    finally:
        _lib.tune_set("posv.cta_min_n", old_min if old_min is not None else 129)
    assert ns[bad] <= 2 or infow[bad] == 3


@pytest.mark.parametrize("cond", [1e2, 1e4, 1e6])
def test_ragged_posv_mixed_backward_error(gpu, cond):
    import torch

    from blast_gb300.ragged import Packed, PosvPlan

    rng = np.random.default_rng(int(np.log10(cond)))
    ns = [64, 96, 128, 200, 255, 256, 300, 384, 450, 512]
    As = [_spd_cond(rng, n, cond) for n in ns]
    Bs = [rng.standard_normal((n, 1)) for n in ns]
    A = Packed(ns, ns, "cuda")
    A.fill_from(As)
    B = Packed(ns, [1] * len(ns), "cuda")
    B.fill_from(Bs)
    X = Packed(ns, [1] * len(ns), "cuda")
    plan = PosvPlan(A, B, X, mixed=True, tol=1e-12, max_iter=10)
    plan.run()
    # the binary64 path on the same batch: the mixed solutions are compared with its solutions
    X64, L64 = Packed(ns, [1] * len(ns), "cuda"), Packed(ns, ns, "cuda")
    PosvPlan(A, B, X64, L64).run()
    torch.cuda.synchronize()
    info, iters, berr = plan.results()
    assert not info.any()
    assert np.all(berr <= 1e-12), berr
    for n, Ah, Bh, Xg, X64g in zip(ns, As, Bs, X.to_list(), X64.to_list()):
        r = Bh - Ah @ Xg
        be = np.abs(r).max() / (np.abs(Ah).sum(1).max() * np.abs(Xg).max() + np.abs(Bh).max())
        assert be <= 1e-12, (n, be)
        # A solution with normwise backward error beta (infinity norms) has a forward error of at
        # most about kappa_inf(A) * beta; both solutions here have beta <= 1e-12 (the binary64
        # path's is near eps), so they differ by at most 2 * kappa_inf(A) * 1e-12.
        bound = 2.5e-12 * np.linalg.cond(Ah, np.inf)
        assert _fwd_inf(Xg, X64g) <= bound, (n, _fwd_inf(Xg, X64g), bound)
        assert _fwd_inf(Xg, np.linalg.solve(Ah, Bh)) <= bound, n


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_ragged_posv_mixed_factorisations(gpu, mode):
    """Every factorisation of the mixed kernel (0: binary32 CUDA-core panel update, 1: tensor-core
    3xTF32 update, 2: tensor-core update with binary64 diagonal blocks, 3: CUDA-core update with
    binary64 diagonal blocks) over every size bin (n <= 64, 128, 256, 512, including sizes that are
    not multiples of 16 or 32) converges to the backward-error tolerance and agrees with the
    binary64 path. A mode other than 0 must also give other bits than mode 0 on some instance,
    which shows that the selected factorisation ran (the per-bin keys of the tuning cache take
    precedence over the global one, so all of them are set)."""
    import torch

    from blast_gb300 import _lib
    from blast_gb300.ragged import Packed, PosvPlan

    rng = np.random.default_rng(40 + mode)
    cond = 1e6
    ns = [1, 5, 16, 17, 33, 64, 65, 100, 127, 128, 129, 191, 250, 256, 257, 333, 480, 505, 512]
    As = [_spd_cond(rng, n, cond) for n in ns]
    Bs = [rng.standard_normal((n, 1)) for n in ns]
    A = Packed(ns, ns, "cuda")
    A.fill_from(As)
    B = Packed(ns, [1] * len(ns), "cuda")
    B.fill_from(Bs)
    X, X64, L64 = Packed(ns, [1] * len(ns), "cuda"), Packed(ns, [1] * len(ns), "cuda"), Packed(ns, ns, "cuda")
    keys = ["posv.mixed"] + [f"posv.mixed.n{b}" for b in (8, 16, 32, 64, 128, 256, 512)]
    old = {k: _lib.tune_get(k) for k in keys}
    X0 = Packed(ns, [1] * len(ns), "cuda")
    try:
        for k in keys:
            _lib.tune_set(k, 0)
        PosvPlan(A, B, X0, mixed=True, tol=1e-12, max_iter=20).run()
        for k in keys:
            _lib.tune_set(k, mode)
        plan = PosvPlan(A, B, X, mixed=True, tol=1e-12, max_iter=20)
        plan.run()
        torch.cuda.synchronize()
    finally:
        for k, v in old.items():
            _lib.tune_set(k, v if v is not None else 0)
    if mode != 0:
        assert any(not np.array_equal(a, b) for a, b in zip(X.to_list(), X0.to_list()))
    PosvPlan(A, B, X64, L64).run()
    torch.cuda.synchronize()
    info, iters, berr = plan.results()
    assert not info.any(), info
    assert np.all(berr <= 1e-12), (berr, ns)
    for n, Ah, Bh, Xg, X64g in zip(ns, As, Bs, X.to_list(), X64.to_list()):
        r = Bh - Ah @ Xg
        be = np.abs(r).max() / (np.abs(Ah).sum(1).max() * np.abs(Xg).max() + np.abs(Bh).max())
        assert be <= 1e-12, (n, be)
        bound = 2.5e-12 * np.linalg.cond(Ah, np.inf)
        assert _fwd_inf(Xg, X64g) <= bound, (n, _fwd_inf(Xg, X64g), bound)


def test_ragged_posv_mixed_reports_breakdown(gpu):
    """A matrix that is not positive definite: the mixed path reports info and a huge backward
    error instead of a solution (the caller re-solves it on the binary64 path)."""
    import torch

    from blast_gb300.ragged import Packed, PosvPlan

    n = 70
    A = Packed([n, n], [n, n], "cuda")
    M = np.eye(n)
    M[40, 40] = -1.0
    A.fill_from([np.eye(n) * 2, M])
    B = Packed([n, n], [1, 1], "cuda")
    B.fill_from([np.ones((n, 1)), np.ones((n, 1))])
    X = Packed([n, n], [1, 1], "cuda")
    plan = PosvPlan(A, B, X, mixed=True)
    plan.run()
    torch.cuda.synchronize()
    info, iters, berr = plan.results()
    assert info[0] == 0 and berr[0] <= 1e-12
    assert info[1] == 41 and not (berr[1] <= 1e-12)


def test_ragged_plans_replay_in_cuda_graph(gpu, oracle_lib):
    """A ragged plan (several size bins, forked streams) captured once into a CUDA graph and
    replayed gives the same results as the direct launch."""
    import torch

    from blast_gb300.ragged import GesvPlan, Packed, PosvPlan

    rng = np.random.default_rng(12)
    ns = [40, 300, 100, 7, 200, 512, 64, 129]
    As = [G @ G.T + n * np.eye(n) for G, n in ((rng.standard_normal((n, n)), n) for n in ns)]
    Bs = [rng.standard_normal((n, 1)) for n in ns]
    A = Packed(ns, ns, "cuda")
    A.fill_from(As)
    B = Packed(ns, [1] * len(ns), "cuda")
    B.fill_from(Bs)
    X = Packed(ns, [1] * len(ns), "cuda")
    L = Packed(ns, ns, "cuda")
    plan = PosvPlan(A, B, X, L)
    plan.run()
    torch.cuda.synchronize()
    ref = X.buf.clone()
    X.buf.zero_()
    g = plan.capture()
    X.buf.zero_()
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(X.buf, ref)

    LU0 = [rng.standard_normal((n, n)) for n in ns]
    A2 = Packed(ns, ns, "cuda")
    A2.fill_from(LU0)
    B2 = Packed(ns, [1] * len(ns), "cuda")
    B2.fill_from(Bs)
    gp = GesvPlan(A2, B2)
    g2 = gp.capture()  # warm-up run + capture modify A2/B2; restore and replay
    A2.fill_from(LU0)
    B2.fill_from(Bs)
    g2.replay()
    torch.cuda.synchronize()
    for n, A0, b, x, p in zip(ns, LU0, Bs, B2.to_list(), gp.pivots()):
        LUr = np.asfortranarray(A0.copy())
        pr = np.zeros(n, dtype=np.int32)
        oracle_lib.getrf(LUr, pr)
        xr = np.asfortranarray(b.copy())
        oracle_lib.getrs(LUr, pr, xr, xr)
        assert np.array_equal(p, pr) and np.array_equal(x, xr)

"""GPU parity of batched getrf / getrs against the oracle (blast::getrf, dense/Getrf.hpp:52-119).

The kernels perform BLAST's operations in BLAST's order (IEEE division by the pivot included), so
factors, pivot sequences and solutions are compared bit for bit; pivot agreement is then exact,
with no near-tie exceptions needed.
"""
import numpy as np
import pytest

from helpers import approx_equal, normwise, to_dev

pytestmark = pytest.mark.gpu


def _oracle_lu(orc, A):
    LU = np.asfortranarray(A.copy())
    ipiv = np.zeros(min(A.shape), dtype=np.int32)
    info = orc.getrf(LU, ipiv)
    return LU, ipiv, info


@pytest.mark.parametrize("m,n", [(1, 1), (2, 2), (3, 3), (4, 4), (5, 5), (8, 8), (9, 9), (12, 12),
                                 (17, 17), (33, 33), (48, 48), (64, 64), (65, 65), (100, 100),
                                 (256, 256), (7, 3), (3, 7), (40, 21), (21, 40), (90, 70), (70, 90),
                                 (300, 129)])
def test_getrf_uniform_bitexact(gpu, oracle_lib, m, n):
    import torch

    rng = np.random.default_rng(m * 1000 + n)
    batch = 8 if max(m, n) > 64 else 64
    A = rng.standard_normal((batch, m, n))
    dA = to_dev(A)
    ipiv = torch.zeros((batch, min(m, n)), dtype=torch.int32, device="cuda")
    info = gpu.getrf(dA, ipiv)
    torch.cuda.synchronize()
    LU, piv = dA.cpu().numpy(), ipiv.cpu().numpy()
    assert not info.cpu().numpy().any()
    for b in range(batch):
        LUr, pr, ir = _oracle_lu(oracle_lib, A[b])
        assert ir == 0
        assert np.array_equal(piv[b], pr), (m, n, b)
        assert np.array_equal(LU[b], LUr), (m, n, b)


def test_getrf_reconstruction_small(gpu, oracle_lib):
    """dense/GetrfTest.cpp:55-82: M, N in 0..5 (here 1..6), P*A == L*U with laswp."""
    import torch

    rng = np.random.default_rng(9)
    for m in range(1, 7):
        for n in range(1, 7):
            A = rng.random((4, m, n))
            dA = to_dev(A)
            ipiv = torch.zeros((4, min(m, n)), dtype=torch.int32, device="cuda")
            gpu.getrf(dA, ipiv)
            torch.cuda.synchronize()
            LU, piv = dA.cpu().numpy(), ipiv.cpu().numpy()
            for b in range(4):
                k = min(m, n)
                L = np.tril(LU[b][:, :k], -1) + np.eye(m, k)
                U = np.triu(LU[b][:k, :])
                PA = np.asfortranarray(A[b].copy())
                oracle_lib.laswp(PA, 0, k, piv[b])
                assert approx_equal(L @ U, PA)


def test_getrf_singular_info(gpu, oracle_lib):
    import torch

    n = 6
    A = np.stack([np.eye(n), np.zeros((n, n)), np.eye(n)])
    A[2, 3, 3] = 0.0  # singular at pivot 3
    dA = to_dev(A)
    ipiv = torch.zeros((3, n), dtype=torch.int32, device="cuda")
    info = gpu.getrf(dA, ipiv).cpu().numpy()
    ref = [_oracle_lu(oracle_lib, A[b])[2] for b in range(3)]
    assert list(info) == ref == [0, 1, 4]


def test_getrs_uniform_bitexact(gpu, oracle_lib):
    import torch

    rng = np.random.default_rng(3)
    for n, nrhs in [(1, 1), (5, 2), (48, 1), (100, 3)]:
        batch = 16
        A = rng.standard_normal((batch, n, n))
        B = rng.standard_normal((batch, n, nrhs))
        dA, dX = to_dev(A), to_dev(B)
        ipiv = torch.zeros((batch, n), dtype=torch.int32, device="cuda")
        info = gpu.getrf(dA, ipiv)
        gpu.getrs(dA, ipiv, dX, info)
        torch.cuda.synchronize()
        X = dX.cpu().numpy()
        for b in range(batch):
            LUr, pr, _ = _oracle_lu(oracle_lib, A[b])
            Xr = np.asfortranarray(B[b].copy())
            oracle_lib.getrs(LUr, pr, Xr, Xr)
            assert np.array_equal(X[b], Xr), (n, nrhs, b)


def test_gesv_ragged_log_uniform(gpu, oracle_lib):
    """The ragged LU workload's shape: n log-uniform in [4, 256], one RHS, one descriptor batch;
    pivots, factors and solutions bit-identical to the oracle."""
    import torch

    from blast_gb300 import _lib, desc

    rng = np.random.default_rng(2026)
    count = 300
    ns = np.floor(np.exp(rng.uniform(np.log(4), np.log(257), count))).astype(int)
    As = [rng.standard_normal((n, n)) for n in ns]
    bs = [rng.standard_normal((n, 1)) for n in ns]
    recs = np.zeros(count, dtype=desc.GETRF_DTYPE)
    dAs, dBs, pivs = [], [], []
    for i, (n, A, b) in enumerate(zip(ns, As, bs)):
        dA, dB = to_dev(A), to_dev(b)
        p = torch.zeros(n, dtype=torch.int32, device="cuda")
        recs[i] = (desc.mat_record(dA), p.data_ptr(), desc.mat_record(dB))
        dAs.append(dA)
        dBs.append(dB)
        pivs.append(p)
    d = desc.upload(recs, "cuda")
    info = torch.full((count,), -7, dtype=torch.int32, device="cuda")
    _lib.call("blastgpu_dgesv_batched", d.data_ptr(), info.data_ptr(), count, int(ns.max()),
              torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert not info.cpu().numpy().any()
    for n, A, b, dA, dB, p in zip(ns, As, bs, dAs, dBs, pivs):
        LUr, pr, _ = _oracle_lu(oracle_lib, A)
        assert np.array_equal(p.cpu().numpy(), pr), n
        assert np.array_equal(dA.cpu().numpy(), LUr), n
        xr = np.asfortranarray(b.copy())
        oracle_lib.getrs(LUr, pr, xr, xr)
        assert np.array_equal(dB.cpu().numpy(), xr), n


def test_getrs_batched_ragged_matches_oracle(gpu, oracle_lib):
    """blastgpu_dgetrs_batched on unsorted ragged sizes with several right-hand sides and a
    partial last warp; bit-identical to the oracle's getrs."""
    import torch

    from blast_gb300 import _lib, desc

    rng = np.random.default_rng(77)
    count = 75
    ns = rng.integers(1, 140, count)
    rs = rng.integers(1, 4, count)
    As = [rng.standard_normal((n, n)) for n in ns]
    Bs = [rng.standard_normal((n, r)) for n, r in zip(ns, rs)]
    recs = np.zeros(count, dtype=desc.GETRF_DTYPE)
    keep = []
    for i, (n, A, B) in enumerate(zip(ns, As, Bs)):
        LUr, pr, _ = _oracle_lu(oracle_lib, A)
        dA, dB = to_dev(LUr), to_dev(B)
        p = torch.from_numpy(pr).cuda()
        recs[i] = (desc.mat_record(dA), p.data_ptr(), desc.mat_record(dB))
        keep.append((LUr, pr, dB, p, dA))
    d = desc.upload(recs, "cuda")
    info = torch.zeros(count, dtype=torch.int32, device="cuda")
    _lib.call("blastgpu_dgetrs_batched", d.data_ptr(), info.data_ptr(), count, int(ns.max()),
              torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    for (LUr, pr, dB, p, dA), B in zip(keep, Bs):
        Xr = np.asfortranarray(B.copy())
        oracle_lib.getrs(LUr, pr, Xr, Xr)
        assert np.array_equal(dB.cpu().numpy(), Xr)
    assert _lib.lib().blastgpu_dgetrs_batched(d.data_ptr(), info.data_ptr(), count, -1, None) == -4
    assert _lib.lib().blastgpu_dgetrs_batched(d.data_ptr(), info.data_ptr(), count, 801, None) == -1004


def test_gesv_plan_log_uniform(gpu, oracle_lib):
    """GesvPlan (two getrf bins on forked streams, then getrs) on the ragged LU
    workload's size distribution: pivots and solutions bit-identical to the oracle."""
    import torch

    from blast_gb300.ragged import GesvPlan, Packed

    rng = np.random.default_rng(2027)
    count = 200
    ns = np.floor(np.exp(rng.uniform(np.log(4), np.log(257), count))).astype(int)
    As = [rng.standard_normal((n, n)) for n in ns]
    bs = [rng.standard_normal((n, 1)) for n in ns]
    A = Packed(ns, ns, "cuda")
    A.fill_from(As)
    B = Packed(ns, np.ones_like(ns), "cuda")
    B.fill_from(bs)
    gp = GesvPlan(A, B)
    gp.run()
    torch.cuda.synchronize()
    assert not gp.info_host().any()
    for n, A0, b, x, p in zip(ns, As, bs, B.to_list(), gp.pivots()):
        LUr, pr, _ = _oracle_lu(oracle_lib, A0)
        xr = np.asfortranarray(b.copy())
        oracle_lib.getrs(LUr, pr, xr, xr)
        assert np.array_equal(p, pr), n
        assert np.array_equal(x, xr), n


@pytest.mark.parametrize("n", [300, 513, 800])
def test_getrs_large_n_bitexact(gpu, oracle_lib, n):
    """getrs beyond the ragged workload's sizes: the solution vectors take 32 n doubles of shared
    memory per warp (200 KB at the n = 800 limit); bit-identical to the oracle."""
    import torch

    rng = np.random.default_rng(n)
    batch, nrhs = 3, 2
    A = rng.standard_normal((batch, n, n))
    B = rng.standard_normal((batch, n, nrhs))
    dA, dB = to_dev(A), to_dev(B)
    ipiv = torch.zeros((batch, n), dtype=torch.int32, device="cuda")
    info = gpu.getrf(dA, ipiv)
    gpu.getrs(dA, ipiv, dB, info)
    torch.cuda.synchronize()
    X = dB.cpu().numpy()
    for b in range(batch):
        LUr, pr, _ = _oracle_lu(oracle_lib, A[b])
        Xr = np.asfortranarray(B[b].copy())
        oracle_lib.getrs(LUr, pr, Xr, Xr)
        assert np.array_equal(X[b], Xr), n


@pytest.mark.parametrize("ns", [[7, 40, 65, 100, 129, 200, 256, 31, 1, 4, 5, 8, 9, 33, 67, 97, 130, 255, 300, 512],
                                [7, 40, 65, 100, 129, 200, 256, 31, 1, 4, 5, 8, 9, 33, 67, 97, 130, 255, 2, 3],
                                [3, 17, 33, 64, 1, 100, 97, 128, 31, 32],
                                [1, 2, 3, 5, 8, 13, 21, 32, 30]])
def test_getrf_kernel_choice_keeps_bits(gpu, oracle_lib, ns):
    """The autotuner's per-bin choices between the warp-per-matrix LU kernel, the CTA kernel's
    right-looking schedule and its left-looking schedule ("getrf.cta.n<bin>", "getrf.lazy.n<bin>"),
    and getrs with its forward half one warp per instance or one thread per instance
    ("getrs.warp_fwd"; the warp form serves batches with n <= 256, so the largest n of each case
    selects its register tile) change the schedule, never the result: factors, pivots and
    solutions are identical under every choice and equal to the oracle's."""
    import torch

    from blast_gb300 import _lib
    from blast_gb300.ragged import GesvPlan, Packed

    rng = np.random.default_rng(91)
    mats = [rng.standard_normal((n, n)) for n in ns]
    bins = (8, 16, 32, 64, 128, 256, 512)
    results = []
    for cta, lazy, warp_fwd in ((0, 0, 1), (1, 0, 1), (1, 1, 1), (1, 0, 0)):
        _lib.tune_set("getrs.warp_fwd", warp_fwd)
        for b in bins:
            _lib.tune_set(f"getrf.cta.n{b}", cta)
            _lib.tune_set(f"getrf.lazy.n{b}", lazy)
        try:
            A = Packed(ns, ns, "cuda")
            A.fill_from(mats)
            B = Packed(ns, [1] * len(ns), "cuda")
            B.fill_from([np.ones((n, 1)) for n in ns])
            plan = GesvPlan(A, B)
            plan.run()
            torch.cuda.synchronize()
            results.append((A.to_list(), plan.pivots(), B.to_list(), plan.info_host()))
        finally:
            _lib.tune_set("getrs.warp_fwd", 1)
            for b in bins:
                _lib.tune_set(f"getrf.cta.n{b}", 1 if b > 64 else 0)
                _lib.tune_set(f"getrf.lazy.n{b}", 0)
    LU0, P0, X0, I0 = results[0]
    assert not I0.any()
    for LU1, P1, X1, I1 in results[1:]:
        for i, n in enumerate(ns):
            assert np.array_equal(LU0[i], LU1[i]) and np.array_equal(P0[i], P1[i]), n
            assert np.array_equal(X0[i], X1[i]) and I0[i] == I1[i], n
    for i, n in enumerate(ns):
        LUr = np.asfortranarray(mats[i].copy())
        pr = np.zeros(n, dtype=np.int32)
        oracle_lib.getrf(LUr, pr)
        assert np.array_equal(LU0[i], LUr) and np.array_equal(P0[i], pr), n


def test_getrf_left_looking_singular_and_ties(gpu, oracle_lib):
    """The left-looking schedule on matrices with exact pivot ties (BLAST's strict '>' keeps the
    first) and with an exactly singular column: factors and pivots equal the oracle's, and a
    singular instance reports the oracle's first zero pivot."""
    import torch

    from blast_gb300.ragged import GesvPlan, Packed

    rng = np.random.default_rng(92)
    n = 150
    tie = np.round(rng.standard_normal((n, n)) * 4) / 4  # many exactly equal magnitudes
    sing = rng.standard_normal((n, n))
    sing[:, 77] = 0.0
    ns = [n, n]
    A = Packed(ns, ns, "cuda")
    A.fill_from([tie, sing])
    B = Packed(ns, [1, 1], "cuda")
    B.fill_from([np.ones((n, 1)), np.ones((n, 1))])
    plan = GesvPlan(A, B)
    plan.run()
    torch.cuda.synchronize()
    info = plan.info_host()
    LUr = np.asfortranarray(tie.copy())
    pr = np.zeros(n, dtype=np.int32)
    assert oracle_lib.getrf(LUr, pr) == 0
    assert info[0] == 0
    assert np.array_equal(A.to_list()[0], LUr) and np.array_equal(plan.pivots()[0], pr)
    LUs = np.asfortranarray(sing.copy())
    ps = np.zeros(n, dtype=np.int32)
    assert info[1] == oracle_lib.getrf(LUs, ps) == 78


def _berr(A, x, b):
    r = b - A @ x
    return float(np.abs(r).max() / (np.abs(A).sum(1).max() * np.abs(x).max() + np.abs(b).max()))


@pytest.mark.parametrize("count,seed", [(300, 5), (64, 6)])
def test_mixed_gesv_refines_to_tolerance(gpu, count, seed):
    """Mixed-precision LU (binary32 factor, binary64 refinement) on the ragged LU workload's
    distribution (n log-uniform in [4, 256], N(0,1) entries) plus the edge sizes 1, 2, 32, 33, 64,
    65 and 256, with 1 to 3 right-hand sides: every instance converges to a normwise backward error
    <= 1e-12, recomputed here in binary64; the solutions agree with LAPACK's within the
    conditioning; A is left untouched and B holds X."""
    import scipy.linalg as sla
    import torch

    from blast_gb300.ragged import MixedGesvPlan, Packed

    rng = np.random.default_rng(seed)
    ns = np.floor(np.exp(rng.uniform(np.log(4), np.log(257), count))).astype(int)
    ns = np.concatenate([ns, [1, 2, 32, 33, 64, 65, 256]])
    rs = 1 + rng.integers(0, 3, len(ns))
    As = [rng.standard_normal((n, n)) for n in ns]
    Bs = [rng.standard_normal((n, r)) for n, r in zip(ns, rs)]
    A = Packed(ns, ns, "cuda")
    A.fill_from(As)
    B = Packed(ns, rs, "cuda")
    B.fill_from(Bs)
    A0 = A.buf.clone()
    plan = MixedGesvPlan(A, B, tol=1e-12, max_iter=10)
    plan.run()
    torch.cuda.synchronize()
    info, iters, berr = plan.results()
    assert not info.any()
    assert np.all(berr <= 1e-12), berr.max()
    assert torch.equal(A.buf, A0)
    for n, Ah, Bh, Xg in zip(ns, As, Bs, B.to_list()):
        assert _berr(Ah, Xg, Bh) <= 1.05e-12, n
        Xr = sla.solve(Ah, Bh)
        cond = np.linalg.cond(Ah, np.inf)
        assert normwise(Xg, Xr) <= 1e-12 * cond * 10, (n, normwise(Xg, Xr), cond)
    assert iters.max() <= 10


def test_mixed_gesv_zero_pivot_reported(gpu):
    """An instance whose binary32 factorisation meets an exactly zero pivot reports info = k + 1,
    gets X = NaN and a NaN backward error; the other instances of the batch are solved."""
    import torch

    from blast_gb300.ragged import MixedGesvPlan, Packed

    rng = np.random.default_rng(8)
    ns = [40, 100, 7, 130]
    As = [rng.standard_normal((n, n)) for n in ns]
    As[1][:, 5] = 0.0  # column 5 is zero: the sixth pivot is exactly zero
    Bs = [rng.standard_normal((n, 1)) for n in ns]
    A = Packed(ns, ns, "cuda")
    A.fill_from(As)
    B = Packed(ns, [1] * len(ns), "cuda")
    B.fill_from(Bs)
    plan = MixedGesvPlan(A, B)
    plan.run()
    torch.cuda.synchronize()
    info, iters, berr = plan.results()
    assert info[1] == 6 and np.isnan(berr[1]) and np.all(np.isnan(B.to_list()[1]))
    for i in (0, 2, 3):
        assert info[i] == 0 and berr[i] <= 1e-12
        assert _berr(As[i], B.to_list()[i], Bs[i]) <= 1.05e-12

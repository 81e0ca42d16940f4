"""Ragged (descriptor) forms of syrkLower, trsm, trmm, the BLAS-2 operations and the adjoints, over
batches of instances of different sizes and layouts (column-major, row-major = BLAST's trans()
view, panel), against the oracle (bit for bit: the descriptor kernels keep the strided kernels'
order of operations) and against the strided entry points. Also: BLAST's trapezoidal potrf
(m > n) and uniform Cholesky batches above n = 64, which the strided entry points hand to the
CTA-per-matrix kernels.

References: dense/Syrk.hpp:15-145, dense/Trsm.hpp:17-66, algorithm/Trmm.hpp:22-310,
dense/Ger.hpp:40-135, dense/Iamax.hpp:66-96, dense/Laswp.hpp:37-43, dense/Swap.hpp:35-44,
dense/Potrf.hpp:66-106.
"""
import numpy as np
import pytest

from helpers import EPS, normwise, spd_batch, to_dev

pytestmark = pytest.mark.gpu

F = np.asfortranarray


class Dev:
    """Device storage for descriptor operands; keeps every buffer alive."""

    def __init__(self):
        import torch

        self.torch = torch
        self.keep = []

    def mat(self, h, layout=0, ps=4):
        """Stores numpy h (r x c) on the device in the given layout; returns the blastgpu_mat record."""
        torch = self.torch
        h = np.asarray(h, dtype=np.float64)
        r, c = h.shape
        if layout == 0:
            buf = h.T.reshape(-1).copy()  # column-major, ld = r
            ld = max(r, 1)
        elif layout == 1:
            buf = h.reshape(-1).copy()  # row-major, ld = c
            ld = max(c, 1)
        else:
            ld = ps * c
            buf = np.full(((r + ps - 1) // ps) * ld + 1, np.nan)
            for i in range(r):
                for j in range(c):
                    buf[(i // ps) * ld + i % ps + j * ps] = h[i, j]
        t = torch.from_numpy(np.ascontiguousarray(buf) if buf.size else np.zeros(1)).cuda()
        self.keep.append((t, r, c, ld, layout, ps))
        return (t.data_ptr(), r, c, ld, layout, ps if layout == 2 else 0, 0)

    def read(self, rec):
        """numpy copy of the matrix a record describes."""
        for t, r, c, ld, layout, ps in self.keep:
            if t.data_ptr() == rec[0]:
                buf = t.cpu().numpy()
                out = np.empty((r, c))
                for i in range(r):
                    for j in range(c):
                        if layout == 0:
                            out[i, j] = buf[i + j * ld]
                        elif layout == 1:
                            out[i, j] = buf[i * ld + j]
                        else:
                            out[i, j] = buf[(i // ps) * ld + i % ps + j * ps]
                return out
        raise KeyError(rec)

    def upload(self, recs):
        from blast_gb300 import desc

        d = desc.upload(recs, "cuda")
        self.keep.append((d, 0, 0, 0, 0, 0))
        return d


def _status(n):
    import torch

    return torch.full((n,), -9, dtype=torch.int32, device="cuda")


def _stream():
    import torch

    return torch.cuda.current_stream().cuda_stream


def test_syrk_lower_batched_ragged_layouts(gpu, oracle_lib):
    import torch

    from blast_gb300 import _lib, desc

    rng = np.random.default_rng(3)
    dev = Dev()
    cases = [(m, k, la, lc) for m in (1, 5, 17, 33) for k in (1, 4, 13) for la, lc in ((0, 0), (1, 0), (2, 2), (1, 2))]
    recs = np.zeros(len(cases), dtype=desc.SYRK_DTYPE)
    hs = []
    for i, (m, k, la, lc) in enumerate(cases):
        A = rng.uniform(-1, 1, (m, k))
        C = rng.uniform(-1, 1, (m, m))
        alpha, beta = (1.0, 1.0) if i % 3 == 0 else (0.7, -1.3)
        rD = dev.mat(np.full((m, m), 5.0), lc)
        recs[i] = (dev.mat(A, la), dev.mat(C, lc), rD, alpha, beta)
        hs.append((A, C, alpha, beta, rD))
    st = _status(len(cases))
    _lib.call("blastgpu_dsyrk_lower_batched", dev.upload(recs).data_ptr(), len(cases), st.data_ptr(), _stream())
    torch.cuda.synchronize()
    assert not st.cpu().numpy().any()
    for (A, C, alpha, beta, rD), (m, k, la, lc) in zip(hs, cases):
        Dr = F(np.full((m, m), 5.0))
        oracle_lib.syrk_lower(alpha, F(A), beta, F(C), Dr)
        D = dev.read(rD)
        assert np.array_equal(np.tril(D), np.tril(Dr)), (m, k, la, lc)
        assert np.all(D[np.triu_indices(m, 1)] == 5.0)  # the strict upper triangle is not written


@pytest.mark.parametrize("side", [0, 1])
def test_trsm_batched_ragged_both_sides(gpu, oracle_lib, side):
    import torch

    from blast_gb300 import _lib, desc

    rng = np.random.default_rng(10 + side)
    for uplo in (0, 1):
        for unit in (0, 1):
            dev = Dev()
            sizes = [(1, 1), (3, 2), (8, 5), (17, 3), (33, 1), (50, 7)]
            recs = np.zeros(len(sizes) * 2, dtype=desc.TRSM_DTYPE)
            hs = []
            for s, (m, n) in enumerate(sizes):
                for view in (0, 1):  # A stored column-major, or its row-major (trans) view
                    ka = m if side == 0 else n
                    T = rng.uniform(-1, 1, (ka, ka)) + ka * np.eye(ka)
                    Av = np.tril(T) if uplo == 0 else np.triu(T)  # the matrix as viewed
                    B = rng.uniform(-1, 1, (m, n))
                    rA = dev.mat(Av, view)
                    rX = dev.mat(B, 0) if s % 2 else None
                    rB = dev.mat(B, 0)
                    recs[2 * s + view] = (rA, rB, rX if rX is not None else rB)  # odd s: out of place
                    hs.append((Av, B, rX if rX is not None else rB))
            st = _status(len(recs))
            _lib.call("blastgpu_dtrsm_batched", side, uplo, unit, dev.upload(recs).data_ptr(), len(recs),
                      st.data_ptr(), _stream())
            torch.cuda.synchronize()
            assert not st.cpu().numpy().any()
            for Av, B, rX in hs:
                Xr = F(np.zeros_like(B))
                if side == 0:
                    oracle_lib.trsm(uplo, unit, F(Av), F(B), Xr)
                else:
                    oracle_lib.trsm_right(uplo, unit, F(Av), F(B), Xr)
                assert np.array_equal(dev.read(rX), Xr), (side, uplo, unit, B.shape)


def test_trmm_batched_all_variants(gpu, oracle_lib):
    import torch

    from blast_gb300 import _lib, desc

    rng = np.random.default_rng(21)
    for side in (0, 1):
        for uplo in (0, 1):
            for unit in (0, 1):
                dev = Dev()
                sizes = [(1, 1), (4, 3), (9, 12), (20, 5)]
                recs = np.zeros(len(sizes), dtype=desc.TRMM_DTYPE)
                hs = []
                for i, (m, n) in enumerate(sizes):
                    ka = m if side == 0 else n
                    A = rng.uniform(-1, 1, (ka, ka))
                    B = rng.uniform(-1, 1, (m, n))
                    alpha = 1.0 if i % 2 else -0.6
                    rC = dev.mat(np.zeros((m, n)), i % 2)
                    recs[i] = (dev.mat(A, (i + 1) % 2), dev.mat(B, 2 if i == 2 else 0), rC, alpha)
                    hs.append((A, B, alpha, rC))
                st = _status(len(sizes))
                _lib.call("blastgpu_dtrmm_batched", side, uplo, unit, dev.upload(recs).data_ptr(), len(sizes),
                          st.data_ptr(), _stream())
                torch.cuda.synchronize()
                assert not st.cpu().numpy().any()
                for A, B, alpha, rC in hs:
                    Cr = F(np.zeros_like(B))
                    oracle_lib.trmm_any(side, uplo, unit, alpha, F(A), F(B), Cr)
                    assert np.array_equal(dev.read(rC), Cr), (side, uplo, unit, B.shape)


def test_blas2_batched(gpu, oracle_lib):
    import torch

    from blast_gb300 import _lib, desc

    rng = np.random.default_rng(5)
    dev = Dev()
    shapes = [(1, 1), (7, 3), (40, 9), (33, 33)]
    # ger, with x a column vector and y a row of a matrix (a 1 x n view)
    recs = np.zeros(len(shapes), dtype=desc.GER_DTYPE)
    hs = []
    for i, (m, n) in enumerate(shapes):
        x = rng.uniform(-1, 1, m)
        Y = rng.uniform(-1, 1, (3, n))
        A = rng.uniform(-1, 1, (m, n))
        rB = dev.mat(np.zeros((m, n)), i % 2)
        recs[i] = (dev.mat(x[:, None]), dev.mat(Y[1:2, :], 1), dev.mat(A, 0), rB, -0.75)
        hs.append((x, Y[1], A, rB))
    st = _status(len(shapes))
    _lib.call("blastgpu_dger_batched", dev.upload(recs).data_ptr(), len(shapes), st.data_ptr(), _stream())
    torch.cuda.synchronize()
    assert not st.cpu().numpy().any()
    for x, y, A, rB in hs:
        Br = F(np.zeros_like(A))
        oracle_lib.ger(-0.75, x, y, F(A), Br)
        assert np.array_equal(dev.read(rB), Br)

    # iamax: ties (first index wins), a leading NaN, row and column vectors; a non-vector gives -1
    vecs = [np.array([1.0, -3.0, 3.0, 2.0]), np.array([np.nan, 5.0, 1.0]), rng.uniform(-1, 1, 77),
            np.array([0.0]), np.array([2.0, np.nan, -2.5])]
    xs = np.zeros(len(vecs) + 1, dtype=desc.MAT_DTYPE)
    for i, v in enumerate(vecs):
        xs[i] = dev.mat(v[None, :], 1) if i % 2 else dev.mat(v[:, None], 0)
    xs[len(vecs)] = dev.mat(np.zeros((2, 2)))
    res = _status(len(xs))
    _lib.call("blastgpu_idamax_batched", dev.upload(xs).data_ptr(), len(xs), res.data_ptr(), _stream())
    torch.cuda.synchronize()
    got = res.cpu().numpy()
    assert list(got[:-1]) == [oracle_lib.idamax(v) for v in vecs] and got[-1] == -1

    # laswp with 0-based pivots; an out-of-range pivot leaves its instance unchanged with status -1
    A = rng.uniform(-1, 1, (6, 4))
    piv = np.array([3, 3, 5, 3, 4, 5], dtype=np.int32)
    rA = dev.mat(A, 1)
    rbad = dev.mat(A, 0)
    p_dev = torch.from_numpy(piv).cuda()
    bad = torch.from_numpy(np.array([0, 9], dtype=np.int32)).cuda()
    recs = np.zeros(2, dtype=desc.LASWP_DTYPE)
    recs[0] = (rA, p_dev.data_ptr(), 1, 5)
    recs[1] = (rbad, bad.data_ptr(), 0, 2)
    st = _status(2)
    _lib.call("blastgpu_dlaswp_batched", dev.upload(recs).data_ptr(), 2, st.data_ptr(), _stream())
    torch.cuda.synchronize()
    Ar = F(A.copy())
    oracle_lib.laswp(Ar, 1, 5, piv)
    assert list(st.cpu().numpy()) == [0, -1]
    assert np.array_equal(dev.read(rA), Ar) and np.array_equal(dev.read(rbad), A)

    # swap a column with a row of another matrix; mismatched lengths give -1
    M = rng.uniform(-1, 1, (5, 5))
    v = rng.uniform(-1, 1, 5)
    rM, rv = dev.mat(M, 0), dev.mat(v[:, None])
    row2 = (rM[0] + 2 * 8, 1, 5, 5, 0, 0, 0)  # row 2 of the column-major M: a 1 x 5 view, ld 5
    recs = np.zeros(2, dtype=desc.SWAP_DTYPE)
    recs[0] = (rv, row2)
    recs[1] = (rv, dev.mat(np.zeros((4, 1))))
    st = _status(2)
    _lib.call("blastgpu_dswap_batched", dev.upload(recs).data_ptr(), 2, st.data_ptr(), _stream())
    torch.cuda.synchronize()
    assert list(st.cpu().numpy()) == [0, -1]
    assert np.array_equal(dev.read(rv)[:, 0], M[2]) and np.array_equal(dev.read(rM)[2], v)


def test_shape_mismatch_reports_status(gpu):
    import torch

    from blast_gb300 import _lib, desc

    dev = Dev()
    recs = np.zeros(2, dtype=desc.TRSM_DTYPE)
    B = np.ones((4, 2))
    recs[0] = (dev.mat(np.eye(4)), dev.mat(B), dev.mat(np.zeros((4, 2))))
    rX = dev.mat(np.full((4, 2), 3.0))
    recs[1] = (dev.mat(np.eye(3)), dev.mat(B), rX)  # A is 3 x 3 for a 4-row B
    st = _status(2)
    _lib.call("blastgpu_dtrsm_batched", 0, 0, 0, dev.upload(recs).data_ptr(), 2, st.data_ptr(), _stream())
    torch.cuda.synchronize()
    assert list(st.cpu().numpy()) == [0, -1]
    assert np.all(dev.read(rX) == 3.0)


def test_adjoints_batched_match_strided(gpu):
    """The descriptor adjoints give the strided adjoints' bits on the same data (uniform batch,
    column-major and transposed views), and numpy's reference gradients on a ragged batch."""
    import torch

    from blast_gb300 import _lib, desc

    rng = np.random.default_rng(8)
    s = _stream()
    batch, m, n, k = 5, 7, 6, 5
    # gemm: D = alpha*A*B^T + beta*C with B given as a transposed view
    A = rng.uniform(-1, 1, (batch, m, k))
    Bt = rng.uniform(-1, 1, (batch, n, k))
    Db = rng.uniform(-1, 1, (batch, m, n))
    dA, dBt, dDb = to_dev(A), to_dev(Bt), to_dev(Db)
    Ab_s, Bb_s, Cb_s = (to_dev(np.zeros(x)) for x in ((batch, m, k), (batch, n, k), (batch, m, n)))
    _lib.call("blastgpu_dgemm_bwd_strided", 0, 1, m, n, k, 0.8, dA.data_ptr(), m, m * k, dBt.data_ptr(), n, n * k,
              -0.5, dDb.data_ptr(), m, m * n, Ab_s.data_ptr(), m, m * k, Bb_s.data_ptr(), n, n * k,
              Cb_s.data_ptr(), m, m * n, batch, s)
    dev = Dev()
    recs = np.zeros(batch, dtype=desc.GEMM_BWD_DTYPE)
    outs = []
    for b in range(batch):
        rAb, rBb, rCb = dev.mat(np.zeros((m, k))), dev.mat(np.zeros((k, n)), 1), dev.mat(np.zeros((m, n)))
        # B as the k x n row-major view of the stored n x k Bt[b]
        recs[b] = (dev.mat(A[b]), dev.mat(Bt[b].T, 1), dev.mat(Db[b]), rAb, rBb, rCb, 0.8, -0.5)
        outs.append((rAb, rBb, rCb))
    st = _status(batch)
    _lib.call("blastgpu_dgemm_bwd_batched", dev.upload(recs).data_ptr(), batch, max(m, n, k), st.data_ptr(), s)
    torch.cuda.synchronize()
    assert not st.cpu().numpy().any()
    for b, (rAb, rBb, rCb) in enumerate(outs):
        assert np.array_equal(dev.read(rAb), Ab_s[b].cpu().numpy())
        assert np.array_equal(dev.read(rBb), Bb_s[b].cpu().numpy().T)
        assert np.array_equal(dev.read(rCb), Cb_s[b].cpu().numpy())

    # trsm: op(A) X = B with op(A) the transposed (upper) view of a lower factor
    Lw = np.tril(rng.uniform(-1, 1, (batch, m, m))) + m * np.eye(m)
    X = rng.uniform(-1, 1, (batch, m, 2))
    Xb = rng.uniform(-1, 1, (batch, m, 2))
    dL, dX, dXb = to_dev(Lw), to_dev(X), to_dev(Xb)
    Bb_s, Ab_s = to_dev(np.zeros((batch, m, 2))), to_dev(np.zeros((batch, m, m)))
    _lib.call("blastgpu_dtrsm_bwd_strided", 1, 1, 0, m, 2, dL.data_ptr(), m, m * m, dX.data_ptr(), m, 2 * m,
              dXb.data_ptr(), m, 2 * m, Bb_s.data_ptr(), m, 2 * m, Ab_s.data_ptr(), m, m * m, batch, s)
    recs = np.zeros(batch, dtype=desc.TRSM_BWD_DTYPE)
    outs = []
    for b in range(batch):
        rBb, rAb = dev.mat(np.zeros((m, 2))), dev.mat(np.zeros((m, m)), 1)
        recs[b] = (dev.mat(Lw[b].T, 1), dev.mat(X[b]), dev.mat(Xb[b]), rBb, rAb)
        outs.append((rBb, rAb))
    st = _status(batch)
    _lib.call("blastgpu_dtrsm_bwd_batched", 1, 0, dev.upload(recs).data_ptr(), batch, st.data_ptr(), s)
    torch.cuda.synchronize()
    assert not st.cpu().numpy().any()
    for b, (rBb, rAb) in enumerate(outs):
        assert np.array_equal(dev.read(rBb), Bb_s[b].cpu().numpy())
        assert np.array_equal(dev.read(rAb).T, Ab_s[b].cpu().numpy())  # Abar in L's storage orientation

    # potrf: ragged sizes against the strided adjoint (one instance at a time) and numpy's gradient
    ns = [1, 4, 9, 16, 30]
    recs = np.zeros(len(ns), dtype=desc.POTRF_BWD_DTYPE)
    hs = []
    for i, nn in enumerate(ns):
        G = rng.uniform(-1, 1, (nn, nn))
        Lc = np.linalg.cholesky(G @ G.T + nn * np.eye(nn))
        Lbar = np.tril(rng.uniform(-1, 1, (nn, nn)))
        rAb = dev.mat(np.zeros((nn, nn)))
        recs[i] = (dev.mat(Lc), dev.mat(Lbar), rAb)
        hs.append((Lc, Lbar, rAb))
    st = _status(len(ns))
    _lib.call("blastgpu_dpotrf_bwd_batched", dev.upload(recs).data_ptr(), len(ns), st.data_ptr(), s)
    torch.cuda.synchronize()
    assert not st.cpu().numpy().any()
    for Lc, Lbar, rAb in hs:
        nn = Lc.shape[0]
        Ab_one = to_dev(np.zeros((1, nn, nn)))
        dLc, dLbar = to_dev(Lc[None]), to_dev(Lbar[None])  # kept alive until the kernel has run
        _lib.call("blastgpu_dpotrf_bwd_strided", nn, dLc.data_ptr(), nn, nn * nn, dLbar.data_ptr(), nn, nn * nn,
                  Ab_one.data_ptr(), nn, nn * nn, 1, s)
        torch.cuda.synchronize()
        got = dev.read(rAb)
        assert np.array_equal(got, Ab_one[0].cpu().numpy())
        # numpy: S = L^-T Phi(L^T Lbar) L^-1, Abar = (S + S^T)/2
        P = np.tril(Lc.T @ Lbar)
        P[np.diag_indices(nn)] *= 0.5
        Li = np.linalg.inv(Lc)
        S = Li.T @ P @ Li
        assert normwise(got, 0.5 * (S + S.T)) <= 1e-10


def test_potrf_trapezoid(gpu, oracle_lib):
    """BLAST's potrf accepts m x n with m >= n (dense/Potrf.hpp:78): strided and descriptor forms,
    column-major and panel storage, against the oracle; m < n is refused."""
    import torch

    from blast_gb300 import _lib, desc
    from oracle import oracle as orc

    rng = np.random.default_rng(17)
    s = _stream()
    for m, n in ((5, 5), (9, 4), (30, 13), (64, 20), (70, 3)):
        batch = 6
        G = rng.standard_normal((batch, m, m))
        A = np.zeros((batch, m, n))
        for b in range(batch):
            S = G[b] @ G[b].T + m * np.eye(m)  # SPD m x m; its first n columns are the trapezoid
            A[b] = S[:, :n]
        dA = to_dev(A)
        dL = to_dev(np.full((batch, m, n), 7.0))
        info = torch.full((batch,), -9, dtype=torch.int32, device="cuda")
        _lib.call("blastgpu_dpotrf_mn_strided", m, n, dA.data_ptr(), m, m * n, dL.data_ptr(), m, m * n,
                  info.data_ptr(), batch, s)
        torch.cuda.synchronize()
        assert not info.cpu().numpy().any()
        L = dL.cpu().numpy()
        for b in range(batch):
            Lr = F(np.zeros((m, n)))
            assert oracle_lib.potrf(F(A[b]), Lr) == 0
            assert normwise(np.tril(L[b]), np.tril(Lr)) <= 10 * m * EPS, (m, n)
            assert np.all(L[b][np.triu_indices(n, 1)] == 7.0)  # the strict upper triangle is not written
        # descriptor form, column-major and AVX2 panels
        for layout, ps in ((0, 0), (2, 4)):
            dev = Dev()
            recs = np.zeros(batch, dtype=desc.POTRF_DTYPE)
            outs = []
            for b in range(batch):
                rL = dev.mat(np.zeros((m, n)), layout, ps or 4)
                recs[b] = (dev.mat(A[b], layout, ps or 4), rL)
                outs.append(rL)
            info.fill_(-9)
            _lib.call("blastgpu_dpotrf_batched", dev.upload(recs).data_ptr(), batch, layout, ps, info.data_ptr(), s)
            torch.cuda.synchronize()
            assert not info.cpu().numpy().any()
            for b in range(batch):
                Lr = F(np.zeros((m, n)))
                if layout == 0:
                    oracle_lib.potrf(F(A[b]), Lr)
                else:
                    sp = 4 * n
                    Ab = np.zeros(((m + 3) // 4) * sp + 1)
                    Lb = np.zeros_like(Ab)
                    for i in range(m):
                        for j in range(n):
                            Ab[(i // 4) * sp + i % 4 + j * 4] = A[b][i, j]
                    orc.lib().oracle_dpotrf_panel(orc.panel_mat(Ab, m, n, 4, sp), orc.panel_mat(Lb, m, n, 4, sp), 4, 16)
                    for i in range(m):
                        for j in range(n):
                            Lr[i, j] = Lb[(i // 4) * sp + i % 4 + j * 4]
                assert normwise(np.tril(dev.read(outs[b])), np.tril(Lr)) <= 10 * m * EPS, (m, n, layout)
    assert _lib.lib().blastgpu_dpotrf_mn_strided(3, 4, None, 3, 0, None, 3, 0, None, 1, None) == -2


@pytest.mark.parametrize("n", [65, 96, 128, 200, 256, 333, 512])
def test_uniform_posv_above_64_runs_cta_kernels(gpu, oracle_lib, n):
    """Uniform batches from n = 65 on go to the CTA-per-matrix kernels through the strided entry
    points (posv, potrf in place, potrs with a given factor), within 10*n*eps of the oracle."""
    import torch

    import blast_gb300 as bg

    rng = np.random.default_rng(n)
    batch, nrhs = 6, 3
    A = spd_batch(rng, batch, n)
    B = rng.standard_normal((batch, n, nrhs))
    dA, dB = to_dev(A), to_dev(B)
    dL = bg.col_major((batch,), n, n, "cuda")
    dL.zero_()
    dX = bg.col_major((batch,), n, nrhs, "cuda")
    info = bg.posv(dA, dL, dB, dX)
    dA2 = to_dev(A)
    info2 = bg.potrf(dA2, dA2)
    dX2 = to_dev(B)
    bg.potrs(dL, dX2, dX2)
    torch.cuda.synchronize()
    assert not info.cpu().numpy().any() and not info2.cpu().numpy().any()
    L, X = np.tril(dL.cpu().numpy()), dX.cpu().numpy()
    L2, X2 = np.tril(dA2.cpu().numpy()), dX2.cpu().numpy()
    assert np.all(np.triu(dL.cpu().numpy(), 1) == 0.0)
    for b in range(batch):
        Lr = F(np.zeros((n, n)))
        assert oracle_lib.potrf(F(A[b]), Lr) == 0
        Xr = F(np.zeros((n, nrhs)))
        oracle_lib.potrs(Lr, F(B[b]), Xr)
        assert normwise(L[b], np.tril(Lr)) <= 10 * n * EPS
        assert np.array_equal(L2[b], L[b])
        assert normwise(X[b], Xr) <= 100 * n * EPS
        assert normwise(X2[b], X[b]) <= 10 * n * EPS

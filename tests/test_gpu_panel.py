"""BLAST's panel storage on the GPU: dense <-> panel conversion (expressions/PanelMatrix.hpp),
panel Cholesky with the AVX2 (panel height 4) and NEON (panel height 2) shapes
(panel/Potrf.hpp:59-106, test/blast/math/panel/PotrfTest.cpp), and gemm on panel operands
(test/blast/math/panel/GemmTest.cpp)."""
import numpy as np
import pytest

from helpers import EPS, approx_equal, normwise, spd_batch, to_dev

pytestmark = pytest.mark.gpu


def _host_panel(a, ps):
    m, n = a.shape
    spacing = ps * n
    buf = np.zeros(((m + ps - 1) // ps) * spacing)
    for i in range(m):
        for j in range(n):
            buf[(i // ps) * spacing + i % ps + j * ps] = a[i, j]
    return buf, spacing


@pytest.mark.parametrize("ps", [2, 4])
def test_dense_panel_roundtrip(gpu, ps):
    import torch

    from blast_gb300 import panel

    rng = np.random.default_rng(ps)
    for m, n in [(1, 1), (5, 3), (7, 9), (24, 24), (33, 17)]:
        A = rng.standard_normal((3, m, n))
        pb = panel.from_dense(to_dev(A), ps)
        raw = pb.buf.cpu().numpy()
        for b in range(3):
            ref, _ = _host_panel(A[b], ps)
            assert np.array_equal(raw[b * pb.stride:b * pb.stride + len(ref)], ref)
        assert np.array_equal(pb.to_numpy(), A)
        out = to_dev(np.zeros((3, m, n)))
        panel.to_dense(pb, out)
        assert np.array_equal(out.cpu().numpy(), A)


@pytest.mark.parametrize("ps,rc", [(4, 16), (2, 32)])
def test_panel_potrf_sweep(gpu, oracle_lib, ps, rc):
    """panel/PotrfTest.cpp:28-49 (M = 0..50): strictly lower output, L*L^T == A, and parity with
    the oracle's panel algorithm of the same shape."""
    from blast_gb300 import panel

    rng = np.random.default_rng(10 + ps)
    for n in list(range(1, 13)) + [17, 24, 31, 48, 50]:
        A = spd_batch(rng, 2, n)
        pa = panel.from_dense(to_dev(A), ps)
        pl = panel.PanelBatch(2, n, n, ps)
        info = panel.potrf(pa, pl).cpu().numpy()
        assert not info.any()
        L = pl.to_numpy()
        for b in range(2):
            assert np.all(np.triu(L[b], 1) == 0)
            assert approx_equal(L[b] @ L[b].T, A[b]), (n, ps)
            buf_a, sp = _host_panel(A[b], ps)
            buf_l = np.zeros_like(buf_a)
            st = oracle_lib.lib().oracle_dpotrf_panel(oracle_lib.panel_mat(buf_a, n, n, ps, sp),
                                                      oracle_lib.panel_mat(buf_l, n, n, ps, sp), ps, rc)
            assert st == 0
            Lr = np.zeros((n, n))
            for i in range(n):
                for j in range(n):
                    Lr[i, j] = buf_l[(i // ps) * sp + i % ps + j * ps]
            assert normwise(L[b], Lr) <= 10 * n * EPS, (n, ps)


@pytest.mark.parametrize("ps", [2, 4])
def test_panel_gemm_nt_bitexact(gpu, oracle_lib, ps):
    """panel/GemmTest.cpp:30-57: D = A*B^T + C on panel operands, M, N, K in 1..20 (sampled),
    through the ragged gemm entry point; per-element order as BLAST's, so bit-identical."""
    import torch

    from blast_gb300 import _lib, desc, panel

    rng = np.random.default_rng(20 + ps)
    sizes = [(m, n, k) for m in (1, 4, 7, 20) for n in (1, 5, 20) for k in (1, 3, 20)]
    recs = np.zeros(len(sizes), dtype=desc.GEMM_DTYPE)
    keep, refs = [], []
    for idx, (m, n, k) in enumerate(sizes):
        A, B, C = rng.random((1, m, k)), rng.random((1, n, k)), rng.random((1, m, n))
        pa, pc = panel.from_dense(to_dev(A), ps), panel.from_dense(to_dev(C), ps)
        pbt = panel.from_dense(to_dev(B), ps)  # B stored as a panel matrix, used transposed
        pd = panel.PanelBatch(1, m, n, ps)
        # B^T as a row-major view would need transposed panels; use B's dense transpose instead
        dBt = to_dev(np.ascontiguousarray(np.swapaxes(B, 1, 2)))
        recs[idx] = (pa.record(0), desc.mat_record(dBt[0]), pc.record(0), pd.record(0), 1.0, 1.0)
        keep += [pa, pc, pbt, pd, dBt]
        Dr = np.zeros((m, n), order="F")
        oracle_lib.gemm(1.0, np.asfortranarray(A[0]), np.asfortranarray(B[0].T), 1.0, np.asfortranarray(C[0]), Dr)
        refs.append(Dr)
    d = desc.upload(recs, "cuda")
    _lib.call("blastgpu_dgemm_batched", d.data_ptr(), len(sizes), 20, 20, 20,
              torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    for (m, n, k), ref, pd in zip(sizes, refs, keep[3::5]):
        assert np.array_equal(pd.to_numpy()[0], ref), (m, n, k)

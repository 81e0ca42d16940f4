"""Pins the CPU oracle (test infrastructure) before it is trusted as the GPU checker.

1. BLAST's own known-answer tests, re-expressed over the oracle with the reference's sizes and
   tolerances (test/blast/math/dense/*Test.cpp, test/blast/math/panel/PotrfTest.cpp).
2. Golden vectors from an independent LAPACK (tests/golden/lapack_golden.npz, made by
   tests/golden/make_golden.py): factors/solutions to 10*n*eps, getrf pivots exactly.
3. Internal consistency: the oracle's fast batch drivers reproduce its per-instance routines bit
   for bit.
"""
from pathlib import Path

import numpy as np
import pytest

from helpers import EPS, approx_equal, normwise, spd

GOLDEN = Path(__file__).resolve().parent / "golden" / "lapack_golden.npz"


@pytest.fixture(scope="module")
def orc(oracle_lib):
    return oracle_lib


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def F(a):
    return np.asfortranarray(a, dtype=np.float64)


# ------------------------------------------------------------------------------------------------
# 1. BLAST's test-suite re-expressed
# ------------------------------------------------------------------------------------------------
def test_gemm_sweep_against_naive(orc):
    """dense/GemmTest.cpp:27-116: m, n, k in 1..20, Cc and Cr (row-major B) variants, compared with
    the naive reference::gemm at 1e-11 (include/test/Tolerance.hpp)."""
    rng = np.random.default_rng(0)
    for m in range(1, 21):
        for n in range(1, 21, 3):
            for k in range(1, 21, 2):
                A, B, C = F(rng.random((m, k))), F(rng.random((k, n))), F(rng.random((m, n)))
                for Bv in (B, np.ascontiguousarray(B)):
                    D, Dn = F(np.zeros((m, n))), F(np.zeros((m, n)))
                    orc.gemm(1.0, A, Bv, 1.0, C, D)
                    orc.gemm_naive(1.0, A, Bv, 1.0, C, Dn)
                    assert approx_equal(D, Dn), (m, n, k)


def test_gemm_unaligned_submatrix_views(orc):
    """dense/GemmTest.cpp:56-88: operands as views at the bottom-right corner of a 20 x 20 parent."""
    rng = np.random.default_rng(1)
    for m, n, k in [(1, 1, 1), (5, 7, 3), (19, 20, 17), (20, 20, 20)]:
        pa, pb, pc, pd = (F(rng.random((20, 20))) for _ in range(4))
        A, B, C, D = pa[20 - m:, 20 - k:], pb[20 - k:, 20 - n:], pc[20 - m:, 20 - n:], pd[20 - m:, 20 - n:]
        orc.gemm(0.5, A, B, 2.0, C, D)
        assert approx_equal(D, 0.5 * A @ B + 2.0 * C)


def test_potrf_sweep_0_to_50(orc):
    """dense/PotrfTest.cpp:26-45: M = 0..50, L*L^T == A at 1e-11."""
    rng = np.random.default_rng(2)
    for n in range(0, 51):
        A = F(spd(rng, n)) if n else F(np.zeros((0, 0)))
        L = F(np.zeros((n, n)))
        assert orc.potrf(A, L) == 0
        assert approx_equal(L @ L.T, A), n
        assert np.all(np.triu(L, 1) == 0)


def test_potrf_in_place(orc):
    """dense/PotrfTest.cpp:67-88: potrf(A, A) with the upper triangle zeroed."""
    rng = np.random.default_rng(3)
    A0 = spd(rng, 3)
    A = F(np.tril(A0))
    assert orc.potrf(A, A) == 0
    assert approx_equal(A @ A.T, A0)


def _panel(a: np.ndarray, ps: int) -> tuple[np.ndarray, int]:
    """Dense -> panel storage (panel/StaticPanelMatrix.hpp:178-184), spacing = ps*cols."""
    m, n = a.shape
    spacing = ps * n
    panels = (m + ps - 1) // ps
    buf = np.zeros(panels * spacing)
    for i in range(m):
        for j in range(n):
            buf[(i // ps) * spacing + i % ps + j * ps] = a[i, j]
    return buf, spacing


def _from_panel(buf, m, n, ps, spacing):
    out = np.zeros((m, n))
    for i in range(m):
        for j in range(n):
            out[i, j] = buf[(i // ps) * spacing + i % ps + j * ps]
    return out


@pytest.mark.parametrize("ss,rc", [(4, 16), (2, 32)])
def test_panel_potrf_sweep(orc, ss, rc):
    """panel/PotrfTest.cpp:28-49 (M = 0..50): L lower-triangular, L*L^T == A. With the AVX2 shape
    (SS = 4, 16 registers, strips of 4) the panel algorithm coincides with the dense one bit for
    bit; with the NEON shape (SS = 2, 32 registers, strips of 2) it differs only in rounding."""
    rng = np.random.default_rng(4)
    for n in range(0, 51, 7):
        A = spd(rng, n) if n else np.zeros((0, 0))
        pa, sp = _panel(A, ss)
        pl, _ = _panel(np.zeros((n, n)), ss)
        st = orc.lib().oracle_dpotrf_panel(orc.panel_mat(pa, n, n, ss, sp), orc.panel_mat(pl, n, n, ss, sp), ss, rc)
        assert st == 0
        L = _from_panel(pl, n, n, ss, sp)
        assert np.all(np.triu(L, 1) == 0)
        assert approx_equal(L @ L.T, A), (n, ss)
        Ld = F(np.zeros((n, n)))
        orc.potrf(F(A), Ld)
        if ss == 4:
            assert np.array_equal(L, Ld)
        else:
            assert normwise(L, Ld) <= 10 * max(n, 1) * EPS


def _lu_restore(LU, ipiv):
    """P*A from the packed factors (GetrfTest.cpp:28-52's luRestore + laswp)."""
    m, n = LU.shape
    k = min(m, n)
    L = np.tril(LU[:, :k], -1) + np.eye(m, k)
    U = np.triu(LU[:k, :])
    return L @ U


def test_getrf_getf2_small_sweep(orc):
    """dense/GetrfTest.cpp:55-82, Getf2Test.cpp:53-80: M, N in 0..5 (and up to 12 to cross the
    blocked path), P*A == L*U with BLAST's laswp."""
    rng = np.random.default_rng(5)
    for m in range(0, 13):
        for n in range(0, 13):
            for routine in (orc.getrf, orc.getf2):
                A = F(rng.random((m, n)))
                LU = A.copy(order="F")
                ipiv = np.zeros(min(m, n), dtype=np.int32)
                assert routine(LU, ipiv) == 0
                PA = A.copy(order="F")
                orc.laswp(PA, 0, min(m, n), ipiv)
                assert approx_equal(_lu_restore(LU, ipiv), PA), (m, n, routine)
                assert np.all((ipiv >= np.arange(len(ipiv))) & (ipiv < max(m, 1)))


def test_getrf_singular(orc):
    """dense/Getf2.hpp:68-69: an exactly-zero pivot is reported ("Matrix is singular")."""
    A = F(np.array([[1.0, 2.0, 3.0], [2.0, 4.0, 6.0], [1.0, 1.0, 1.0]]))
    ipiv = np.zeros(3, dtype=np.int32)
    assert orc.getrf(A, ipiv) == 3 or orc.getrf(F(np.zeros((3, 3))), ipiv) == 1
    assert orc.getrf(F(np.zeros((3, 3))), np.zeros(3, dtype=np.int32)) == 1


@pytest.mark.parametrize("uplo,unit", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_trsm_sweep(orc, uplo, unit):
    """dense/TrsmTest.cpp:14-106: A*X == B at 1e-10, m, n in 1..50 (sampled), X aliasing B."""
    rng = np.random.default_rng(6)
    for m in range(1, 51, 7):
        for n in range(1, 51, 9):
            A = rng.random((m, m)) + np.eye(m)
            At = np.tril(A) if uplo == 0 else np.triu(A)
            if unit:
                np.fill_diagonal(At, 1.0)
            B = F(rng.random((m, n)))
            X = F(np.zeros((m, n)))
            orc.trsm(uplo, unit, F(A), B, X)
            assert approx_equal(At @ X, B, 1e-10, 1e-10), (m, n)
            Xa = B.copy(order="F")
            orc.trsm(uplo, unit, F(A), Xa, Xa)
            assert np.array_equal(Xa, X)


def test_syrk_sweep(orc):
    """dense/SyrkTest.cpp:27-65: D_lower = A*A^T + C_lower at 1e-10, m, k in 1..20."""
    rng = np.random.default_rng(7)
    for m in range(1, 21):
        for k in range(1, 21, 4):
            A = F(rng.random((m, k)))
            C = rng.random((m, m))
            C = F(C + C.T)
            D = F(np.zeros((m, m)))
            orc.syrk_lower(1.0, A, 1.0, C, D)
            ref = np.tril(A @ A.T + C)
            assert approx_equal(D, ref, 1e-10, 1e-10), (m, k)


def test_trmm_sweep(orc):
    """dense/TrmmTest.cpp:15-60: left-upper and right-lower, m, n in 1..20, vs the naive
    reference::trmm (reference/Trmm.hpp:42-130), which reads only the named triangle."""
    rng = np.random.default_rng(8)
    for m in range(1, 21, 3):
        for n in range(1, 21, 3):
            alpha = rng.random()
            A = F(rng.random((m, m)))
            B = F(rng.random((m, n)))
            C = F(np.zeros((m, n)))
            assert orc.trmm(0, 1, 0, alpha, A, B, C) == 0
            assert approx_equal(C, alpha * np.triu(A) @ B, 1e-10, 1e-10)
            A2 = F(rng.random((n, n)))
            B2 = F(rng.random((m, n)))
            C2 = F(np.zeros((m, n)))
            assert orc.trmm(1, 0, 0, alpha, A2, B2, C2) == 0
            assert approx_equal(C2, alpha * B2 @ np.tril(A2), 1e-10, 1e-10)
    # variants BLAST rejects with std::logic_error (algorithm/Trmm.hpp:101-124, 240)
    A = F(np.eye(3))
    assert orc.trmm(0, 0, 0, 1.0, A, A, F(np.zeros((3, 3)))) == -100
    assert orc.trmm(1, 1, 0, 1.0, A, A, F(np.zeros((3, 3)))) == -100
    assert orc.trmm(0, 1, 1, 1.0, A, A, F(np.zeros((3, 3)))) == -100


def test_trmm_any_and_trsm_right_against_numpy(orc):
    """The oracle's extensions beyond BLAST (no reference algorithm, so pinned by the definition):
    every (side, uplo, unit) trmm is alpha * tri(A) * B or alpha * B * tri(A), reading only the
    named triangle (unit: an implicit 1 diagonal); the right-side solve X op(A) = B with op(A)
    triangular (uplo and unit describe op(A))."""
    rng = np.random.default_rng(12)

    def tri(A, uplo, unit):
        T = np.triu(A) if uplo else np.tril(A)
        if unit:
            np.fill_diagonal(T, 1.0)
        return T

    for m, n in [(1, 1), (3, 5), (7, 2), (12, 12), (20, 9)]:
        for side in (0, 1):
            for uplo in (0, 1):
                for unit in (0, 1):
                    k = m if side == 0 else n
                    A = F(rng.random((k, k)) + 9.0 * (1 - unit) * np.eye(k))
                    A_junk = A.copy()  # the other triangle (and a unit diagonal) must not be read
                    other = np.tril_indices(k, -1) if uplo else np.triu_indices(k, 1)
                    A_junk[other] = np.nan
                    if unit:
                        np.fill_diagonal(A_junk, np.nan)
                    B = F(rng.random((m, n)))
                    C = F(np.zeros((m, n)))
                    alpha = float(rng.uniform(0.5, 2))
                    assert orc.trmm_any(side, uplo, unit, alpha, F(A_junk), B, C) == 0
                    want = alpha * (tri(A, uplo, unit) @ B if side == 0 else B @ tri(A, uplo, unit))
                    assert approx_equal(C, want, 1e-12, 1e-12), (m, n, side, uplo, unit)
        for uplo in (0, 1):
            for unit in (0, 1):
                for trans in (0, 1):
                    A = F(rng.random((n, n)) + 4.0 * np.eye(n))
                    B = F(rng.random((m, n)))
                    X = F(np.zeros((m, n)))
                    assert orc.trsm_right(uplo, unit, A, B, X, trans) == 0
                    T = tri(A.T if trans else A, uplo, unit)  # uplo describes op(A), as in BLAST's trsm
                    assert approx_equal(X @ T, B, 1e-12, 1e-12), (m, n, uplo, unit, trans)


def test_laswp_against_numpy(orc):
    """blast::laswp (dense/Laswp.hpp:37-43): for k = k0..k1-1 swap rows k and ipiv[k]."""
    rng = np.random.default_rng(13)
    m, ncols = 17, 6
    for k0, k1 in [(0, 17), (3, 11), (5, 5)]:
        A = F(rng.random((m, ncols)))
        ipiv = np.array([rng.integers(k, m) for k in range(m)], dtype=np.int32)
        want = A.copy()
        for k in range(k0, k1):
            want[[k, ipiv[k]]] = want[[ipiv[k], k]]
        orc.laswp(A, k0, k1, ipiv)
        assert np.array_equal(A, want)


def test_iamax(orc):
    """dense/Iamax.cpp:25-38 plus the scan's tie and NaN rules (dense/Iamax.hpp:82-95)."""
    rng = np.random.default_rng(9)
    for n in range(1, 40):
        x = rng.standard_normal(n)
        i = orc.idamax(x)
        assert np.all(np.abs(x) <= abs(x[i]))
        assert i == int(np.argmax(np.abs(x)))  # first maximum
    assert orc.idamax(np.array([1.0, -3.0, 3.0, 2.0])) == 1
    assert orc.idamax(np.array([np.nan, 5.0])) == 0
    assert orc.idamax(np.array([1.0, np.nan, 0.5])) == 0


# ------------------------------------------------------------------------------------------------
# 2. LAPACK golden vectors
# ------------------------------------------------------------------------------------------------
def test_ger_sweep(orc):
    """blast::ger against A + alpha*x*y^T, sizes of dense/GerTest.cpp (m, n in 1..20, 1e-10)."""
    rng = np.random.default_rng(5)
    for m in range(1, 21):
        for n in range(1, 21):
            x, y, A = rng.random(m), rng.random(n), np.asfortranarray(rng.random((m, n)))
            alpha = float(rng.random())
            B = np.asfortranarray(np.zeros((m, n)))
            orc.ger(alpha, x, y, A, B)
            assert approx_equal(B, A + alpha * np.outer(x, y), 1e-10, 1e-10)
            # b_ij = fma(alpha*x_i, y_j, a_ij): exact for these small dyadic values
    x, y = np.array([0.5, 0.25]), np.array([2.0, 4.0])
    A = np.asfortranarray(np.ones((2, 2)))
    orc.ger(2.0, x, y, A, A)
    assert np.array_equal(A, [[3.0, 5.0], [2.0, 3.0]])


def test_golden_potrf_potrs(orc, golden):
    for n in (1, 2, 4, 5, 13, 24, 48):
        A, Lg = golden[f"potrf_A_{n}"], golden[f"potrf_L_{n}"]
        L = F(np.zeros((n, n)))
        assert orc.potrf(F(A), L) == 0
        assert normwise(L, Lg) <= 10 * n * EPS
        B, Xg = golden[f"potrs_B_{n}"], golden[f"potrs_X_{n}"]
        X = F(np.zeros_like(B))
        orc.potrs(L, F(B), X)
        assert normwise(X, Xg) <= 100 * n * EPS


def test_golden_getrf_pivots_exact(orc, golden):
    for n in (1, 3, 4, 5, 8, 9, 17, 33, 64):
        A, LUg, pg = golden[f"getrf_A_{n}"], golden[f"getrf_LU_{n}"], golden[f"getrf_piv_{n}"]
        LU = F(A)
        ipiv = np.zeros(n, dtype=np.int32)
        assert orc.getrf(LU, ipiv) == 0
        assert np.array_equal(ipiv, pg), n
        assert normwise(LU, LUg) <= 10 * n * EPS
        b, xg = golden[f"getrs_b_{n}"], golden[f"getrs_x_{n}"]
        x = F(b.reshape(n, 1))
        orc.getrs(LU, ipiv, x, x)
        assert normwise(x.ravel(), xg) <= 1000 * n * EPS


def test_golden_gemm_and_trsm(orc, golden):
    for (m, n, k) in ((1, 1, 1), (3, 5, 7), (24, 24, 24), (20, 13, 9)):
        A, B, C = (golden[f"gemm_{x}_{m}_{n}_{k}"] for x in "ABC")
        D = F(np.zeros((m, n)))
        orc.gemm(0.75, F(A), F(B), -0.5, F(C), D)
        assert normwise(D, golden[f"gemm_D_{m}_{n}_{k}"]) <= 10 * k * EPS
    for uplo in (0, 1):
        for unit in (0, 1):
            A, B = golden[f"trsm_A_{uplo}{unit}"], golden[f"trsm_B_{uplo}{unit}"]
            X = F(np.zeros_like(B))
            orc.trsm(uplo, unit, F(A), F(B), X)
            assert normwise(X, golden[f"trsm_X_{uplo}{unit}"]) <= 100 * 17 * EPS


# ------------------------------------------------------------------------------------------------
# 3. Batch drivers == per-instance routines (bitwise)
# ------------------------------------------------------------------------------------------------
def test_posv_batch_matches_single(orc):
    rng = np.random.default_rng(10)
    batch, n, nrhs = 6, 48, 8
    G = rng.standard_normal((batch, n, n))
    A = G @ np.swapaxes(G, 1, 2) + n * np.eye(n)
    B = rng.standard_normal((batch, n, nrhs))
    Lb, Xb, info = orc.posv_batch(A, B, threads=2)
    assert not info.any()
    for b in range(batch):
        L = F(np.zeros((n, n)))
        orc.potrf(F(A[b]), L)
        X = F(np.zeros((n, nrhs)))
        orc.potrs(L, F(B[b]), X)
        assert np.array_equal(np.tril(Lb[b]), L)
        assert np.array_equal(Xb[b], X)


def test_gemm_batch_matches_single(orc):
    rng = np.random.default_rng(11)
    A, B, C = (rng.uniform(-1, 1, (5, 24, 24)) for _ in range(3))
    D = orc.gemm_batch(1.0, A, B, 1.0, C, threads=2)
    for b in range(5):
        Ds = F(np.zeros((24, 24)))
        orc.gemm(1.0, F(A[b]), F(B[b]), 1.0, F(C[b]), Ds)
        assert np.array_equal(D[b], Ds)


def test_gesv_ragged_matches_single(orc):
    rng = np.random.default_rng(12)
    ns = [4, 17, 1, 33, 8]
    As = [rng.standard_normal((n, n)) for n in ns]
    bs = [rng.standard_normal(n) for n in ns]
    LU, xs, pv, info = orc.gesv_ragged(ns, As, bs, threads=2)
    assert not info.any()
    for n, A, b, lu, x, p in zip(ns, As, bs, LU, xs, pv):
        LUs = F(A)
        ip = np.zeros(n, dtype=np.int32)
        orc.getrf(LUs, ip)
        assert np.array_equal(lu, LUs) and np.array_equal(p, ip)
        assert normwise(A @ x, b) <= 1e-12 * n

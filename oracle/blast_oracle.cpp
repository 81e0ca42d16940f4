// CPU oracle: restatement of BLAST's hot-path arithmetic (test infrastructure only).
//
// Build: oracle/Makefile, without -ffast-math and with -ffp-contract=off, so that a fused
// multiply-add happens exactly where this file calls std::fma and nowhere else.
//
// Conventions restated from the reference (paths relative to the reference's include/blast/math):
//  * RegisterMatrix::ger(alpha, a, b) (register_matrix/RegisterMatrix.hpp:610-706) forms
//    ax = alpha*a rounded, then v = fma(ax, b, v).  With alpha = -1 the product is exact, so
//    v = fma(-a, b, v).
//  * fnmadd(x, y, z) (simd/SimdVec.hpp:323-334) is the fused -(x*y)+z == fma(-x, y, z).
//  * Scalar loops `acc -= a*b` in dense/Trsm.hpp:39-65 are contracted to one fused multiply-add
//    by both GCC (default -ffp-contract=fast) and Clang (-ffp-contract=on) on FMA targets, which
//    are the reference's recommended flags (cmake/InitialCache.cmake:2-3); they are restated as
//    fma(-a, b, acc).
#include "blast_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------------------------
// Addressing
// ---------------------------------------------------------------------------------------------
struct Gen {
    double* p;
    int64_t ld;
    int layout, ps;
    explicit Gen(oracle_mat const& m) : p(m.data), ld(m.ld), layout(m.layout), ps(m.ps > 0 ? m.ps : 1) {}
    Gen(double* p_, int64_t ld_) : p(p_), ld(ld_), layout(0), ps(1) {}
    double& operator()(int64_t i, int64_t j) const {
        if (layout == 0) return p[i + j * ld];
        if (layout == 1) return p[i * ld + j];
        return p[(i / ps) * ld + i % ps + j * ps];
    }
};

// Column-major accessor (the fast path of the batch drivers; same arithmetic as Gen).
struct Col {
    double* p;
    int64_t ld;
    double& operator()(int64_t i, int64_t j) const { return p[i + j * ld]; }
};

// Transposed view (BLAST's trans(): expressions/MatTransExpr.hpp:139-160).
template <class A>
struct Trans {
    A a;
    double& operator()(int64_t i, int64_t j) const { return a(j, i); }
};

bool valid(oracle_mat const& m) {
    if (m.rows < 0 || m.cols < 0) return false;
    if (m.rows == 0 || m.cols == 0) return true;
    if (!m.data) return false;
    if (m.layout == 0) return m.ld >= m.rows;
    if (m.layout == 1) return m.ld >= m.cols;
    if (m.layout == 2) return m.ps > 0 && m.ld >= m.ps * m.cols;
    return false;
}

// ---------------------------------------------------------------------------------------------
// gemm: D = alpha*A*B + beta*C
// Per element (register_matrix/Gemm.hpp:71-92): acc = 0; for k ascending acc = fma(a_ik, b_kj, acc);
// acc *= alpha (RegisterMatrix.hpp:102-109); d = fma(beta, c, acc) (axpy, RegisterMatrix.hpp:113-139).
// The tile cover (algorithm/arch/avx2/Tile.hpp:45-139) only decides which register holds which
// element; the per-element order above is the same for every tile shape.
// ---------------------------------------------------------------------------------------------
template <class MA, class MB, class MC, class MD>
void gemm_impl(int M, int N, int K, double alpha, MA A, MB B, double beta, MC C, MD D) {
    constexpr int TM = 12, TN = 4;
    for (int j0 = 0; j0 < N; j0 += TN) {
        int const nj = std::min(TN, N - j0);
        for (int i0 = 0; i0 < M; i0 += TM) {
            int const ni = std::min(TM, M - i0);
            double acc[TN][TM] = {};
            for (int k = 0; k < K; ++k) {
                for (int jj = 0; jj < nj; ++jj) {
                    double const b = B(k, j0 + jj);
                    for (int ii = 0; ii < ni; ++ii)
                        acc[jj][ii] = std::fma(A(i0 + ii, k), b, acc[jj][ii]);
                }
            }
            for (int jj = 0; jj < nj; ++jj)
                for (int ii = 0; ii < ni; ++ii) {
                    double const v = acc[jj][ii] * alpha;
                    D(i0 + ii, j0 + jj) = std::fma(beta, C(i0 + ii, j0 + jj), v);
                }
        }
    }
}

// Column-major fast path with compile-time tile (lets the compiler vectorise the FMAs).
void gemm_col(int M, int N, int K, double alpha, const double* A, int64_t lda, const double* B,
              int64_t ldb, double beta, const double* C, int64_t ldc, double* D, int64_t ldd) {
    constexpr int TM = 12, TN = 4;
    for (int j0 = 0; j0 < N; j0 += TN) {
        int const nj = std::min(TN, N - j0);
        int i0 = 0;
        if (nj == TN) {
            for (; i0 + TM <= M; i0 += TM) {
                double acc[TN][TM] = {};
                for (int k = 0; k < K; ++k) {
                    const double* a = A + i0 + k * lda;
                    for (int jj = 0; jj < TN; ++jj) {
                        double const b = B[k + (j0 + jj) * ldb];
                        for (int ii = 0; ii < TM; ++ii) acc[jj][ii] = std::fma(a[ii], b, acc[jj][ii]);
                    }
                }
                for (int jj = 0; jj < TN; ++jj)
                    for (int ii = 0; ii < TM; ++ii)
                        D[i0 + ii + (j0 + jj) * ldd] =
                            std::fma(beta, C[i0 + ii + (j0 + jj) * ldc], acc[jj][ii] * alpha);
            }
        }
        for (; i0 < M; i0 += TM) {
            int const ni = std::min(TM, M - i0);
            double acc[TN][TM] = {};
            for (int k = 0; k < K; ++k)
                for (int jj = 0; jj < nj; ++jj) {
                    double const b = B[k + (j0 + jj) * ldb];
                    for (int ii = 0; ii < ni; ++ii)
                        acc[jj][ii] = std::fma(A[i0 + ii + k * lda], b, acc[jj][ii]);
                }
            for (int jj = 0; jj < nj; ++jj)
                for (int ii = 0; ii < ni; ++ii)
                    D[i0 + ii + (j0 + jj) * ldd] =
                        std::fma(beta, C[i0 + ii + (j0 + jj) * ldc], acc[jj][ii] * alpha);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Cholesky (left-looking, column strips of width kn).
// dense/Potrf.hpp:66-106 (kn = 4, row tiles 12/8/4 chosen by `i + 2*TS < M`, `i + TS < M`, `i < M`)
// and panel/Potrf.hpp:59-106 (kn = min((RC-4)/3, SS), row tiles 3SS/2SS/SS).
// Per element (r >= c, c in strip [k, k+kn)), following potrf_backend (dense/Potrf.hpp:20-63):
//   s = a_rc;  for l < k: s = fma(-l_rl, l_cl, s)            (ger(-1, ...), :40-41)
//   for j in [k, c): s = fma(-l_cj, l_rj, s)                  (RegisterMatrix::potrf :716-726 /
//                                                              RegisterMatrix::trsm :574-584)
//   rows inside the strip's diagonal tile: l_rc = s / sqrt(s_cc)   (RegisterMatrix.hpp:728-737)
//   rows in later tiles:                   l_rc = s / l_cc          (RegisterMatrix.hpp:586-590)
// where l_cc = s_cc / sqrt(s_cc) is what the diagonal tile stores.
// ---------------------------------------------------------------------------------------------
template <class MA, class ML>
int potrf_impl(int M, int N, MA A, ML L, int kn, int tile) {
    int info = 0;
    std::vector<double> sq(kn);
    for (int k = 0; k < N; k += kn) {
        int const nc = std::min(kn, N - k);
        // Height of the diagonal tile: the first tile of the strip's row loop.
        int diag_rows;
        if (k + 2 * tile < M) diag_rows = 3 * tile;
        else if (k + tile < M) diag_rows = 2 * tile;
        else diag_rows = tile;
        int const diag_end = std::min(M, k + diag_rows);
        for (int cc = 0; cc < nc; ++cc) {
            int const c = k + cc;
            // Column c of the strip, rows c..M-1 (rows above c in the diagonal tile are not stored
            // by storeLower in the dense variant).
            for (int r = c; r < M; ++r) {
                double s = A(r, c);
                for (int l = 0; l < k; ++l) s = std::fma(-L(r, l), L(c, l), s);
                for (int j = k; j < c; ++j) s = std::fma(-L(c, j), L(r, j), s);
                if (r == c) {
                    if (!(s > 0.0) && info == 0) info = c + 1;
                    sq[cc] = std::sqrt(s);
                    L(c, c) = s / sq[cc];
                } else if (r < diag_end) {
                    L(r, c) = s / sq[cc];
                } else {
                    L(r, c) = s / L(c, c);
                }
            }
        }
    }
    return info;
}

// Column-major Cholesky for the batched entry point (oracle_dposv_batch), shaped like BLAST's
// kernel (dense/Potrf.hpp:20-106): per strip of 4 columns, register tiles of KM = 12/8/4 rows
// whose inner loops run over contiguous rows, so the compiler vectorises them the way BLAST's
// SIMD tiles are. Same per-element operations, in the same order, as potrf_impl (tile = kn = 4):
// bitwise identical.
template <int KM>
void potrf_tile_col(int n, int k, int i, int nc, const double* A, int64_t lda, double* L, int64_t ldl,
                    double* sq, bool diag, int& info) {
    double acc[4][KM];
    int const nr = std::min(KM, n - i);
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < KM; ++r)
            acc[c][r] = (c < nc && r < nr) ? A[(i + r) + (k + c) * lda] : 0.0;
    if (nr == KM && nc == 4) {
        for (int l = 0; l < k; ++l) {
            const double* a = L + i + l * ldl;
            double const b0 = L[k + l * ldl], b1 = L[k + 1 + l * ldl];
            double const b2 = L[k + 2 + l * ldl], b3 = L[k + 3 + l * ldl];
            for (int r = 0; r < KM; ++r) {
                double const ar = -a[r];
                acc[0][r] = std::fma(ar, b0, acc[0][r]);
                acc[1][r] = std::fma(ar, b1, acc[1][r]);
                acc[2][r] = std::fma(ar, b2, acc[2][r]);
                acc[3][r] = std::fma(ar, b3, acc[3][r]);
            }
        }
    } else {
        for (int l = 0; l < k; ++l)
            for (int c = 0; c < nc; ++c) {
                double const b = L[k + c + l * ldl];
                for (int r = 0; r < nr; ++r) acc[c][r] = std::fma(-L[i + r + l * ldl], b, acc[c][r]);
            }
    }
    for (int c = 0; c < nc; ++c) {
        for (int j = 0; j < c; ++j) {
            double const lcj = diag ? acc[j][c] : L[(k + c) + (k + j) * ldl];
            for (int r = 0; r < KM; ++r) acc[c][r] = std::fma(-lcj, acc[j][r], acc[c][r]);
        }
        if (diag) {
            double const s = acc[c][c];
            if (!(s > 0.0) && info == 0) info = k + c + 1;
            sq[c] = std::sqrt(s);
            for (int r = 0; r < KM; ++r) acc[c][r] = acc[c][r] / sq[c];
        } else {
            double const d = L[(k + c) + (k + c) * ldl];
            for (int r = 0; r < KM; ++r) acc[c][r] = acc[c][r] / d;
        }
    }
    for (int c = 0; c < nc; ++c)
        for (int r = diag ? c : 0; r < nr; ++r) L[(i + r) + (k + c) * ldl] = acc[c][r];
}

int potrf_col(int n, const double* A, int64_t lda, double* L, int64_t ldl) {
    int info = 0;
    double sq[4];
    for (int k = 0; k < n; k += 4) {
        int const nc = std::min(4, n - k);
        int i = k;
        while (i < n) {
            int const rem = n - i;
            if (rem > 8) { potrf_tile_col<12>(n, k, i, nc, A, lda, L, ldl, sq, i == k, info); i += 12; }
            else if (rem > 4) { potrf_tile_col<8>(n, k, i, nc, A, lda, L, ldl, sq, i == k, info); i += 8; }
            else { potrf_tile_col<4>(n, k, i, nc, A, lda, L, ldl, sq, i == k, info); i += 4; }
        }
    }
    return info;
}

// The two solves of potrs for the batched entry point, vectorised across right-hand sides with a
// row-major scratch copy of X; per element the same order as trsm_impl (dense/Trsm.hpp:39-65).
constexpr int kMaxRhs = 8;
void potrs_col(int n, int nrhs, const double* L, int64_t ldl, const double* B, int64_t ldb,
               double* X, int64_t ldx, double* xr /* n*kMaxRhs scratch */) {
    for (int j0 = 0; j0 < nrhs; j0 += kMaxRhs) {
        int const nj = std::min(kMaxRhs, nrhs - j0);
        for (int i = 0; i < n; ++i) {
            double acc[kMaxRhs];
            for (int j = 0; j < nj; ++j) acc[j] = B[i + (j0 + j) * ldb];
            for (int k = 0; k < i; ++k) {
                double const a = -L[i + k * ldl];
                const double* x = xr + k * kMaxRhs;
                for (int j = 0; j < kMaxRhs; ++j) acc[j] = std::fma(a, x[j], acc[j]);
            }
            double const d = L[i + i * ldl];
            for (int j = 0; j < kMaxRhs; ++j) xr[i * kMaxRhs + j] = j < nj ? acc[j] / d : 0.0;
        }
        for (int i = n; i-- > 0;) {
            double acc[kMaxRhs];
            for (int j = 0; j < kMaxRhs; ++j) acc[j] = xr[i * kMaxRhs + j];
            for (int k = i + 1; k < n; ++k) {
                double const a = -L[k + i * ldl];
                const double* x = xr + k * kMaxRhs;
                for (int j = 0; j < kMaxRhs; ++j) acc[j] = std::fma(a, x[j], acc[j]);
            }
            double const d = L[i + i * ldl];
            for (int j = 0; j < kMaxRhs; ++j) xr[i * kMaxRhs + j] = acc[j] / d;
        }
        for (int j = 0; j < nj; ++j)
            for (int i = 0; i < n; ++i) X[i + (j0 + j) * ldx] = xr[i * kMaxRhs + j];
    }
}

// ---------------------------------------------------------------------------------------------
// trsm (dense/Trsm.hpp:17-66): left side, scalar loops; X may alias B.
//   lower: for i ascending   acc = b_ij; for k < i  acc = fma(-a_ik, x_kj, acc)
//   upper: for i descending  acc = b_ij; for k > i (ascending) acc = fma(-a_ik, x_kj, acc)
//   non-unit: x_ij = acc / a_ii
// ---------------------------------------------------------------------------------------------
template <class MA, class MB, class MX>
void trsm_impl(int uplo, int unit, int M, int N, MA A, MB B, MX X) {
    for (int j = 0; j < N; ++j) {
        if (uplo == 0) {
            for (int i = 0; i < M; ++i) {
                double acc = B(i, j);
                for (int k = 0; k < i; ++k) acc = std::fma(-A(i, k), X(k, j), acc);
                X(i, j) = unit ? acc : acc / A(i, i);
            }
        } else {
            for (int i = M; i-- > 0;) {
                double acc = B(i, j);
                for (int k = i + 1; k < M; ++k) acc = std::fma(-A(i, k), X(k, j), acc);
                X(i, j) = unit ? acc : acc / A(i, i);
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------
// getf2 (dense/Getf2.hpp:52-77) on an m x n block; ipiv block-relative.
// iamax (dense/Iamax.hpp:82-95): first index of the largest |x| with a strict '>' scan.
// ger (dense/Ger.hpp:40-135): b_ij = fma(-x_i, y_j, a_ij).
// Returns the block-relative k+1 of the first exactly-zero pivot, else 0. BLAST throws at that
// point; the oracle stops there too.
// ---------------------------------------------------------------------------------------------
template <class MA>
int iamax_col(int n, MA A, int i0, int j) {
    double value = std::fabs(A(i0, j));
    int index = 0;
    for (int i = 1; i < n; ++i) {
        double const v = std::fabs(A(i0 + i, j));
        if (v > value) { value = v; index = i; }
    }
    return index;
}

template <class MA>
int getf2_impl(int m, int n, MA A, int i0, int j0, int32_t* ipiv) {
    for (int k = 0; k < m && k < n; ++k) {
        int const ip = iamax_col(m - k, A, i0 + k, j0 + k) + k;
        ipiv[k] = ip;
        if (ip != k)
            for (int j = 0; j < n; ++j) std::swap(A(i0 + k, j0 + j), A(i0 + ip, j0 + j));
        double const piv = A(i0 + k, j0 + k);
        if (piv == 0.0) return k + 1;
        for (int i = k + 1; i < m; ++i) A(i0 + i, j0 + k) /= piv;
        for (int j = k + 1; j < n; ++j) {
            double const y = A(i0 + k, j0 + j);
            for (int i = k + 1; i < m; ++i)
                A(i0 + i, j0 + j) = std::fma(-A(i0 + i, j0 + k), y, A(i0 + i, j0 + j));
        }
    }
    return 0;
}

// laswp on columns [c0, c1) (dense/Laswp.hpp:37-43).
template <class MA>
void laswp_impl(MA A, int c0, int c1, int k0, int k1, const int32_t* ipiv) {
    for (int k = k0; k < k1; ++k)
        if (k != ipiv[k])
            for (int j = c0; j < c1; ++j) std::swap(A(k, j), A(ipiv[k], j));
}

// getrf (dense/Getrf.hpp:52-119), NB = TileSize<double> = 4.
template <class MA>
int getrf_impl(int M, int N, MA A, int32_t* ipiv) {
    constexpr int NB = 4;
    int k = 0;
    for (; k + NB < M && k + NB < N; k += NB) {
        int const r = getf2_impl(M - k, NB, A, k, k, ipiv + k);
        for (int i = k; i < k + NB; ++i) ipiv[i] += k;
        if (r) return k + r;
        laswp_impl(A, 0, k, k, k + NB, ipiv);
        laswp_impl(A, k + NB, N, k, k + NB, ipiv);
        // U12 := L11^{-1} A12 (trsm<Lower, unit>, in place)
        for (int j = k + NB; j < N; ++j)
            for (int i = 0; i < NB; ++i) {
                double acc = A(k + i, j);
                for (int q = 0; q < i; ++q) acc = std::fma(-A(k + i, k + q), A(k + q, j), acc);
                A(k + i, j) = acc;
            }
        // A22 := -1 * A21*A12 + 1 * A22 through the gemm path (K = NB):
        // acc over q ascending from 0, acc *= -1, d = fma(1, c, acc).
        for (int j = k + NB; j < N; ++j)
            for (int i = k + NB; i < M; ++i) {
                double acc = 0.0;
                for (int q = 0; q < NB; ++q) acc = std::fma(A(i, k + q), A(k + q, j), acc);
                acc = acc * -1.0;
                A(i, j) = std::fma(1.0, A(i, j), acc);
            }
    }
    if (k < M && k < N) {
        int const r = getf2_impl(M - k, N - k, A, k, k, ipiv + k);
        for (int i = k; i < M && i < N; ++i) ipiv[i] += k;
        if (r) return k + r;
    } else {
        for (int i = k; i < M && i < N; ++i) ipiv[i] += k;
    }
    laswp_impl(A, 0, k, k, std::min(M, N), ipiv);
    return 0;
}

// syrkLower (dense/Syrk.hpp:15-145): v = beta*c (rounded, RegisterMatrix::load(beta, p));
// for k ascending: v = fma(alpha*a_ik, a_jk, v) (ger(alpha, ...)); lower part only.
template <class MA, class MC, class MD>
void syrk_impl(int M, int K, double alpha, MA A, double beta, MC C, MD D) {
    for (int j = 0; j < M; ++j)
        for (int i = j; i < M; ++i) {
            double v = beta * C(i, j);
            for (int k = 0; k < K; ++k) v = std::fma(alpha * A(i, k), A(j, k), v);
            D(i, j) = v;
        }
}

// trmm (algorithm/Trmm.hpp):
//  left upper  (:22-126, RegisterMatrix::trmm :745-791):  c_ij = sum_{k>=i} fma(alpha*a_ik, b_kj, .)
//  right lower (:146-242, RegisterMatrix::trmm :795-880): c_ij = sum_{k>=j} fma(alpha*b_ik, a_kj, .)
// with the sum running over k ascending from 0. The strictly-other triangle of A is not referenced
// (the contract documented in reference/Trmm.hpp:30-40).
template <class MA, class MB, class MC>
void trmm_left_upper(int M, int N, double alpha, MA A, MB B, MC C) {
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < M; ++i) {
            double acc = 0.0;
            for (int k = i; k < M; ++k) acc = std::fma(alpha * A(i, k), B(k, j), acc);
            C(i, j) = acc;
        }
}

template <class MA, class MB, class MC>
void trmm_right_lower(int M, int N, double alpha, MA A, MB B, MC C) {
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < M; ++i) {
            double acc = 0.0;
            for (int k = j; k < N; ++k) acc = std::fma(alpha * B(i, k), A(k, j), acc);
            C(i, j) = acc;
        }
}

template <class ML, class MB, class MX>
void potrs_impl(int n, int nrhs, ML L, MB B, MX X) {
    trsm_impl(0, 0, n, nrhs, L, B, X);
    trsm_impl(1, 0, n, nrhs, Trans<ML>{L}, X, X);
}

template <class MA, class MB, class MX>
void getrs_impl(int n, int nrhs, MA LU, const int32_t* ipiv, MB B, MX X) {
    for (int j = 0; j < nrhs; ++j)
        for (int i = 0; i < n; ++i) X(i, j) = B(i, j);
    laswp_impl(X, 0, nrhs, 0, n, ipiv);
    trsm_impl(0, 1, n, nrhs, LU, X, X);
    trsm_impl(1, 0, n, nrhs, LU, X, X);
}

}  // namespace

extern "C" {

int oracle_dgemm(double alpha, oracle_mat A, oracle_mat B, double beta, oracle_mat C, oracle_mat D) {
    if (!valid(A)) return -2;
    if (!valid(B)) return -3;
    if (!valid(C)) return -5;
    if (!valid(D)) return -6;
    int const M = A.rows, K = A.cols, N = B.cols;
    if (B.rows != K || C.rows != M || C.cols != N || D.rows != M || D.cols != N) return -1;
    gemm_impl(M, N, K, alpha, Gen(A), Gen(B), beta, Gen(C), Gen(D));
    return 0;
}

int oracle_dgemm_naive(double alpha, oracle_mat A, oracle_mat B, double beta, oracle_mat C, oracle_mat D) {
    // reference/Gemm.hpp:46-56: v += a*b (contracted), d = alpha*v + beta*c.
    int const M = A.rows, K = A.cols, N = B.cols;
    if (B.rows != K || C.rows != M || C.cols != N || D.rows != M || D.cols != N) return -1;
    Gen a(A), b(B), c(C), d(D);
    for (int i = 0; i < M; ++i)
        for (int j = 0; j < N; ++j) {
            double v = 0.0;
            for (int k = 0; k < K; ++k) v = std::fma(a(i, k), b(k, j), v);
            d(i, j) = std::fma(alpha, v, beta * c(i, j));
        }
    return 0;
}

int oracle_dsyrk_lower(double alpha, oracle_mat A, double beta, oracle_mat C, oracle_mat D) {
    if (!valid(A)) return -2;
    if (!valid(C)) return -4;
    if (!valid(D)) return -5;
    int const M = A.rows, K = A.cols;
    if (C.rows != M || C.cols != M || D.rows != M || D.cols != M) return -1;
    syrk_impl(M, K, alpha, Gen(A), beta, Gen(C), Gen(D));
    return 0;
}

int oracle_dpotrf(oracle_mat A, oracle_mat L) {
    if (!valid(A)) return -1;
    if (!valid(L)) return -2;
    int const M = A.rows, N = A.cols;
    if (N > M || L.rows != M || L.cols != N) return -1;
    return potrf_impl(M, N, Gen(A), Gen(L), 4, 4);
}

int oracle_dpotrf_panel(oracle_mat A, oracle_mat L, int ss, int rc) {
    if (!valid(A)) return -1;
    if (!valid(L)) return -2;
    int const M = A.rows, N = A.cols;
    if (N > M || L.rows != M || L.cols != N || ss <= 0) return -1;
    int const kn = std::min((rc - 4) / 3, ss);
    if (kn <= 0) return -4;
    int const info = potrf_impl(M, N, Gen(A), Gen(L), kn, ss);
    // BLAST's panel variant stores whole register tiles, so the strict upper part of each diagonal
    // tile receives rounding residues of the symmetric elimination (its test bounds them by the
    // absolute tolerance, test/blast/math/panel/PotrfTest.cpp:40-43). The oracle stores exact zeros.
    Gen l(L);
    for (int k = 0; k < N; k += kn)
        for (int c = k; c < std::min(N, k + kn); ++c)
            for (int r = k; r < c; ++r) l(r, c) = 0.0;
    return info;
}

int oracle_dgetrf(oracle_mat A, int32_t* ipiv) {
    if (!valid(A)) return -1;
    if (A.layout != 0) return -1;  // the row-major overload does not pivot (dense/Getrf.hpp:141-162)
    if (std::min(A.rows, A.cols) > 0 && !ipiv) return -2;
    return getrf_impl(A.rows, A.cols, Gen(A), ipiv);
}

int oracle_dgetf2(oracle_mat A, int32_t* ipiv) {
    if (!valid(A)) return -1;
    if (std::min(A.rows, A.cols) > 0 && !ipiv) return -2;
    return getf2_impl(A.rows, A.cols, Gen(A), 0, 0, ipiv);
}

void oracle_dlaswp(oracle_mat A, int k0, int k1, const int32_t* ipiv) {
    laswp_impl(Gen(A), 0, A.cols, k0, k1, ipiv);
}

int oracle_idamax(int n, const double* x, int incx) {
    if (n <= 0) return -1;
    double value = std::fabs(x[0]);
    int index = 0;
    for (int i = 1; i < n; ++i) {
        double const v = std::fabs(x[(int64_t)i * incx]);
        if (v > value) { value = v; index = i; }
    }
    return index;
}

int oracle_dger(double alpha, const double* x, int incx, const double* y, int incy, oracle_mat A,
                oracle_mat B) {
    if (!valid(A)) return -6;
    if (!valid(B) || B.rows != A.rows || B.cols != A.cols) return -7;
    Gen a(A), b(B);
    for (int j = 0; j < A.cols; ++j) {
        double const yj = y[(int64_t)j * incy];
        for (int i = 0; i < A.rows; ++i) b(i, j) = std::fma(alpha * x[(int64_t)i * incx], yj, a(i, j));
    }
    return 0;
}

int oracle_dtrsm(int uplo, int unit, int trans_a, oracle_mat A, oracle_mat B, oracle_mat X) {
    if (!valid(A)) return -4;
    if (!valid(B)) return -5;
    if (!valid(X)) return -6;
    int const M = B.rows, N = B.cols;
    if (A.rows != M || A.cols != M || X.rows != M || X.cols != N) return -1;
    if (trans_a) trsm_impl(uplo, unit, M, N, Trans<Gen>{Gen(A)}, Gen(B), Gen(X));
    else trsm_impl(uplo, unit, M, N, Gen(A), Gen(B), Gen(X));
    return 0;
}

int oracle_dtrmm(int side, int uplo, int unit, double alpha, oracle_mat A, oracle_mat B, oracle_mat C) {
    if (!valid(A)) return -5;
    if (!valid(B)) return -6;
    if (!valid(C)) return -7;
    int const M = B.rows, N = B.cols;
    if (C.rows != M || C.cols != N) return -1;
    if (unit) return -100;
    if (side == 0) {
        if (uplo != 1) return -100;
        if (A.rows != M || A.cols != M) return -1;
        trmm_left_upper(M, N, alpha, Gen(A), Gen(B), Gen(C));
    } else {
        if (uplo != 0) return -100;
        if (A.rows != N || A.cols != N) return -1;
        trmm_right_lower(M, N, alpha, Gen(A), Gen(B), Gen(C));
    }
    return 0;
}

int oracle_dtrmm_any(int side, int uplo, int unit, double alpha, oracle_mat A, oracle_mat B, oracle_mat C) {
    if (!valid(A)) return -5;
    if (!valid(B)) return -6;
    if (!valid(C)) return -7;
    int const M = B.rows, N = B.cols;
    int const K = side == 0 ? M : N;
    if (C.rows != M || C.cols != N || A.rows != K || A.cols != K) return -1;
    Gen a(A), b(B), c(C);
    auto av = [&](int i, int q) { return (unit && i == q) ? 1.0 : a(i, q); };
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < M; ++i) {
            double acc = 0.0;
            if (side == 0) {
                int const q0 = uplo == 1 ? i : 0, q1 = uplo == 1 ? M : i + 1;
                for (int q = q0; q < q1; ++q) acc = std::fma(alpha * av(i, q), b(q, j), acc);
            } else {
                int const q0 = uplo == 1 ? 0 : j, q1 = uplo == 1 ? j + 1 : N;
                for (int q = q0; q < q1; ++q) acc = std::fma(alpha * b(i, q), av(q, j), acc);
            }
            c(i, j) = acc;
        }
    return 0;
}

int oracle_dtrsm_right(int uplo, int unit, int trans_a, oracle_mat A, oracle_mat B, oracle_mat X) {
    if (!valid(A)) return -4;
    if (!valid(B)) return -5;
    if (!valid(X)) return -6;
    int const M = B.rows, N = B.cols;
    if (A.rows != N || A.cols != N || X.rows != M || X.cols != N) return -1;
    Gen a0(A), b(B), x(X);
    auto a = [&](int q, int j) { return trans_a ? a0(j, q) : a0(q, j); };
    for (int i = 0; i < M; ++i) {
        if (uplo == 1) {
            for (int j = 0; j < N; ++j) {
                double acc = b(i, j);
                for (int q = 0; q < j; ++q) acc = std::fma(-x(i, q), a(q, j), acc);
                x(i, j) = unit ? acc : acc / a(j, j);
            }
        } else {
            for (int j = N; j-- > 0;) {
                double acc = b(i, j);
                for (int q = j + 1; q < N; ++q) acc = std::fma(-x(i, q), a(q, j), acc);
                x(i, j) = unit ? acc : acc / a(j, j);
            }
        }
    }
    return 0;
}

int oracle_dpotrs(oracle_mat L, oracle_mat B, oracle_mat X) {
    int const n = L.rows;
    if (L.cols != n || B.rows != n || X.rows != n || X.cols != B.cols) return -1;
    potrs_impl(n, B.cols, Gen(L), Gen(B), Gen(X));
    return 0;
}

int oracle_dgetrs(oracle_mat LU, const int32_t* ipiv, oracle_mat B, oracle_mat X) {
    int const n = LU.rows;
    if (LU.cols != n || B.rows != n || X.rows != n || X.cols != B.cols) return -1;
    getrs_impl(n, B.cols, Gen(LU), ipiv, Gen(B), Gen(X));
    return 0;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int oracle_dposv_batch(int n, int nrhs, int64_t batch, const double* A, int64_t sa, double* L,
                       const double* B, int64_t sb, double* X, int32_t* info, int threads) {
    if (n < 0 || nrhs < 0 || batch < 0) return -1;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads)
#endif
    for (int64_t b = 0; b < batch; ++b) {
        thread_local std::vector<double> scratch;
        if ((int)scratch.size() < n * kMaxRhs) scratch.resize((size_t)n * kMaxRhs);
        double* l = L + b * sa;
        double* x = X + b * sb;
        int const r = potrf_col(n, A + b * sa, n, l, n);
        if (info) info[b] = r;
        if (nrhs > 0) potrs_col(n, nrhs, l, n, B + b * sb, n, x, n, scratch.data());
    }
    return 0;
}

int oracle_dgemm_batch(int m, int n, int k, double alpha, const double* A, int64_t sa,
                       const double* B, int64_t sb, double beta, const double* C, int64_t sc,
                       double* D, int64_t sd, int64_t batch, int threads) {
    if (m < 0 || n < 0 || k < 0 || batch < 0) return -1;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
#endif
    for (int64_t b = 0; b < batch; ++b)
        gemm_col(m, n, k, alpha, A + b * sa, m, B + b * sb, k, beta, C + b * sc, m, D + b * sd, m);
    return 0;
}

int oracle_dgesv_ragged(int64_t batch, const int32_t* n, const int64_t* offA, double* A,
                        const int64_t* offb, double* b, int32_t* ipiv, const int64_t* offp,
                        int32_t* info, int threads) {
    if (batch < 0) return -1;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
#endif
    for (int64_t i = 0; i < batch; ++i) {
        int const ni = n[i];
        Col a{A + offA[i], ni};
        int32_t* p = ipiv + offp[i];
        int const r = getrf_impl(ni, ni, a, p);
        if (info) info[i] = r;
        if (r == 0) getrs_impl(ni, 1, a, p, Col{b + offb[i], ni}, Col{b + offb[i], ni});
    }
    return 0;
}

}  // extern "C"

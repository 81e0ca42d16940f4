/*
 * CPU oracle for the batched BLAST kernels: a restatement of BLAST's hot-path arithmetic
 * (mkatliar/blast, header-only C++) in plain C++.
 *
 * THIS IS TEST INFRASTRUCTURE. Only the test-suite, the smoke check and the CPU-baseline leg of
 * the benchmark load it. The GPU library never calls it and has no CPU fallback.
 *
 * Every routine reproduces, per output element, the order of rounded operations that BLAST's
 * kernels perform (which products are fused, in which order the sum runs, where the division
 * and the square root happen). Each function cites the reference file:line it restates; the
 * implementation file carries the detailed citations.
 *
 * Parity status: BLAST itself cannot be compiled in this environment (its dependencies Blaze,
 * xsimd and Boost are absent), so the restatement is pinned by (1) the reference's own
 * known-answer tests re-expressed in tests/ (reconstruction, triangularity and naive-kernel
 * comparisons at the reference's tolerances and size sweeps) and (2) LAPACK (SciPy) golden
 * vectors committed under tests/golden/. Bitwise agreement with a BLAST binary is unpinned.
 *
 * Matrix descriptors: element (i, j) of an oracle_mat lives at
 *   column-major (layout 0): data[i + j*ld]
 *   row-major    (layout 1): data[i*ld + j]
 *   panel        (layout 2): data[(i/ps)*ld + i%ps + j*ps]   (ld = panel spacing, ps = panel rows)
 * which are BLAST's dense (dense/StaticMatrix.hpp:152-165) and panel
 * (panel/StaticPanelMatrix.hpp:178-184) addressing formulas.
 */
#ifndef BLAST_ORACLE_H
#define BLAST_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_mat {
    double* data;
    int32_t rows, cols;
    int32_t ld;
    int32_t layout; /* 0 column-major, 1 row-major, 2 panel */
    int32_t ps;     /* panel height for layout 2 */
    int32_t pad_;
} oracle_mat;

/* D = alpha*A*B + beta*C  (algorithm/Gemm.hpp:41-97, register_matrix/Gemm.hpp:64-124). 0 or -k. */
int oracle_dgemm(double alpha, oracle_mat A, oracle_mat B, double beta, oracle_mat C, oracle_mat D);

/* Naive reference gemm used by BLAST's own tests (reference/Gemm.hpp:38-56). */
int oracle_dgemm_naive(double alpha, oracle_mat A, oracle_mat B, double beta, oracle_mat C, oracle_mat D);

/* D_lower = alpha*A*A^T + beta*C_lower (dense/Syrk.hpp:15-145). */
int oracle_dsyrk_lower(double alpha, oracle_mat A, double beta, oracle_mat C, oracle_mat D);

/* Lower Cholesky, dense storage (dense/Potrf.hpp:20-106), ts = BLAST TileSize (4 for double).
 * Returns 0, or j+1 for the first non-positive / NaN pivot (BLAST itself does not check; the
 * factor then holds NaN exactly as BLAST would produce). */
int oracle_dpotrf(oracle_mat A, oracle_mat L);

/* Lower Cholesky, panel storage (panel/Potrf.hpp:23-106); ss = SIMD width, rc = register count. */
int oracle_dpotrf_panel(oracle_mat A, oracle_mat L, int ss, int rc);

/* LU with partial pivoting, column-major (dense/Getrf.hpp:52-119). ipiv: 0-based absolute.
 * Returns 0, or k+1 for the first exactly-zero pivot (BLAST throws "Matrix is singular"). */
int oracle_dgetrf(oracle_mat A, int32_t* ipiv);

/* Unblocked LU (dense/Getf2.hpp:52-77). */
int oracle_dgetf2(oracle_mat A, int32_t* ipiv);

/* Row interchanges ipiv[k0..k1) (dense/Laswp.hpp:37-43). */
void oracle_dlaswp(oracle_mat A, int k0, int k1, const int32_t* ipiv);

/* First index of max |x| (dense/Iamax.hpp:82-95). */
int oracle_idamax(int n, const double* x, int incx);

/* blast::ger (dense/Ger.hpp:40-135 with RegisterMatrix::ger, register_matrix/RegisterMatrix.hpp:
 * 610-628): b_ij = fma(alpha*x_i, y_j, a_ij), alpha*x_i rounded first. B may alias A. */
int oracle_dger(double alpha, const double* x, int incx, const double* y, int incy, oracle_mat A,
                oracle_mat B);

/* Left triangular solve A*X = B, uplo 0 lower / 1 upper, unit 0/1; X may alias B
 * (dense/Trsm.hpp:17-66). trans_a=1 solves with A^T (BLAST's trans() view). */
int oracle_dtrsm(int uplo, int unit, int trans_a, oracle_mat A, oracle_mat B, oracle_mat X);

/* trmm: side 0 = left  C = alpha*A*B (A upper)   (algorithm/Trmm.hpp:93-126)
 *       side 1 = right C = alpha*B*A (A lower)   (algorithm/Trmm.hpp:146-242)
 * Other (side, uplo) pairs and unit diagonals return -100 (BLAST throws std::logic_error). */
int oracle_dtrmm(int side, int uplo, int unit, double alpha, oracle_mat A, oracle_mat B, oracle_mat C);

/* Variants with no reference algorithm (BLAST throws std::logic_error for them,
 * algorithm/Trmm.hpp:101-124, 240; RegisterMatrix.hpp:592-597 for the right-side solve). Defined
 * as the per-element pattern of the implemented ones: trmm accumulates fma(alpha*a_iq, b_qj, .)
 * (left) or fma(alpha*b_iq, a_qj, .) (right) over the triangle's q range ascending, a unit
 * diagonal read as 1; the right solve X op(A) = B substitutes column by column (op(A) upper: j
 * ascending; lower: j descending), acc = fma(-x_iq, a_qj, acc) for q ascending, IEEE division.
 * oracle_dtrmm_any computes every (side, uplo, unit); uplo of the solve refers to op(A). */
int oracle_dtrmm_any(int side, int uplo, int unit, double alpha, oracle_mat A, oracle_mat B, oracle_mat C);
int oracle_dtrsm_right(int uplo, int unit, int trans_a, oracle_mat A, oracle_mat B, oracle_mat X);

/* Composed solves (BLAST has no potrs/getrs; they are trsm sequences):
 * potrs: L*Y = B, L^T*X = Y.   getrs: laswp(B), unit-lower solve, upper solve. X may alias B. */
int oracle_dpotrs(oracle_mat L, oracle_mat B, oracle_mat X);
int oracle_dgetrs(oracle_mat LU, const int32_t* ipiv, oracle_mat B, oracle_mat X);

/* ---- batch drivers: one instance per call, instances spread over threads (OpenMP) ---- */
/* Uniform column-major batch of potrf + potrs (the Cholesky-solve workload).  A: n x n per
 * instance at stride sa, L output (may equal A), B: n x nrhs at stride sb, X output (may equal B). */
int oracle_dposv_batch(int n, int nrhs, int64_t batch, const double* A, int64_t sa, double* L,
                       const double* B, int64_t sb, double* X, int32_t* info, int threads);
int oracle_dgemm_batch(int m, int n, int k, double alpha, const double* A, int64_t sa,
                       const double* B, int64_t sb, double beta, const double* C, int64_t sc,
                       double* D, int64_t sd, int64_t batch, int threads);
/* Ragged LU solve: per instance n[i], A at offset offA[i] (ld = n[i]), b at offb[i]. */
int oracle_dgesv_ragged(int64_t batch, const int32_t* n, const int64_t* offA, double* A,
                        const int64_t* offb, double* b, int32_t* ipiv, const int64_t* offp,
                        int32_t* info, int threads);
int oracle_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif

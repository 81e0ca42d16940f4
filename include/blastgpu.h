/*
 * blastgpu.h - C ABI of the batched GB300 (sm_103a) implementation of BLAST's small-matrix
 * dense kernels (mkatliar/blast, "BLAS Templates").
 *
 * BLAST is a header-only C++ template library: every routine works on ONE matrix in the
 * caller's thread, and reports errors by throwing. This ABI replaces those call sites with
 * batched, stream-ordered entry points:
 *
 *   - plain pointers and sizes only (no C++ or torch types), callable from C, C++ (see
 *     blastgpu/blast.hpp for a shim with BLAST's own function names), Python ctypes, etc.;
 *   - every pointer to matrix data is a DEVICE pointer (the library never copies host data);
 *   - a batch of one instance is the drop-in for one BLAST call; a "strided" entry point takes
 *     a uniform batch (instance b at base + b*stride), a "batched" entry point takes an array of
 *     per-instance descriptors in device memory (ragged batches: every instance its own sizes
 *     and layouts); every operation has a "batched" form;
 *   - every call is asynchronous on the given stream, allocates nothing and never synchronises;
 *   - the return value is a status (0 = success; a negative value -i means argument i, counted
 *     from 1, is invalid, LAPACK style; see blastgpu_status); numerical failures are reported per
 *     instance in an `info` array (LAPACK convention) instead of BLAST's exceptions.
 *
 * Element (i, j) of a blastgpu_mat lives at
 *   BLASTGPU_COL_MAJOR  data[i + j*ld]                         (dense/StaticMatrix.hpp:152-165)
 *   BLASTGPU_ROW_MAJOR  data[i*ld + j]                         (BLAST's trans() views)
 *   BLASTGPU_PANEL      data[(i/ps)*ld + i%ps + j*ps]          (panel/StaticPanelMatrix.hpp:178-184)
 * with ld >= rows (col), >= cols (row), >= ps*cols (panel; BLAST calls it the panel "spacing").
 *
 * All floating-point work is IEEE binary64. Results agree with BLAST's algorithm run on the same
 * inputs to a normwise relative error <= 10*n*eps (most kernels reproduce BLAST's order of fused
 * multiply-adds exactly; divisions by a pivot are done as multiplications by its reciprocal).
 */
#ifndef BLASTGPU_H
#define BLASTGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Opaque CUDA stream handle (identical to cudaStream_t / CUstream). NULL = legacy default stream. */
typedef struct CUstream_st* blastgpu_stream_t;

typedef enum blastgpu_status {
    BLASTGPU_SUCCESS = 0,
    /* -1 ... -99: -(index of the first invalid argument) */
    BLASTGPU_ERR_NOT_IMPLEMENTED = -1001, /* variant BLAST itself rejects with std::logic_error */
    BLASTGPU_ERR_CUDA = -1002,            /* a CUDA launch/runtime error; see blastgpu_last_cuda_error() */
    BLASTGPU_ERR_NO_DEVICE = -1003,       /* no usable sm_103 device */
    BLASTGPU_ERR_TOO_LARGE = -1004        /* a size beyond what the selected kernel supports */
} blastgpu_status;

typedef enum blastgpu_layout {
    BLASTGPU_COL_MAJOR = 0,
    BLASTGPU_ROW_MAJOR = 1,
    BLASTGPU_PANEL = 2
} blastgpu_layout;

typedef enum blastgpu_uplo { BLASTGPU_LOWER = 0, BLASTGPU_UPPER = 1 } blastgpu_uplo;
typedef enum blastgpu_side { BLASTGPU_LEFT = 0, BLASTGPU_RIGHT = 1 } blastgpu_side;

/* One matrix (or a view of one): BLAST's MatrixPointer + its extents. 32 bytes. */
typedef struct blastgpu_mat {
    double* data;     /* device pointer to element (0, 0) */
    int32_t rows;
    int32_t cols;
    int32_t ld;       /* leading dimension / panel spacing, in elements */
    int32_t layout;   /* blastgpu_layout */
    int32_t ps;       /* panel height for BLASTGPU_PANEL (BLAST: SIMD width, 4 on AVX2, 2 on NEON) */
    int32_t reserved; /* must be 0 */
} blastgpu_mat;

/* ---------------------------------------------------------------------------------------------
 * Library information
 * ------------------------------------------------------------------------------------------- */
int blastgpu_version(void);                /* 10000*major + 100*minor + patch */
const char* blastgpu_status_string(int status);
int blastgpu_last_cuda_error(void);        /* cudaError_t of the last BLASTGPU_ERR_CUDA (per thread) */
/* Number of kernels this library has launched since load (all threads); for launch accounting. */
int64_t blastgpu_launch_count(void);

/* Kernel-selection parameters (no BLAST counterpart): the autotuner stores its per-size-bin
 * choices here (process-wide). Keys are documented beside the entry points they affect; an
 * unknown key is stored and ignored. tune_get returns -1 for a key that was never set. */
int blastgpu_tune_set(const char* key, int value);
int blastgpu_tune_get(const char* key, int* value);

/* Diagnostics (no BLAST counterpart). selftest_recip: y[i] = 1/sqrt(x[i]) (which = 0) or 1/x[i]
 * (which = 1) with the library's Newton-Raphson helpers, device arrays. probe_fp64_tflops:
 * measures the device's binary64 FMA throughput (TFLOP/s) on `stream` and synchronises it. */
int blastgpu_selftest_recip(int which, const double* x, double* y, int n, blastgpu_stream_t stream);
int blastgpu_probe_fp64_tflops(double* tflops, blastgpu_stream_t stream);
/* probe_fp64_dmma_tflops: the same measurement for the binary64 tensor-core instruction
 * (mma.sync m8n8k4 f64), so that its rate can be compared with the FMA pipe's on the same GPU. */
int blastgpu_probe_fp64_dmma_tflops(double* tflops, blastgpu_stream_t stream);
/* probe_mma_tflops: the same for the warp-level tensor-core instruction of the mixed path's
 * tensor-core panel update (kind 0: mma.sync m16n8k8 TF32) and its BF16 counterpart (kind 1:
 * m16n8k16), binary32 accumulation. */
int blastgpu_probe_mma_tflops(int kind, double* tflops, blastgpu_stream_t stream);

/* blastgpu_dposv_strided for operands outside device memory: A and B are read in place and L and
 * X written in place, each element once, from/to any memory the GPU can address (pinned host
 * buffers; on hardware-coherent systems such as GB300 any host allocation), so a host-resident batch
 * is solved in one launch without staging copies. The factorisation re-reads its partial results
 * from the device workspaces L_work (n*n doubles per instance) and X_work (n*nrhs per instance),
 * which must be device memory. Same results as blastgpu_dposv_strided, bit for bit.
 * No reference counterpart (BLAST's matrices are host memory by construction). */
int blastgpu_dposv_mirror_strided(int n, int nrhs, const double* A, int lda, int64_t stride_a,
                                  const double* B, int ldb, int64_t stride_b, double* L, int ldl,
                                  int64_t stride_l, double* X, int ldx, int64_t stride_x, double* L_work,
                                  double* X_work, int32_t* info, int64_t batch, blastgpu_stream_t stream);

/* D = chol(beta*C + alpha*op(A)*op(A)^T), lower triangle; op(A) = A (n x k) or, with trans_a = 1,
 * the transpose of a k x n A. The Riccati-recursion kernel that BLAST benchmarks as syrk followed
 * by potrf (bench/blas/SyrkPotrf.cpp:15-40; BLASFEO's dsyrk_dpotrf_ln,
 * include/blasfeo/blasfeo_api/SyrkPotrf.hpp:15-40), fused: the values of syrkLower
 * (dense/Syrk.hpp:15-145) are formed in the factorisation's register tiles, so the result equals
 * blastgpu_dsyrk_lower_strided then blastgpu_dpotrf_strided bit for bit without storing the sum.
 * Reads only the lower triangle of C; D may alias C, not A. info[b] as blastgpu_dpotrf_strided. */
int blastgpu_dsyrk_potrf_strided(int n, int k, int trans_a, double alpha, const double* A, int lda,
                                 int64_t stride_a, double beta, const double* C, int ldc, int64_t stride_c,
                                 double* D, int ldd, int64_t stride_d, int32_t* info, int64_t batch,
                                 blastgpu_stream_t stream);

/* ---------------------------------------------------------------------------------------------
 * BLAS-2 building blocks of BLAST's LU, batched (uniform batches; vectors with increments).
 *   ger:   B = A + alpha*x*y^T, b_ij = fma(alpha*x_i, y_j, a_ij)   (blast::ger, dense/Ger.hpp:40-135);
 *          B may equal A.
 *   iamax: result[b] = first index of the largest |x_i|            (blast::iamax, dense/Iamax.hpp:66-96)
 *   laswp: swap rows k and ipiv[k] of A's ncols columns, k = k0..k1-1 (blast::laswp, dense/Laswp.hpp:37-43)
 *   swap:  exchange vectors x and y                                (blast::swap, dense/Swap.hpp:35-44)
 * trsvLeftLower / trsvLeftUpper (dense/Trsv.hpp:15-68) are blastgpu_dtrsm_strided with n = 1.
 * ------------------------------------------------------------------------------------------- */
int blastgpu_dger_strided(int m, int n, double alpha, const double* x, int incx, int64_t stride_x,
                          const double* y, int incy, int64_t stride_y, const double* A, int lda,
                          int64_t stride_a, double* B, int ldb, int64_t stride_b, int64_t batch,
                          blastgpu_stream_t stream);
int blastgpu_idamax_strided(int n, const double* x, int incx, int64_t stride_x, int32_t* result,
                            int64_t batch, blastgpu_stream_t stream);
int blastgpu_dlaswp_strided(int ncols, double* A, int lda, int64_t stride_a, int k0, int k1,
                            const int32_t* ipiv, int64_t stride_ipiv, int64_t batch,
                            blastgpu_stream_t stream);
int blastgpu_dswap_strided(int n, double* x, int incx, int64_t stride_x, double* y, int incy,
                           int64_t stride_y, int64_t batch, blastgpu_stream_t stream);

/* ---------------------------------------------------------------------------------------------
 * Layout conversion: dst = src element by element, for any pair of layouts (column-major,
 * row-major, panel of height ps). Replaces BLAST's assign() between panel and dense matrices
 * (expressions/PanelMatrix.hpp:63-240). Panel padding rows (beyond `rows`) are not written.
 * status[b] (optional) = 0, or -1 if the instance's shapes differ.
 * ------------------------------------------------------------------------------------------- */
typedef struct blastgpu_copy_desc {
    blastgpu_mat src;
    blastgpu_mat dst;
} blastgpu_copy_desc; /* 64 bytes */

int blastgpu_dcopy_batched(const blastgpu_copy_desc* desc, int64_t batch, int32_t* status,
                           blastgpu_stream_t stream);

/* ---------------------------------------------------------------------------------------------
 * gemm: D = alpha*A*B + beta*C
 * Replaces blast::gemm(alpha, A, B, beta, C, D)        (algorithm/Gemm.hpp:80-97),
 *          blast::gemm(A, B, C, D)                     (algorithm/Gemm.hpp:113-118, alpha=beta=1),
 *          blast::gemm(M, N, K, alpha, pA, pB, beta, pC, pD) (algorithm/Gemm.hpp:41-62).
 * trans_a/trans_b = 1 take A / B as row-major storage (BLAST's trans() view of a column-major
 * matrix).  C may equal D (in place, as getrf's trailing update does, dense/Getrf.hpp:91-101).
 * Per element: acc = sum_k fma(a_ik, b_kj, acc) in ascending k; d = fma(beta, c, alpha*acc).
 * ------------------------------------------------------------------------------------------- */
int blastgpu_dgemm_strided(int trans_a, int trans_b, int m, int n, int k, double alpha,
                           const double* A, int lda, int64_t stride_a,
                           const double* B, int ldb, int64_t stride_b, double beta,
                           const double* C, int ldc, int64_t stride_c,
                           double* D, int ldd, int64_t stride_d,
                           int64_t batch, blastgpu_stream_t stream);

typedef struct blastgpu_gemm_desc {
    blastgpu_mat A, B, C, D;
    double alpha, beta;
} blastgpu_gemm_desc; /* 144 bytes */

/* desc: device array of `batch` descriptors; max_m/max_n/max_k bound every instance's sizes
 * (they select the kernel shape; instances may be smaller). */
int blastgpu_dgemm_batched(const blastgpu_gemm_desc* desc, int64_t batch, int max_m, int max_n,
                           int max_k, blastgpu_stream_t stream);

/* ---------------------------------------------------------------------------------------------
 * syrkLower: D_lower = alpha*A*A^T + beta*C_lower, A m x k, C and D m x m, column-major; only
 * the lower triangle of C is read and of D written. Replaces blast::syrkLower(alpha, A, beta, C, D)
 * (dense/Syrk.hpp:15-145); bit-identical to its order of operations. D may equal C.
 * ------------------------------------------------------------------------------------------- */
int blastgpu_dsyrk_lower_strided(int m, int k, double alpha, const double* A, int lda, int64_t stride_a,
                                 double beta, const double* C, int ldc, int64_t stride_c, double* D,
                                 int ldd, int64_t stride_d, int64_t batch, blastgpu_stream_t stream);

/* trsm: solves op(A)*X = B for X, A m x m triangular (uplo), op(A) = A or A^T (trans_a), unit
 * diagonal if unit = 1, B and X m x n column-major; X may equal B. Replaces
 * blast::trsm<UpLo, UNIT>(A, B, X) (dense/Trsm.hpp:17-66), with trans_a covering BLAST's trans()
 * view of A; bit-identical to BLAST's scalar substitution (IEEE division by the diagonal). */
int blastgpu_dtrsm_strided(int uplo, int trans_a, int unit, int m, int n, const double* A, int lda,
                           int64_t stride_a, const double* B, int ldb, int64_t stride_b, double* X,
                           int ldx, int64_t stride_x, int64_t batch, blastgpu_stream_t stream);

/* trmm: C = alpha*A*B (side = LEFT, A m x m) or C = alpha*B*A (side = RIGHT, A n x n), A triangular
 * (uplo; unit = 1: unit diagonal, not read), B and C m x n column-major; C must not overlap A or B.
 * Replaces blast::trmm(alpha, A, uplo, diag, B, C) and blast::trmm(alpha, B, A, uplo, diag, C)
 * (algorithm/Trmm.hpp:260-310), bit-identical for the variants BLAST implements (left upper, right
 * lower, non-unit). BLAST throws std::logic_error for the others (algorithm/Trmm.hpp:101-124, 240);
 * they are computed here in the same per-element pattern. Only the named triangle of A is read. */
/* Right-side solve X*op(A) = B for X, A n x n triangular (uplo of op(A)), B and X m x n; X may
 * equal B. No BLAST counterpart: RegisterMatrix::trsm leaves this side unimplemented
 * (register_matrix/RegisterMatrix.hpp:592-597). Per row, column substitution with fused
 * multiply-adds in ascending k and IEEE division by the diagonal. */
int blastgpu_dtrsm_right_strided(int uplo, int trans_a, int unit, int m, int n, const double* A, int lda,
                                 int64_t stride_a, const double* B, int ldb, int64_t stride_b, double* X,
                                 int ldx, int64_t stride_x, int64_t batch, blastgpu_stream_t stream);

int blastgpu_dtrmm_strided(int side, int uplo, int unit, int m, int n, double alpha, const double* A,
                           int lda, int64_t stride_a, const double* B, int ldb, int64_t stride_b,
                           double* C, int ldc, int64_t stride_c, int64_t batch, blastgpu_stream_t stream);

/* ---------------------------------------------------------------------------------------------
 * potrf: lower Cholesky factor L of a symmetric positive definite n x n A (only the lower
 * triangle of A is read; the strict upper triangle of L is not written). L may equal A. Uniform
 * batches with n >= posv.cta_min_n (a tuning key: 65 unless set; the GB300 tuning cache that the
 * Python package applies sets 129) run one CTA per matrix in panels of 32 columns
 * (the ragged kernels' factorisation), below that one thread per matrix with BLAST's tiles; both
 * are within 10*n*eps of BLAST's algorithm. The same holds for posv and potrs below.
 * Replaces blast::potrf(A, L) dense (dense/Potrf.hpp:66-106) and panel (panel/Potrf.hpp:59-106).
 * info[b] = 0, or j+1 if the j-th pivot was not positive (BLAST does not check and returns NaNs;
 * the factor is computed the same way and carries the same NaNs). info may be NULL.
 * ------------------------------------------------------------------------------------------- */
int blastgpu_dpotrf_strided(int n, const double* A, int lda, int64_t stride_a,
                            double* L, int ldl, int64_t stride_l, int32_t* info,
                            int64_t batch, blastgpu_stream_t stream);

/* potrf of m x n trapezoids, m >= n: BLAST's potrf(A, L) accepts them (dense/Potrf.hpp:78-105; it
 * throws only for columns(A) > rows(A)): the top n x n block is factored and the m - n rows below
 * it are solved against its factor in the same strips and tiles. A and L are m x n column-major
 * (L may equal A); info as blastgpu_dpotrf_strided. blastgpu_dpotrf_strided is the case m = n. */
int blastgpu_dpotrf_mn_strided(int m, int n, const double* A, int lda, int64_t stride_a, double* L, int ldl,
                               int64_t stride_l, int32_t* info, int64_t batch, blastgpu_stream_t stream);

/* Ragged potrf over descriptors, including BLAST's panel storage. Every descriptor's A and L
 * must have the given layout (BLASTGPU_COL_MAJOR, or BLASTGPU_PANEL with panel height ps = 4
 * (AVX2 panels) or 2 (NEON panels)) and A, L must both be m x n with m >= n (trapezoids as
 * blastgpu_dpotrf_mn_strided); instances that do not get info = -1. The panel variants run
 * BLAST's panel algorithm (panel/Potrf.hpp:59-106): strips of KN = min((RC-4)/3, SS) columns
 * (4 for ps = 4, 2 for ps = 2), row tiles of 3, 2 and 1 panels. */
typedef struct blastgpu_potrf_desc {
    blastgpu_mat A; /* n x n SPD input, lower triangle read */
    blastgpu_mat L; /* n x n factor output (may equal A) */
} blastgpu_potrf_desc; /* 64 bytes */

int blastgpu_dpotrf_batched(const blastgpu_potrf_desc* desc, int64_t batch, int layout, int ps,
                            int32_t* info, blastgpu_stream_t stream);

/* potrf followed by the two triangular solves L*Y = B, L^T*X = Y (BLAST has no potrs; this is
 * potrf + trsm<Lower> + trsm<Upper> on trans(L), dense/Trsm.hpp:17-66), fused in one kernel.
 * B is n x nrhs; X may equal B; L may equal A. */
int blastgpu_dposv_strided(int n, int nrhs, const double* A, int lda, int64_t stride_a,
                           double* L, int ldl, int64_t stride_l,
                           const double* B, int ldb, int64_t stride_b,
                           double* X, int ldx, int64_t stride_x, int32_t* info,
                           int64_t batch, blastgpu_stream_t stream);

/* The two triangular solves alone, given the factor L from potrf. X may equal B. */
int blastgpu_dpotrs_strided(int n, int nrhs, const double* L, int ldl, int64_t stride_l,
                            const double* B, int ldb, int64_t stride_b,
                            double* X, int ldx, int64_t stride_x,
                            int64_t batch, blastgpu_stream_t stream);

/* ---------------------------------------------------------------------------------------------
 * getrf: LU factorisation with partial pivoting, A = P*L*U, of column-major m x n matrices.
 * Replaces blast::getrf(A, ipiv) (dense/Getrf.hpp:52-119; its row-major overload does not pivot
 * and has no counterpart here). ipiv receives min(m, n) 0-based absolute pivot rows (BLAST's
 * size_t ipiv[], here int32). info[b] = 0, or k+1 for the first exactly-zero pivot (BLAST throws
 * std::invalid_argument "Matrix is singular", dense/Getf2.hpp:68-69); A and ipiv of such an
 * instance are unspecified, as after BLAST's exception. Factors and pivots are bit-identical to
 * BLAST's algorithm (same operations in the same order, IEEE division by the pivot).
 * ------------------------------------------------------------------------------------------- */
int blastgpu_dgetrf_strided(int m, int n, double* A, int lda, int64_t stride_a, int32_t* ipiv,
                            int64_t stride_ipiv, int32_t* info, int64_t batch, blastgpu_stream_t stream);

/* getrs: X := A^{-1} X from getrf's factors: laswp(X, ipiv), trsm<Lower, unit>, trsm<Upper>
 * (BLAST has no getrs; dense/Laswp.hpp:37-43 and dense/Trsm.hpp:17-66 in BLAST's order).
 * Instances whose info entry is non-zero are skipped (info may be NULL). */
int blastgpu_dgetrs_strided(int n, int nrhs, const double* LU, int lda, int64_t stride_a,
                            const int32_t* ipiv, int64_t stride_ipiv, double* X, int ldx,
                            int64_t stride_x, const int32_t* info, int64_t batch,
                            blastgpu_stream_t stream);

/* Ragged batches: one descriptor per instance, device-resident. A must be column-major. */
typedef struct blastgpu_getrf_desc {
    blastgpu_mat A;  /* m x n, overwritten by L and U */
    int32_t* ipiv;   /* min(m, n) pivots */
    blastgpu_mat B;  /* n x nrhs right-hand sides, overwritten by X (getrs / gesv only) */
} blastgpu_getrf_desc; /* 72 bytes */

/* max_n bounds every instance's max(m, n) and selects the kernel: one warp per matrix for small
 * sizes, one CTA per matrix above n = 64 (tunable per size bin). */
int blastgpu_dgetrf_batched(const blastgpu_getrf_desc* desc, int32_t* info, int64_t batch,
                            int max_n, blastgpu_stream_t stream);
/* getrs on every instance (BLAST's laswp + trsm<Lower, unit> + trsm<Upper> order); max_n bounds
 * every n (at most 800). Instances with info != 0 are skipped. */
int blastgpu_dgetrs_batched(const blastgpu_getrf_desc* desc, const int32_t* info, int64_t batch, int max_n,
                            blastgpu_stream_t stream);
/* getrf followed by getrs on every instance (two launches on `stream`). */
int blastgpu_dgesv_batched(const blastgpu_getrf_desc* desc, int32_t* info, int64_t batch,
                           int max_n, blastgpu_stream_t stream);

/* Mixed-precision LU solve with iterative refinement (no BLAST counterpart; the mixed-precision
 * form of blastgpu_dposv_mixed_batched applied to getrf/getrs): per instance, A (binary64, read only) is rounded to
 * binary32 in the caller's workspace and factored there by the same blocked partial-pivoting
 * algorithm as blastgpu_dgetrf_batched; X := A^{-1} B (B overwritten) is then refined in binary64
 * (r = b - A x, correction solved with the binary32 factor on r / |r|_inf) until the normwise
 * backward error |r|_inf / (|A|_inf |x|_inf + |b|_inf) <= tol or max_iter corrections. Square
 * matrices with n <= 256. Per instance: info (0, or k+1 of an exactly zero binary32 pivot; such
 * instances get X = NaN and berr = NaN and should be solved with blastgpu_dgesv_batched), iters
 * (corrections, the most over the right-hand sides) and berr (the largest backward error). The
 * pivots are the binary32 factorisation's and may differ from the binary64 ones. */
typedef struct blastgpu_gesv_mixed_desc {
    blastgpu_mat A;     /* n x n general matrix, column-major, binary64; not written */
    int32_t* ipiv;      /* n pivots of the binary32 factorisation (0-based, absolute) */
    blastgpu_mat B;     /* n x nrhs column-major right-hand sides; overwritten by X */
    int64_t ws_offset;  /* byte offset of this instance's scratch in `workspace`
                           (blastgpu_dgesv_mixed_workspace_bytes(n) bytes, 4-byte aligned) */
} blastgpu_gesv_mixed_desc;   /* 80 bytes */

size_t blastgpu_dgesv_mixed_workspace_bytes(int n);
int blastgpu_dgesv_mixed_batched(const blastgpu_gesv_mixed_desc* desc, int64_t batch, int max_n, void* workspace,
                                 double tol, int max_iter, int32_t* info, int32_t* iters, double* berr,
                                 blastgpu_stream_t stream);

/* ---------------------------------------------------------------------------------------------
 * Ragged Cholesky solves, n <= 512, one CTA per matrix, one launch for the whole batch.
 * Per instance: potrf(A, L) (lower triangle of A read), then X = A^{-1} B (X may alias B).
 * ------------------------------------------------------------------------------------------- */
typedef struct blastgpu_posv_desc {
    blastgpu_mat A;     /* n x n SPD, column-major; lower triangle read */
    blastgpu_mat L;     /* n x n column-major factor output (binary64 path); unused by the mixed path */
    blastgpu_mat B;     /* n x nrhs column-major right-hand sides */
    blastgpu_mat X;     /* n x nrhs column-major solutions */
    int64_t ws_offset;  /* mixed path: byte offset of this instance's scratch in `workspace`
                           (blastgpu_dposv_mixed_workspace_bytes(n) bytes, 256-byte aligned) */
} blastgpu_posv_desc;   /* 136 bytes */

/* Binary64 path (BLAST's arithmetic, divisions as reciprocal multiplications). max_n bounds every
 * instance's n and selects the register tiling (n <= 64, 128, 256, 512). */
int blastgpu_dposv_batched(const blastgpu_posv_desc* desc, int64_t batch, int max_n, int32_t* info,
                           blastgpu_stream_t stream);

/* Mixed precision (no BLAST counterpart): binary32 Cholesky factor, binary64 residuals, binary32
 * correction solves, iterated per instance until the normwise backward error
 * |b - A x|_inf / (|A|_inf |x|_inf + |b|_inf) <= tol or max_iter corrections were applied.
 * Outputs per instance: info (binary32 factorisation breakdown, j+1), iters (corrections
 * applied, max over right-hand sides), berr (final backward error, max over right-hand sides).
 * Instances with info != 0 or berr > tol need the binary64 path (the caller re-solves them). */
size_t blastgpu_dposv_mixed_workspace_bytes(int n);
int blastgpu_dposv_mixed_batched(const blastgpu_posv_desc* desc, int64_t batch, int max_n,
                                 void* workspace, double tol, int max_iter, int32_t* info,
                                 int32_t* iters, double* berr, blastgpu_stream_t stream);

/* Allocation-free variant of blastgpu_dposv_mixed_batched (no counterpart in the reference: BLAST
 * allocates nothing because it keeps its work in registers). For callers that cannot allocate
 * device memory when they solve: a model-predictive controller calling the solver from its
 * control loop, where allocation is ruled out after start-up because its latency is unbounded,
 * or a host application that owns every device allocation. The binary32 factors go to a fixed
 * scratch array inside the library's device memory instead of caller workspace:
 *   - capacity BLASTGPU_NOALLOC_SCRATCH_BYTES = 32 MiB, reserved on every GPU that loads the
 *     library until the process exits;
 *   - scratch_bytes states the bytes the descriptors' ws_offset ranges use (max over instances
 *     of ws_offset + blastgpu_dposv_mixed_workspace_bytes(n)); larger than the capacity returns
 *     BLASTGPU_ERR_TOO_LARGE and launches nothing;
 *   - the kernel checks every descriptor's range [ws_offset, ws_offset + 4*n*n) against the
 *     capacity as well: an instance whose range is not inside the array (or whose ws_offset is
 *     not a multiple of 4) is not solved and gets info = -1, iters = 0, berr = NaN, while the
 *     other instances of the batch are solved normally;
 *   - the first call on a device looks up the array's device address (cudaGetSymbolAddress) and
 *     caches it; make that first call before any stream capture. cudaDeviceReset unloads the
 *     library's device code and so invalidates the cached address: after a reset, do not call
 *     this entry point again in the same process;
 *   - every call reuses the same array (nothing in it needs clearing: each factor is written
 *     before it is read), so calls whose kernels overlap on the GPU race: serialise them.
 * No cudaMalloc, cudaFree or allocating library routine is called. Results equal
 * blastgpu_dposv_mixed_batched's. */
#define BLASTGPU_NOALLOC_SCRATCH_BYTES ((size_t)32 << 20)
int blastgpu_dposv_mixed_batched_noalloc(const blastgpu_posv_desc* desc, int64_t batch, int max_n,
                                         size_t scratch_bytes, double tol, int max_iter, int32_t* info,
                                         int32_t* iters, double* berr, blastgpu_stream_t stream);

/* ---------------------------------------------------------------------------------------------
 * Ragged (descriptor) forms of syrkLower, trsm, trmm and the BLAS-2 operations: one device array
 * of per-instance descriptors, every operand a blastgpu_mat view of any layout (column-major,
 * row-major = BLAST's trans() view, panel), so one call takes one instance or a batch of
 * instances of different sizes and layouts. Per element the order of rounded operations is the
 * strided entry point's (bit-identical results). status[b] (optional) = 0, or -1 if the
 * instance's shapes do not fit together (nothing is written for it). A vector operand is a
 * blastgpu_mat with one column (element i at (i, 0)) or one row (element i at (0, i)), so a
 * column or a row of a matrix is a vector view too (BLAST's column()/row(),
 * RowColumnVectorPointer.hpp:179-231).
 * ------------------------------------------------------------------------------------------- */
typedef struct blastgpu_syrk_desc {
    blastgpu_mat A;        /* m x k */
    blastgpu_mat C, D;     /* m x m; lower triangle of C read, of D written; D may equal C */
    double alpha, beta;
} blastgpu_syrk_desc;      /* 112 bytes */
/* Replaces blast::syrkLower(alpha, A, beta, C, D) (dense/Syrk.hpp:15-145). */
int blastgpu_dsyrk_lower_batched(const blastgpu_syrk_desc* desc, int64_t batch, int32_t* status,
                                 blastgpu_stream_t stream);

typedef struct blastgpu_trsm_desc {
    blastgpu_mat A;        /* triangular, m x m (side LEFT) or n x n (side RIGHT), as viewed */
    blastgpu_mat B, X;     /* m x n; X may equal B */
} blastgpu_trsm_desc;      /* 96 bytes */
/* side = LEFT: A*X = B, replaces blast::trsm<UpLo, UNIT>(A, B, X) (dense/Trsm.hpp:17-66);
 * side = RIGHT: X*A = B (no BLAST counterpart, see blastgpu_dtrsm_right_strided). uplo names the
 * triangle of A as viewed (the row-major view of a lower factor is upper: BLAST's
 * trsm<Upper>(trans(L), ..)); unit = 1: unit diagonal, not read. */
int blastgpu_dtrsm_batched(int side, int uplo, int unit, const blastgpu_trsm_desc* desc, int64_t batch,
                           int32_t* status, blastgpu_stream_t stream);

typedef struct blastgpu_trmm_desc {
    blastgpu_mat A;        /* triangular, m x m (LEFT) or n x n (RIGHT) */
    blastgpu_mat B, C;     /* m x n; C must not overlap A or B */
    double alpha;
} blastgpu_trmm_desc;      /* 104 bytes */
/* C = alpha*A*B (LEFT) or alpha*B*A (RIGHT); replaces blast::trmm (algorithm/Trmm.hpp:260-310), all
 * (side, uplo, unit) variants as blastgpu_dtrmm_strided. */
int blastgpu_dtrmm_batched(int side, int uplo, int unit, const blastgpu_trmm_desc* desc, int64_t batch,
                           int32_t* status, blastgpu_stream_t stream);

typedef struct blastgpu_ger_desc {
    blastgpu_mat x, y;     /* vectors of length m and n */
    blastgpu_mat A, B;     /* m x n; B may equal A */
    double alpha;
} blastgpu_ger_desc;       /* 136 bytes */
/* B = A + alpha*x*y^T (blast::ger, dense/Ger.hpp:40-135). */
int blastgpu_dger_batched(const blastgpu_ger_desc* desc, int64_t batch, int32_t* status, blastgpu_stream_t stream);
/* result[b] = first index of the largest |x_i| of vector desc[b] (blast::iamax, dense/Iamax.hpp:66-96),
 * -1 if desc[b] is not a vector. */
int blastgpu_idamax_batched(const blastgpu_mat* desc, int64_t batch, int32_t* result, blastgpu_stream_t stream);

typedef struct blastgpu_laswp_desc {
    blastgpu_mat A;
    const int32_t* ipiv;   /* device pointer; rows k0 .. k1-1 are swapped with ipiv[k] */
    int32_t k0, k1;
} blastgpu_laswp_desc;     /* 48 bytes */
/* blast::laswp (dense/Laswp.hpp:37-43) on every column of A; an instance whose ipiv[k0..k1-1] names
 * a row outside A gets status -1 and is left unchanged. */
int blastgpu_dlaswp_batched(const blastgpu_laswp_desc* desc, int64_t batch, int32_t* status,
                            blastgpu_stream_t stream);

typedef struct blastgpu_swap_desc {
    blastgpu_mat x, y;     /* vectors of the same length */
} blastgpu_swap_desc;      /* 64 bytes */
/* blast::swap (dense/Swap.hpp:35-44). */
int blastgpu_dswap_batched(const blastgpu_swap_desc* desc, int64_t batch, int32_t* status, blastgpu_stream_t stream);

/* ---------------------------------------------------------------------------------------------
 * Adjoints (no BLAST counterpart). For X = A^{-1} B with A SPD and a scalar loss l:
 *   dl/dB = A^{-1} dl/dX,   dl/dA = -(dl/dB X^T + X dl/dB^T) / 2  (symmetrised),
 * from the forward factor L (recompute = 0), or recomputing L from A into the L matrix
 * (recompute = 1, e.g. in caller workspace) when the forward factor was not kept.
 * ------------------------------------------------------------------------------------------- */
typedef struct blastgpu_posv_bwd_desc {
    blastgpu_mat A;     /* n x n SPD input (read only when recompute = 1) */
    blastgpu_mat L;     /* n x n factor: input, or output when recompute = 1 */
    blastgpu_mat X;     /* n x nrhs forward solution */
    blastgpu_mat Xbar;  /* n x nrhs incoming gradient dl/dX */
    blastgpu_mat Bbar;  /* n x nrhs output dl/dB */
    blastgpu_mat Abar;  /* n x n output dl/dA (full symmetric matrix written) */
} blastgpu_posv_bwd_desc; /* 192 bytes */

int blastgpu_dposv_bwd_batched(const blastgpu_posv_bwd_desc* desc, int64_t batch, int max_n,
                               int recompute, int32_t* info, blastgpu_stream_t stream);

/* Adjoint of gemm D = alpha*op(A)*op(B) + beta*C (blastgpu_dgemm_strided's forward arguments):
 * given Dbar = dl/dD (m x n), ACCUMULATES dl/dA into Abar (A's shape and orientation:
 * m x k, or k x m when trans_a), dl/dB into Bbar (k x n, or n x k when trans_b) and dl/dC into
 * Cbar (m x n): op(A)bar += alpha*Dbar*op(B)^T, op(B)bar += alpha*op(A)^T*Dbar,
 * Cbar += beta*Dbar. Zero the outputs first for plain gradients. Abar, Bbar or Cbar may be null
 * (not wanted). Uses blastgpu_dgemm_strided, so each product keeps its ascending-k order.
 * For batch > 1 no output may have batch stride 0 (instances write concurrently). */
int blastgpu_dgemm_bwd_strided(int trans_a, int trans_b, int m, int n, int k, double alpha, const double* A,
                               int lda, int64_t stride_a, const double* B, int ldb, int64_t stride_b, double beta,
                               const double* Dbar, int lddb, int64_t stride_db, double* Abar, int ldab,
                               int64_t stride_ab, double* Bbar, int ldbb, int64_t stride_bb, double* Cbar, int ldcb,
                               int64_t stride_cb, int64_t batch, blastgpu_stream_t stream);

/* Adjoint of trsm op(A)*X = B (blastgpu_dtrsm_strided's forward arguments; uplo and unit describe
 * op(A)): given the solution X and Xbar = dl/dX (m x n), WRITES Bbar = op(A)^{-T} Xbar (Bbar may
 * equal Xbar) and, if Abar is not null, ACCUMULATES -Bbar*X^T on op(A)'s triangle (strictly
 * below/above the diagonal when unit) into Abar in A's own orientation; Abar's other entries are
 * not touched. Bbar must not alias X, A or Abar; for batch > 1 no output may have stride 0. */
int blastgpu_dtrsm_bwd_strided(int uplo, int trans_a, int unit, int m, int n, const double* A, int lda,
                               int64_t stride_a, const double* X, int ldx, int64_t stride_x, const double* Xbar,
                               int ldxb, int64_t stride_xb, double* Bbar, int ldbb, int64_t stride_bb, double* Abar,
                               int ldab, int64_t stride_ab, int64_t batch, blastgpu_stream_t stream);

/* Adjoint of the Cholesky factorisation L = chol(A), lower (blastgpu_dpotrf_strided): given L and
 * Lbar = dl/dL (lower triangles read), WRITES the symmetric gradient Abar = (S + S^T)/2 in full,
 * S = L^{-T} Phi(L^T Lbar) L^{-1}, Phi = lower triangle with the diagonal halved (I. Murray,
 * "Differentiation of the Cholesky decomposition", 2016); the convention of
 * blastgpu_dposv_bwd_batched. Abar must not alias L or Lbar; for batch > 1 its stride is not 0. */
int blastgpu_dpotrf_bwd_strided(int n, const double* L, int ldl, int64_t stride_l, const double* Lbar, int ldlb,
                                int64_t stride_lb, double* Abar, int ldab, int64_t stride_ab, int64_t batch,
                                blastgpu_stream_t stream);

/* Ragged forms of the three adjoints (no BLAST counterpart). Operands are views (A, B as the
 * forward call saw them, so op() is the view), gradients are views in their operand's own
 * orientation; a gradient with data = NULL is not wanted. status as the ragged forms above
 * (-1 also for a transposed product over panel storage, which has no transposed view).
 *   gemm:  Abar += alpha*Dbar*B^T, Bbar += alpha*A^T*Dbar, Cbar += beta*Dbar  (accumulate);
 *          max_dim bounds every instance's m, n and k (it selects the gemm tiling);
 *   trsm:  A*X = B (left, uplo/unit of A as viewed): Bbar = A^{-T}*Xbar (written; may equal Xbar),
 *          Abar -= Bbar*X^T on A's triangle (accumulated; optional);
 *   potrf: Abar = (S + S^T)/2, S = L^{-T} Phi(L^T*Lbar) L^{-1} (written in full). */
typedef struct blastgpu_gemm_bwd_desc {
    blastgpu_mat A, B, Dbar;         /* m x k, k x n, m x n */
    blastgpu_mat Abar, Bbar, Cbar;   /* m x k, k x n, m x n (each optional) */
    double alpha, beta;
} blastgpu_gemm_bwd_desc;            /* 208 bytes */
int blastgpu_dgemm_bwd_batched(const blastgpu_gemm_bwd_desc* desc, int64_t batch, int max_dim, int32_t* status,
                               blastgpu_stream_t stream);

typedef struct blastgpu_trsm_bwd_desc {
    blastgpu_mat A, X, Xbar, Bbar, Abar;   /* m x m, m x n, m x n, m x n, m x m (Abar optional) */
} blastgpu_trsm_bwd_desc;                  /* 160 bytes */
int blastgpu_dtrsm_bwd_batched(int uplo, int unit, const blastgpu_trsm_bwd_desc* desc, int64_t batch,
                               int32_t* status, blastgpu_stream_t stream);

typedef struct blastgpu_potrf_bwd_desc {
    blastgpu_mat L, Lbar, Abar;            /* n x n each; Abar must not alias L or Lbar */
} blastgpu_potrf_bwd_desc;                 /* 96 bytes */
int blastgpu_dpotrf_bwd_batched(const blastgpu_potrf_bwd_desc* desc, int64_t batch, int32_t* status,
                                blastgpu_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* BLASTGPU_H */

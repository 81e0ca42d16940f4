// Batched syrkLower, trsm and trmm, binary64, sm_103a.
//
// References (per element, the order of rounded operations reproduced here):
//  * blast::syrkLower (dense/Syrk.hpp:15-145): v = beta*c_ij (RegisterMatrix::load(beta, C));
//    for k ascending v = fma(alpha*a_ik, a_jk, v) (gemm over ger(alpha, ...)); lower part only.
//  * blast::trsm<UpLo, UNIT> (dense/Trsm.hpp:17-66): scalar substitution per right-hand-side
//    column; lower: i ascending, acc = b_ij; for k < i acc -= a_ik x_kj; upper: i descending,
//    k ascending from i+1; non-unit: x_ij = acc / a_ii. X may alias B. trans(A) is BLAST's
//    transposed view (the potrs backward solve uses trsm<Upper> on trans(L)).
//  * blast::trmm (algorithm/Trmm.hpp:93-242, RegisterMatrix::trmm :745-880):
//    left upper  c_ij = sum_{k>=i} fma(alpha*a_ik, b_kj, .), k ascending from 0-accumulator;
//    right lower c_ij = sum_{k>=j} fma(alpha*b_ik, a_kj, .).
//    BLAST throws std::logic_error for the other (side, uplo) pairs and for unit diagonals
//    (algorithm/Trmm.hpp:101-124, 240); they are computed here in the same pattern: left lower
//    over k = 0..i, right upper over k = 0..j, k ascending, a unit diagonal read as 1.
//  * Right-side triangular solve X op(A) = B (RegisterMatrix.hpp:592-597 leaves it unimplemented;
//    no BLAST counterpart): per row i, op(A) upper: j ascending, acc = b_ij, for k < j ascending
//    acc = fma(-x_ik, a_kj, acc); lower: j descending, k > j ascending; non-unit x_ij = acc / a_jj.
//
// GPU mapping: syrk and trmm run one warp per instance with lanes over output elements (every
// element is an independent chain of fused multiply-adds); trsm runs one thread per
// (instance, right-hand-side column), since each column's substitution is a chain of dependent
// dot products in BLAST's order. Results are bit-identical to BLAST's algorithm.
#include "common.cuh"

namespace blastgpu {
namespace {

struct Strided {
    double* p;
    int ld;
    int64_t stride;
    int layout;  // BLASTGPU_COL_MAJOR or BLASTGPU_ROW_MAJOR
    __device__ __forceinline__ double& at(int64_t b, int i, int j) const {
        double* q = p + b * stride;
        return layout == BLASTGPU_ROW_MAJOR ? q[(int64_t)i * ld + j] : q[i + (int64_t)j * ld];
    }
};

// ALPHA1: alpha is 1, so alpha*a is a exactly and the multiplication is left out (same bits).
template <bool ALPHA1>
__global__ void __launch_bounds__(128) syrk_lower_kernel(int m, int k, double alpha, Strided A, double beta,
                                                         Strided C, Strided D, int64_t batch) {
    int64_t const b = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= batch) return;
    int const total = m * (m + 1) / 2;
    for (int e = lane; e < total; e += 32) {
        // e -> (i, j), i >= j, column by column
        int j = 0, rem = e;
        while (rem >= m - j) { rem -= m - j; ++j; }
        int const i = j + rem;
        double v = beta * C.at(b, i, j);
        for (int q = 0; q < k; ++q) v = fma(ALPHA1 ? A.at(b, i, q) : alpha * A.at(b, i, q), A.at(b, j, q), v);
        D.at(b, i, j) = v;
    }
}

__global__ void __launch_bounds__(128) trsm_kernel(int uplo, int trans_a, int unit, int m, int n,
                                                   Strided A, Strided B, Strided X, int64_t batch) {
    int64_t const t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= batch * n) return;
    int64_t const b = t / n;
    int const j = (int)(t - b * n);
    auto a = [&](int i, int q) -> double { return trans_a ? A.at(b, q, i) : A.at(b, i, q); };
    if (uplo == BLASTGPU_LOWER) {
        for (int i = 0; i < m; ++i) {
            double acc = B.at(b, i, j);
            for (int q = 0; q < i; ++q) acc = fma(-a(i, q), X.at(b, q, j), acc);
            X.at(b, i, j) = unit ? acc : acc / a(i, i);
        }
    } else {
        for (int i = m; i-- > 0;) {
            double acc = B.at(b, i, j);
            for (int q = i + 1; q < m; ++q) acc = fma(-a(i, q), X.at(b, q, j), acc);
            X.at(b, i, j) = unit ? acc : acc / a(i, i);
        }
    }
}

template <bool ALPHA1>
__global__ void __launch_bounds__(128) trmm_kernel(int side, int uplo, int unit, int m, int n, double alpha,
                                                   Strided A, Strided B, Strided C, int64_t batch) {
    int64_t const b = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= batch) return;
    auto a = [&](int i, int q) -> double { return (unit && i == q) ? 1.0 : A.at(b, i, q); };
    bool const upper = uplo == BLASTGPU_UPPER;
    for (int e = lane; e < m * n; e += 32) {
        int const i = e % m, j = e / m;
        double acc = 0.0;
        if (side == BLASTGPU_LEFT) {
            int const q0 = upper ? i : 0, q1 = upper ? m : i + 1;
            for (int q = q0; q < q1; ++q) acc = fma(ALPHA1 ? a(i, q) : alpha * a(i, q), B.at(b, q, j), acc);
        } else {
            int const q0 = upper ? 0 : j, q1 = upper ? j + 1 : n;
            for (int q = q0; q < q1; ++q) acc = fma(ALPHA1 ? B.at(b, i, q) : alpha * B.at(b, i, q), a(q, j), acc);
        }
        C.at(b, i, j) = acc;
    }
}

// X op(A) = B, one thread per (instance, row of X).
__global__ void __launch_bounds__(128) trsm_right_kernel(int uplo, int trans_a, int unit, int m, int n, Strided A,
                                                         Strided B, Strided X, int64_t batch) {
    int64_t const t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= batch * m) return;
    int64_t const b = t / m;
    int const i = (int)(t - b * m);
    auto a = [&](int q, int j) -> double { return trans_a ? A.at(b, j, q) : A.at(b, q, j); };
    if (uplo == BLASTGPU_UPPER) {
        for (int j = 0; j < n; ++j) {
            double acc = B.at(b, i, j);
            for (int q = 0; q < j; ++q) acc = fma(-X.at(b, i, q), a(q, j), acc);
            X.at(b, i, j) = unit ? acc : acc / a(j, j);
        }
    } else {
        for (int j = n; j-- > 0;) {
            double acc = B.at(b, i, j);
            for (int q = j + 1; q < n; ++q) acc = fma(-X.at(b, i, q), a(q, j), acc);
            X.at(b, i, j) = unit ? acc : acc / a(j, j);
        }
    }
}

}  // namespace
}  // namespace blastgpu

namespace blastgpu {

int launch_syrk_lower(int m, int k, int trans_a, double alpha, const double* A, int lda, int64_t sa,
                      double beta, const double* C, int ldc, int64_t sc, double* D, int ldd, int64_t sd,
                      int64_t batch, cudaStream_t s) {
    if (batch == 0 || m == 0) return BLASTGPU_SUCCESS;
    if ((batch + 3) / 4 > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    // op(A) = A^T of a k x m column-major A is the row-major reading of the same storage
    Strided a{const_cast<double*>(A), lda, sa, trans_a ? BLASTGPU_ROW_MAJOR : BLASTGPU_COL_MAJOR};
    Strided c{const_cast<double*>(C), ldc, sc, BLASTGPU_COL_MAJOR};
    Strided d{D, ldd, sd, BLASTGPU_COL_MAJOR};
    if (alpha == 1.0)
        syrk_lower_kernel<true><<<(unsigned)((batch + 3) / 4), 128, 0, s>>>(m, k, alpha, a, beta, c, d, batch);
    else
        syrk_lower_kernel<false><<<(unsigned)((batch + 3) / 4), 128, 0, s>>>(m, k, alpha, a, beta, c, d, batch);
    return check_launch();
}

}  // namespace blastgpu

using namespace blastgpu;

extern "C" {

int blastgpu_dsyrk_lower_strided(int m, int k, double alpha, const double* A, int lda, int64_t stride_a,
                                 double beta, const double* C, int ldc, int64_t stride_c, double* D,
                                 int ldd, int64_t stride_d, int64_t batch, blastgpu_stream_t stream) {
    if (m < 0) return -1;
    if (k < 0) return -2;
    if (m > 0 && k > 0 && !A) return -4;
    if (lda < (m > 0 ? m : 1)) return -5;
    if (m > 0 && !C) return -8;
    if (ldc < (m > 0 ? m : 1)) return -9;
    if (m > 0 && !D) return -11;
    if (ldd < (m > 0 ? m : 1)) return -12;
    if (batch < 0) return -14;
    return launch_syrk_lower(m, k, 0, alpha, A, lda, stride_a, beta, C, ldc, stride_c, D, ldd, stride_d, batch,
                             as_cuda(stream));
}

int blastgpu_dtrsm_strided(int uplo, int trans_a, int unit, int m, int n, const double* A, int lda,
                           int64_t stride_a, const double* B, int ldb, int64_t stride_b, double* X,
                           int ldx, int64_t stride_x, int64_t batch, blastgpu_stream_t stream) {
    if (uplo != BLASTGPU_LOWER && uplo != BLASTGPU_UPPER) return -1;
    if (trans_a != 0 && trans_a != 1) return -2;
    if (unit != 0 && unit != 1) return -3;
    if (m < 0) return -4;
    if (n < 0) return -5;
    if (m > 0 && !A) return -6;
    if (lda < (m > 0 ? m : 1)) return -7;
    if (m > 0 && n > 0 && !B) return -9;
    if (ldb < (m > 0 ? m : 1)) return -10;
    if (m > 0 && n > 0 && !X) return -12;
    if (ldx < (m > 0 ? m : 1)) return -13;
    if (batch < 0) return -15;
    if (batch == 0 || m == 0 || n == 0) return BLASTGPU_SUCCESS;
    int64_t const threads = batch * n;
    if ((threads + 127) / 128 > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    Strided a{const_cast<double*>(A), lda, stride_a, BLASTGPU_COL_MAJOR};
    Strided bb{const_cast<double*>(B), ldb, stride_b, BLASTGPU_COL_MAJOR};
    Strided x{X, ldx, stride_x, BLASTGPU_COL_MAJOR};
    trsm_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, as_cuda(stream)>>>(uplo, trans_a, unit, m, n, a, bb, x, batch);
    return check_launch();
}

int blastgpu_dtrmm_strided(int side, int uplo, int unit, int m, int n, double alpha, const double* A,
                           int lda, int64_t stride_a, const double* B, int ldb, int64_t stride_b,
                           double* C, int ldc, int64_t stride_c, int64_t batch, blastgpu_stream_t stream) {
    if (side != BLASTGPU_LEFT && side != BLASTGPU_RIGHT) return -1;
    if (uplo != BLASTGPU_LOWER && uplo != BLASTGPU_UPPER) return -2;
    if (unit != 0 && unit != 1) return -3;
    if (m < 0) return -4;
    if (n < 0) return -5;
    int const ka = side == BLASTGPU_LEFT ? m : n;
    if (ka > 0 && !A) return -7;
    if (lda < (ka > 0 ? ka : 1)) return -8;
    if (m > 0 && n > 0 && !B) return -10;
    if (ldb < (m > 0 ? m : 1)) return -11;
    if (m > 0 && n > 0 && !C) return -13;
    if (ldc < (m > 0 ? m : 1)) return -14;
    if (batch < 0) return -16;
    if (batch == 0 || m == 0 || n == 0) return BLASTGPU_SUCCESS;
    if ((batch + 3) / 4 > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    Strided a{const_cast<double*>(A), lda, stride_a, BLASTGPU_COL_MAJOR};
    Strided bb{const_cast<double*>(B), ldb, stride_b, BLASTGPU_COL_MAJOR};
    Strided c{C, ldc, stride_c, BLASTGPU_COL_MAJOR};
    unsigned const blocks = (unsigned)((batch + 3) / 4);
    if (alpha == 1.0)
        trmm_kernel<true><<<blocks, 128, 0, as_cuda(stream)>>>(side, uplo, unit, m, n, alpha, a, bb, c, batch);
    else
        trmm_kernel<false><<<blocks, 128, 0, as_cuda(stream)>>>(side, uplo, unit, m, n, alpha, a, bb, c, batch);
    return check_launch();
}

int blastgpu_dtrsm_right_strided(int uplo, int trans_a, int unit, int m, int n, const double* A, int lda,
                                 int64_t stride_a, const double* B, int ldb, int64_t stride_b, double* X,
                                 int ldx, int64_t stride_x, int64_t batch, blastgpu_stream_t stream) {
    if (uplo != BLASTGPU_LOWER && uplo != BLASTGPU_UPPER) return -1;
    if (trans_a != 0 && trans_a != 1) return -2;
    if (unit != 0 && unit != 1) return -3;
    if (m < 0) return -4;
    if (n < 0) return -5;
    if (n > 0 && !A) return -6;
    if (lda < (n > 0 ? n : 1)) return -7;
    if (m > 0 && n > 0 && !B) return -9;
    if (ldb < (m > 0 ? m : 1)) return -10;
    if (m > 0 && n > 0 && !X) return -12;
    if (ldx < (m > 0 ? m : 1)) return -13;
    if (batch < 0) return -15;
    if (batch == 0 || m == 0 || n == 0) return BLASTGPU_SUCCESS;
    int64_t const threads = batch * m;
    if ((threads + 127) / 128 > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    Strided a{const_cast<double*>(A), lda, stride_a, BLASTGPU_COL_MAJOR};
    Strided bb{const_cast<double*>(B), ldb, stride_b, BLASTGPU_COL_MAJOR};
    Strided x{X, ldx, stride_x, BLASTGPU_COL_MAJOR};
    trsm_right_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, as_cuda(stream)>>>(uplo, trans_a, unit, m, n, a,
                                                                                    bb, x, batch);
    return check_launch();
}

}  // extern "C"

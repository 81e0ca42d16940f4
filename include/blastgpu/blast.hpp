// blastgpu/blast.hpp - BLAST's function names and error behaviour over the blastgpu C ABI.
//
// A BLAST call site such as
//     blast::potrf(A, L);                      // dense/Potrf.hpp:66-106
//     blast::gemm(alpha, A, trans(B), beta, C, D);  // algorithm/Gemm.hpp:80-97
// becomes, with the matrices resident on the GPU,
//     blastgpu::potrf(A, L, stream);
//     blastgpu::gemm(alpha, A, trans(B), beta, C, D, stream);
// where A, L, ... are blastgpu::Matrix views of device memory (one instance) or
// blastgpu::Batch views (a uniform batch: instance b starts b*stride elements after the first).
// Sizes are checked as BLAST checks them and reported with the same exception types:
// std::invalid_argument for mismatched sizes or a singular LU pivot, std::logic_error for the
// variants BLAST does not implement. Every call is asynchronous on `stream`; getrf's singular
// pivots are reported per instance in a device array, which check_singular() turns into BLAST's
// exception once the caller has copied it to the host.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../blastgpu.h"

namespace blastgpu {

enum class UpLo { Lower = BLASTGPU_LOWER, Upper = BLASTGPU_UPPER };

// Non-owning view of one column-major (or, for BLAST's trans() views, row-major) device matrix.
struct Matrix {
    double* data = nullptr;
    int rows = 0, cols = 0, ld = 0;
    bool row_major = false;
};

inline Matrix matrix(double* data, int rows, int cols, int ld = -1) {
    return Matrix{data, rows, cols, ld < 0 ? rows : ld, false};
}

// BLAST's trans(): the same storage seen transposed (expressions/MatTransExpr.hpp:139-160).
inline Matrix trans(Matrix m) { return Matrix{m.data, m.cols, m.rows, m.ld, !m.row_major}; }

// BLAST's submatrix() view (views/Submatrix.hpp:234-282).
inline Matrix submatrix(Matrix m, int i, int j, int rows, int cols) {
    if (i < 0 || j < 0 || i + rows > m.rows || j + cols > m.cols)
        throw std::invalid_argument("Invalid submatrix specification");
    std::int64_t const off = m.row_major ? (std::int64_t)i * m.ld + j : i + (std::int64_t)j * m.ld;
    return Matrix{m.data + off, rows, cols, m.ld, m.row_major};
}

// A uniform batch: `count` matrices shaped like `first`, `stride` elements apart.
struct Batch {
    Matrix first;
    std::int64_t stride = 0;
    std::int64_t count = 1;
};

inline Batch batch(Matrix m) { return Batch{m, 0, 1}; }
inline Batch trans(Batch b) { return Batch{trans(b.first), b.stride, b.count}; }

namespace detail {
inline void check(int status, const char* what) {
    if (status == BLASTGPU_SUCCESS) return;
    if (status == BLASTGPU_ERR_NOT_IMPLEMENTED) throw std::logic_error(std::string(what) + ": not implemented");
    if (status < 0 && status > -100)
        throw std::invalid_argument(std::string(what) + ": invalid argument " + std::to_string(-status));
    throw std::runtime_error(std::string(what) + ": " + blastgpu_status_string(status));
}
inline std::int64_t common_count(std::initializer_list<Batch const*> bs) {
    std::int64_t n = 1;
    for (auto* b : bs)
        if (b->count != 1) {
            if (n != 1 && n != b->count) throw std::invalid_argument("Batch sizes do not match");
            n = b->count;
        }
    return n;
}
inline std::int64_t stride_for(Batch const& b, std::int64_t n) { return b.count == n ? b.stride : 0; }
}  // namespace detail

// D = alpha*A*B + beta*C  (blast::gemm, algorithm/Gemm.hpp:80-97)
inline void gemm(double alpha, Batch const& A, Batch const& B, double beta, Batch const& C, Batch const& D,
                 blastgpu_stream_t stream = nullptr) {
    int const M = A.first.rows, N = B.first.cols, K = A.first.cols;
    if (B.first.rows != K) throw std::invalid_argument("Matrix sizes do not match");
    if (C.first.rows != M || C.first.cols != N) throw std::invalid_argument("Matrix sizes do not match");
    if (D.first.rows != M || D.first.cols != N) throw std::invalid_argument("Matrix sizes do not match");
    if (C.first.row_major || D.first.row_major) throw std::logic_error("C and D must be column-major");
    std::int64_t const n = detail::common_count({&A, &B, &C, &D});
    detail::check(blastgpu_dgemm_strided(A.first.row_major, B.first.row_major, M, N, K, alpha, A.first.data,
                                         A.first.ld, detail::stride_for(A, n), B.first.data, B.first.ld,
                                         detail::stride_for(B, n), beta, C.first.data, C.first.ld,
                                         detail::stride_for(C, n), D.first.data, D.first.ld,
                                         detail::stride_for(D, n), n, stream),
                  "gemm");
}

// D = A*B + C  (algorithm/Gemm.hpp:113-118)
inline void gemm(Batch const& A, Batch const& B, Batch const& C, Batch const& D, blastgpu_stream_t stream = nullptr) {
    gemm(1.0, A, B, 1.0, C, D, stream);
}

// L := chol(A), lower (blast::potrf, dense/Potrf.hpp:66-106). info: optional device array.
inline void potrf(Batch const& A, Batch const& L, std::int32_t* info = nullptr, blastgpu_stream_t stream = nullptr) {
    if (A.first.cols > A.first.rows) throw std::invalid_argument("Invalid matrix size");
    if (L.first.rows != A.first.rows || L.first.cols != A.first.cols) throw std::invalid_argument("Invalid matrix size");
    if (A.first.rows != A.first.cols) throw std::logic_error("trapezoidal potrf is not implemented by the batched ABI");
    std::int64_t const n = detail::common_count({&A, &L});
    detail::check(blastgpu_dpotrf_strided(A.first.rows, A.first.data, A.first.ld, detail::stride_for(A, n),
                                          L.first.data, L.first.ld, detail::stride_for(L, n), info, n, stream),
                  "potrf");
}

// Solve A*X = B with A triangular (blast::trsm<UPLO, UNIT>, dense/Trsm.hpp:17-66).
template <UpLo UPLO, bool UNIT>
inline void trsm(Batch const& A, Batch const& B, Batch const& X, blastgpu_stream_t stream = nullptr) {
    int const M = B.first.rows, N = B.first.cols;
    if (A.first.rows != M || A.first.cols != M) throw std::invalid_argument("Invalid argument size");
    if (X.first.rows != M || X.first.cols != N) throw std::invalid_argument("Invalid argument size");
    std::int64_t const n = detail::common_count({&A, &B, &X});
    detail::check(blastgpu_dtrsm_strided(static_cast<int>(UPLO), A.first.row_major, UNIT, M, N, A.first.data,
                                         A.first.ld, detail::stride_for(A, n), B.first.data, B.first.ld,
                                         detail::stride_for(B, n), X.first.data, X.first.ld,
                                         detail::stride_for(X, n), n, stream),
                  "trsm");
}

// D_lower = alpha*A*A^T + beta*C_lower (blast::syrkLower, dense/Syrk.hpp:15-145)
inline void syrkLower(double alpha, Batch const& A, double beta, Batch const& C, Batch const& D,
                      blastgpu_stream_t stream = nullptr) {
    int const M = A.first.rows, K = A.first.cols;
    if (C.first.rows != M || C.first.cols != M || D.first.rows != M || D.first.cols != M)
        throw std::invalid_argument("Matrix sizes do not match");
    std::int64_t const n = detail::common_count({&A, &C, &D});
    detail::check(blastgpu_dsyrk_lower_strided(M, K, alpha, A.first.data, A.first.ld, detail::stride_for(A, n),
                                               beta, C.first.data, C.first.ld, detail::stride_for(C, n),
                                               D.first.data, D.first.ld, detail::stride_for(D, n), n, stream),
                  "syrkLower");
}

// C = alpha*A*B, A triangular (algorithm/Trmm.hpp:260-283). Keeps BLAST's behaviour: the
// variants BLAST does not implement throw std::logic_error (the C ABI computes them).
inline void trmm(double alpha, Batch const& A, UpLo uplo, bool diag, Batch const& B, Batch const& C,
                 blastgpu_stream_t stream = nullptr) {
    if (diag) throw std::logic_error("Unit-triangular matrices support not implemented in trmm()");
    if (uplo != UpLo::Upper)
        throw std::logic_error("Left product with lower-triangular matrices not implemented in trmm()");
    int const M = B.first.rows, N = B.first.cols;
    if (A.first.rows != M || A.first.cols != M) throw std::invalid_argument("Matrix sizes do not match");
    if (C.first.rows != M || C.first.cols != N) throw std::invalid_argument("Matrix sizes do not match");
    std::int64_t const n = detail::common_count({&A, &B, &C});
    detail::check(blastgpu_dtrmm_strided(BLASTGPU_LEFT, static_cast<int>(uplo), diag, M, N, alpha, A.first.data,
                                         A.first.ld, detail::stride_for(A, n), B.first.data, B.first.ld,
                                         detail::stride_for(B, n), C.first.data, C.first.ld,
                                         detail::stride_for(C, n), n, stream),
                  "trmm");
}

// C = alpha*B*A, A triangular (algorithm/Trmm.hpp:287-310); BLAST's exceptions kept as above.
inline void trmm(double alpha, Batch const& B, Batch const& A, UpLo uplo, bool diag, Batch const& C,
                 blastgpu_stream_t stream = nullptr) {
    if (diag) throw std::logic_error("Unit-triangular matrices support not implemented in trmm()");
    if (uplo != UpLo::Lower)
        throw std::logic_error("Right product with upper-triangular matrices not implemented in trmm()");
    int const M = B.first.rows, N = B.first.cols;
    if (A.first.rows != N || A.first.cols != N) throw std::invalid_argument("Matrix sizes do not match");
    if (C.first.rows != M || C.first.cols != N) throw std::invalid_argument("Matrix sizes do not match");
    std::int64_t const n = detail::common_count({&A, &B, &C});
    detail::check(blastgpu_dtrmm_strided(BLASTGPU_RIGHT, static_cast<int>(uplo), diag, M, N, alpha, A.first.data,
                                         A.first.ld, detail::stride_for(A, n), B.first.data, B.first.ld,
                                         detail::stride_for(B, n), C.first.data, C.first.ld,
                                         detail::stride_for(C, n), n, stream),
                  "trmm");
}

// A = P*L*U in place (blast::getrf, dense/Getrf.hpp:52-119); ipiv: device int32, min(m, n) per
// instance at ipiv_stride; info: device int32 per instance (0, or k+1 for the first exactly-zero
// pivot). Copy info to the host and pass it to check_singular() to get BLAST's exception.
inline void getrf(Batch const& A, std::int32_t* ipiv, std::int64_t ipiv_stride, std::int32_t* info,
                  blastgpu_stream_t stream = nullptr) {
    if (A.first.row_major) throw std::logic_error("getrf needs column-major storage");
    detail::check(blastgpu_dgetrf_strided(A.first.rows, A.first.cols, A.first.data, A.first.ld, A.stride, ipiv,
                                          ipiv_stride, info, A.count, stream),
                  "getrf");
}

// ---- BLAS-2 building blocks ------------------------------------------------------------------
// A vector: size elements at data[i*inc]; a batch of vectors repeats it every `stride` doubles.
struct Vector {
    double* data;
    int size;
    int inc;
};
inline Vector vector(double* data, int size, int inc = 1) { return Vector{data, size, inc}; }
struct VectorBatch {
    Vector first;
    std::int64_t stride;  // doubles between consecutive instances (0: one vector shared by all)
    std::int64_t count;
};
inline VectorBatch batch(Vector v) { return VectorBatch{v, 0, 1}; }

namespace detail {
inline std::int64_t vstride_for(VectorBatch const& b, std::int64_t n) { return b.count == n ? b.stride : 0; }
inline std::int64_t max_count(std::initializer_list<std::int64_t> cs) {
    std::int64_t n = 1;
    for (auto c : cs) n = c > n ? c : n;
    for (auto c : cs)
        if (c != 1 && c != n) throw std::invalid_argument("Batch sizes do not match");
    return n;
}
inline Batch as_column(VectorBatch const& v) {
    if (v.first.inc != 1) throw std::logic_error("trsv needs unit-stride vectors");
    return Batch{Matrix{v.first.data, v.first.size, 1, v.first.size > 0 ? v.first.size : 1, false}, v.stride,
                 v.count};
}
}  // namespace detail

// B = A + alpha*x*y^T (blast::ger, dense/Ger.hpp:40-135); B may be A.
inline void ger(double alpha, VectorBatch const& x, VectorBatch const& y, Batch const& A, Batch const& B,
                blastgpu_stream_t stream = nullptr) {
    int const M = x.first.size, N = y.first.size;
    if (A.first.rows != M || A.first.cols != N || B.first.rows != M || B.first.cols != N)
        throw std::invalid_argument("Matrix sizes do not match");
    if (A.first.row_major || B.first.row_major) throw std::logic_error("ger needs column-major storage");
    std::int64_t const n = detail::max_count({x.count, y.count, A.count, B.count});
    if (B.count != n) throw std::invalid_argument("B must hold the whole batch");
    detail::check(blastgpu_dger_strided(M, N, alpha, x.first.data, x.first.inc, detail::vstride_for(x, n),
                                        y.first.data, y.first.inc, detail::vstride_for(y, n), A.first.data,
                                        A.first.ld, detail::stride_for(A, n), B.first.data, B.first.ld, B.stride,
                                        n, stream),
                  "ger");
}

// result[b] = first index of the largest |x_i| (blast::iamax, dense/Iamax.hpp:66-96); device int32.
inline void iamax(VectorBatch const& x, std::int32_t* result, blastgpu_stream_t stream = nullptr) {
    if (x.first.size <= 0) throw std::invalid_argument("Vector must be non-empty");
    detail::check(blastgpu_idamax_strided(x.first.size, x.first.data, x.first.inc, x.stride, result, x.count,
                                          stream),
                  "iamax");
}

// Rows k and ipiv[k] of A exchanged for k = k0..k1-1 (blast::laswp, dense/Laswp.hpp:37-43).
inline void laswp(Batch const& A, int k0, int k1, std::int32_t const* ipiv, std::int64_t ipiv_stride,
                  blastgpu_stream_t stream = nullptr) {
    if (A.first.row_major) throw std::logic_error("laswp needs column-major storage");
    detail::check(blastgpu_dlaswp_strided(A.first.cols, A.first.data, A.first.ld, A.stride, k0, k1, ipiv,
                                          ipiv_stride, A.count, stream),
                  "laswp");
}

// Exchanges x and y (blast::swap, dense/Swap.hpp:35-44).
inline void swap(VectorBatch const& x, VectorBatch const& y, blastgpu_stream_t stream = nullptr) {
    if (x.first.size != y.first.size || x.count != y.count) throw std::invalid_argument("Vector sizes must be equal");
    detail::check(blastgpu_dswap_strided(x.first.size, x.first.data, x.first.inc, x.stride, y.first.data,
                                         y.first.inc, y.stride, x.count, stream),
                  "swap");
}

// Solve A*x = b, A lower / upper triangular (blast::trsvLeftLower / trsvLeftUpper,
// dense/Trsv.hpp:15-68): trsm with one right-hand side, the same operation order.
inline void trsvLeftLower(Batch const& A, VectorBatch const& b, VectorBatch const& x,
                          blastgpu_stream_t stream = nullptr) {
    trsm<UpLo::Lower, false>(A, detail::as_column(b), detail::as_column(x), stream);
}
inline void trsvLeftUpper(Batch const& A, VectorBatch const& b, VectorBatch const& x,
                          blastgpu_stream_t stream = nullptr) {
    trsm<UpLo::Upper, false>(A, detail::as_column(b), detail::as_column(x), stream);
}

// Throws what BLAST's getf2 throws for a singular pivot (dense/Getf2.hpp:68-69), given the
// per-instance info copied to the host.
inline void check_singular(std::int32_t const* info_host, std::int64_t count) {
    for (std::int64_t i = 0; i < count; ++i)
        if (info_host[i] != 0) throw std::invalid_argument("Matrix is singular");
}

}  // namespace blastgpu

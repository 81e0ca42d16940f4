// blastgpu/blast.hpp - BLAST's function names and error behaviour over the blastgpu C ABI.
//
// A BLAST call site such as
//     blast::potrf(A, L);                      // dense/Potrf.hpp:66-106
//     blast::gemm(alpha, A, trans(B), beta, C, D);  // algorithm/Gemm.hpp:80-97
// becomes, with the matrices resident on the GPU,
//     blastgpu::potrf(A, L, stream);
//     blastgpu::gemm(alpha, A, trans(B), beta, C, D, stream);
// where A, L, ... are blastgpu::Matrix views of device memory (one instance),
// blastgpu::Batch views (a uniform batch: instance b starts b*stride elements after the first), or
// std::vector<Matrix> (a ragged batch: every instance its own sizes, layouts and addresses, handed to
// the descriptor entry points through a DescriptorArena). BLAST's own matrix types have
// device-resident counterparts that own their storage: StaticMatrix<M, N>, DynamicMatrix,
// StaticPanelMatrix<M, N, PS>, DynamicPanelMatrix; each converts to a Matrix view.
// Sizes are checked as BLAST checks them and reported with the same exception types:
// std::invalid_argument for mismatched sizes or a singular LU pivot, std::logic_error for the
// variants BLAST does not implement. Every call is asynchronous on `stream`; getrf's singular
// pivots are reported per instance in a device array, which check_singular() turns into BLAST's
// exception once the caller has copied it to the host.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../blastgpu.h"

namespace blastgpu {

enum class UpLo { Lower = BLASTGPU_LOWER, Upper = BLASTGPU_UPPER };

// Non-owning view of one device matrix: column-major, row-major (BLAST's trans() views), or
// BLAST's panel storage (panel > 0: element (i, j) at (i/panel)*ld + i%panel + j*panel, ld being the
// panel spacing, panel/StaticPanelMatrix.hpp:165-184).
struct Matrix {
    double* data = nullptr;
    int rows = 0, cols = 0, ld = 0;
    bool row_major = false;
    int panel = 0;
};

inline Matrix matrix(double* data, int rows, int cols, int ld = -1) {
    return Matrix{data, rows, cols, ld < 0 ? rows : ld, false, 0};
}

// A panel-storage view: panel height ps (BLAST's SIMD width: 4 on AVX2, 2 on NEON), spacing ld.
inline Matrix panel_matrix(double* data, int rows, int cols, int ps, int spacing = -1) {
    return Matrix{data, rows, cols, spacing < 0 ? ps * cols : spacing, false, ps};
}

// BLAST's trans(): the same storage seen transposed (expressions/MatTransExpr.hpp:139-160).
inline Matrix trans(Matrix m) {
    if (m.panel) throw std::logic_error("trans() of panel storage is not a view");
    return Matrix{m.data, m.cols, m.rows, m.ld, !m.row_major, 0};
}

// Offset of element (i, j) in the view's storage.
inline std::int64_t element_offset(Matrix const& m, int i, int j) {
    if (m.panel) return (std::int64_t)(i / m.panel) * m.ld + i % m.panel + (std::int64_t)j * m.panel;
    return m.row_major ? (std::int64_t)i * m.ld + j : i + (std::int64_t)j * m.ld;
}

// BLAST's submatrix() view (views/Submatrix.hpp:234-282); on panel storage the first row must
// start a panel.
inline Matrix submatrix(Matrix m, int i, int j, int rows, int cols) {
    if (i < 0 || j < 0 || rows < 0 || cols < 0 || i + rows > m.rows || j + cols > m.cols)
        throw std::invalid_argument("Invalid submatrix specification");
    if (m.panel && i % m.panel != 0) throw std::invalid_argument("Invalid submatrix specification");
    return Matrix{m.data + element_offset(m, i, j), rows, cols, m.ld, m.row_major, m.panel};
}

// The C ABI's description of a view.
inline blastgpu_mat to_mat(Matrix const& m) {
    blastgpu_mat r;
    r.data = m.data;
    r.rows = m.rows;
    r.cols = m.cols;
    r.ld = m.ld > 0 ? m.ld : 1;
    r.layout = m.panel ? BLASTGPU_PANEL : (m.row_major ? BLASTGPU_ROW_MAJOR : BLASTGPU_COL_MAJOR);
    r.ps = m.panel;
    r.reserved = 0;
    return r;
}

// ---- BLAST's matrix types, device-resident ---------------------------------------------------
// They own their device memory (allocated at construction, zero-filled, freed at destruction) and
// convert to Matrix views. Like BLAST's DynamicMatrix (dense/DynamicMatrix.hpp:44-83, whose copy
// throws "Not implemented"), they are not copyable; they move.
namespace detail {
inline double* device_zeros(std::size_t count) {
    double* p = nullptr;
    if (count == 0) count = 1;
    if (cudaMalloc(&p, count * sizeof(double)) != cudaSuccess) throw std::bad_alloc();
    if (cudaMemset(p, 0, count * sizeof(double)) != cudaSuccess) {
        cudaFree(p);
        throw std::runtime_error("cudaMemset failed");
    }
    return p;
}

class DeviceStorage {
public:
    explicit DeviceStorage(std::size_t count) : p_(device_zeros(count)) {}
    DeviceStorage(DeviceStorage const&) = delete;
    DeviceStorage& operator=(DeviceStorage const&) = delete;
    DeviceStorage(DeviceStorage&& o) noexcept : p_(o.p_) { o.p_ = nullptr; }
    DeviceStorage& operator=(DeviceStorage&& o) noexcept {
        std::swap(p_, o.p_);
        return *this;
    }
    ~DeviceStorage() {
        if (p_) cudaFree(p_);
    }
    double* get() const { return p_; }

private:
    double* p_;
};
}  // namespace detail

// dense/StaticMatrix.hpp:27-166: M x N known at compile time, column-major, spacing M.
template <int M, int N>
class StaticMatrix {
public:
    StaticMatrix() : s_((std::size_t)M * N) {}
    static constexpr int rows() { return M; }
    static constexpr int columns() { return N; }
    static constexpr int spacing() { return M; }
    double* data() const { return s_.get(); }
    operator Matrix() const { return Matrix{s_.get(), M, N, M, false, 0}; }

private:
    detail::DeviceStorage s_;
};

// dense/DynamicMatrix.hpp:26-151: sizes known at run time, column-major, spacing m.
class DynamicMatrix {
public:
    DynamicMatrix(int m, int n) : m_(m), n_(n), s_((std::size_t)(m > 0 ? m : 0) * (n > 0 ? n : 0)) {
        if (m < 0 || n < 0) throw std::invalid_argument("Invalid matrix size");
    }
    int rows() const { return m_; }
    int columns() const { return n_; }
    int spacing() const { return m_; }
    double* data() const { return s_.get(); }
    operator Matrix() const { return Matrix{s_.get(), m_, n_, m_ > 0 ? m_ : 1, false, 0}; }

private:
    int m_, n_;
    detail::DeviceStorage s_;
};

// panel/StaticPanelMatrix.hpp:36-184: panels of PS rows, spacing PS*N, ceil(M/PS) panels.
template <int M, int N, int PS = 4>
class StaticPanelMatrix {
public:
    StaticPanelMatrix() : s_((std::size_t)((M + PS - 1) / PS) * PS * N) {}
    static constexpr int rows() { return M; }
    static constexpr int columns() { return N; }
    static constexpr int spacing() { return PS * N; }
    double* data() const { return s_.get(); }
    operator Matrix() const { return Matrix{s_.get(), M, N, PS * N, false, PS}; }

private:
    detail::DeviceStorage s_;
};

// panel/DynamicPanelMatrix.hpp:35-188: as StaticPanelMatrix with run-time sizes.
class DynamicPanelMatrix {
public:
    DynamicPanelMatrix(int m, int n, int ps = 4)
        : m_(m), n_(n), ps_(ps), s_(ps > 0 && m > 0 && n > 0 ? (std::size_t)((m + ps - 1) / ps) * ps * n : 1) {
        if (m < 0 || n < 0 || ps <= 0) throw std::invalid_argument("Invalid matrix size");
    }
    int rows() const { return m_; }
    int columns() const { return n_; }
    int spacing() const { return ps_ * n_; }
    double* data() const { return s_.get(); }
    operator Matrix() const { return Matrix{s_.get(), m_, n_, ps_ * n_ > 0 ? ps_ * n_ : 1, false, ps_}; }

private:
    int m_, n_, ps_;
    detail::DeviceStorage s_;
};

// Copies a column-major host array (ld = rows) into a view, or a view into one (synchronous).
inline void copy_to_device(Matrix const& m, double const* host) {
    for (int j = 0; j < m.cols; ++j)
        for (int i = 0; i < m.rows; ++i)
            if (cudaMemcpy(m.data + element_offset(m, i, j), host + i + (std::int64_t)j * m.rows, sizeof(double),
                           cudaMemcpyHostToDevice) != cudaSuccess)
                throw std::runtime_error("cudaMemcpy failed");
}
inline void copy_to_host(Matrix const& m, double* host) {
    for (int j = 0; j < m.cols; ++j)
        for (int i = 0; i < m.rows; ++i)
            if (cudaMemcpy(host + i + (std::int64_t)j * m.rows, m.data + element_offset(m, i, j), sizeof(double),
                           cudaMemcpyDeviceToHost) != cudaSuccess)
                throw std::runtime_error("cudaMemcpy failed");
}

// A uniform batch: `count` matrices shaped like `first`, `stride` elements apart.
struct Batch {
    Matrix first;
    std::int64_t stride = 0;
    std::int64_t count = 1;
};

inline Batch batch(Matrix m) { return Batch{m, 0, 1}; }
inline Batch trans(Batch b) { return Batch{trans(b.first), b.stride, b.count}; }

// ---- Ragged batches ----------------------------------------------------------------------------
// Device memory for the descriptor arrays of ragged calls, owned by the caller and reused: it grows
// and never shrinks. Each call stages its descriptors in pinned host memory and copies them on
// `stream`; before the staging buffer is rewritten, the previous copy is waited for. Calls on one
// stream may share an arena (stream order keeps a kernel's descriptors intact until it has read
// them); calls on different streams need an arena each.
class DescriptorArena {
public:
    DescriptorArena() = default;
    DescriptorArena(DescriptorArena const&) = delete;
    DescriptorArena& operator=(DescriptorArena const&) = delete;
    ~DescriptorArena() {
        if (copied_) cudaEventDestroy(copied_);
        if (dev_) cudaFree(dev_);
        if (host_) cudaFreeHost(host_);
    }
    template <class D>
    D* upload(std::vector<D> const& v, blastgpu_stream_t stream) {
        std::size_t const bytes = v.size() * sizeof(D);
        if (!copied_ && cudaEventCreateWithFlags(&copied_, cudaEventDisableTiming) != cudaSuccess)
            throw std::runtime_error("cudaEventCreate failed");
        if (cudaEventSynchronize(copied_) != cudaSuccess) throw std::runtime_error("cudaEventSynchronize failed");
        if (bytes > cap_) {
            if (dev_) cudaFree(dev_);
            if (host_) cudaFreeHost(host_);
            dev_ = host_ = nullptr;
            cap_ = 0;
            if (cudaMalloc(&dev_, bytes) != cudaSuccess || cudaMallocHost(&host_, bytes) != cudaSuccess)
                throw std::bad_alloc();
            cap_ = bytes;
        }
        if (bytes) {
            std::memcpy(host_, v.data(), bytes);
            cudaStream_t const s = reinterpret_cast<cudaStream_t>(stream);
            if (cudaMemcpyAsync(dev_, host_, bytes, cudaMemcpyHostToDevice, s) != cudaSuccess ||
                cudaEventRecord(copied_, s) != cudaSuccess)
                throw std::runtime_error("descriptor upload failed");
        }
        return static_cast<D*>(dev_);
    }

private:
    void* dev_ = nullptr;
    void* host_ = nullptr;
    std::size_t cap_ = 0;
    cudaEvent_t copied_ = nullptr;
};

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
inline void dense_only(std::initializer_list<Batch const*> bs, const char* what) {
    for (auto* b : bs)
        if (b->first.panel)
            throw std::logic_error(std::string(what) + ": panel storage takes the overload with a DescriptorArena");
}
template <class T>
inline void same_count(std::vector<T> const& a, std::size_t n) {
    if (a.size() != n) throw std::invalid_argument("Batch sizes do not match");
}
}  // namespace detail

// D = alpha*A*B + beta*C  (blast::gemm, algorithm/Gemm.hpp:80-97)
inline void gemm(double alpha, Batch const& A, Batch const& B, double beta, Batch const& C, Batch const& D,
                 blastgpu_stream_t stream = nullptr) {
    int const M = A.first.rows, N = B.first.cols, K = A.first.cols;
    if (B.first.rows != K) throw std::invalid_argument("Matrix sizes do not match");
    if (C.first.rows != M || C.first.cols != N) throw std::invalid_argument("Matrix sizes do not match");
    if (D.first.rows != M || D.first.cols != N) throw std::invalid_argument("Matrix sizes do not match");
    if (C.first.row_major || D.first.row_major) throw std::logic_error("C and D must be column-major");
    detail::dense_only({&A, &B, &C, &D}, "gemm");
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
    if (A.first.row_major || L.first.row_major) throw std::logic_error("potrf needs column-major storage");
    detail::dense_only({&A, &L}, "potrf");
    std::int64_t const n = detail::common_count({&A, &L});
    // M x N with M > N: BLAST's trapezoid (dense/Potrf.hpp:78-105)
    detail::check(blastgpu_dpotrf_mn_strided(A.first.rows, A.first.cols, A.first.data, A.first.ld,
                                             detail::stride_for(A, n), L.first.data, L.first.ld,
                                             detail::stride_for(L, n), info, n, stream),
                  "potrf");
}

// Solve A*X = B with A triangular (blast::trsm<UPLO, UNIT>, dense/Trsm.hpp:17-66).
template <UpLo UPLO, bool UNIT>
inline void trsm(Batch const& A, Batch const& B, Batch const& X, blastgpu_stream_t stream = nullptr) {
    int const M = B.first.rows, N = B.first.cols;
    if (A.first.rows != M || A.first.cols != M) throw std::invalid_argument("Invalid argument size");
    if (X.first.rows != M || X.first.cols != N) throw std::invalid_argument("Invalid argument size");
    detail::dense_only({&A, &B, &X}, "trsm");
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
    detail::dense_only({&A, &C, &D}, "syrkLower");
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

// ---- Row and column views (RowColumnVectorPointer.hpp:179-231) ---------------------------------
// BLAST's column(p) / row(p) turn a matrix pointer into a vector pointer; here column(m, j) and
// row(m, i) are a column and a row of a view (combine with submatrix() for any segment). The result
// is a one-column / one-row Matrix, which the ragged BLAS-2 calls take as a vector.
inline Matrix column(Matrix const& m, int j = 0) { return submatrix(m, 0, j, m.rows, 1); }
inline Matrix row(Matrix const& m, int i = 0) {
    if (i < 0 || i >= m.rows) throw std::invalid_argument("Invalid row index");
    if (m.panel) return Matrix{m.data + element_offset(m, i, 0), 1, m.cols, m.ld, false, m.panel};
    return submatrix(m, i, 0, 1, m.cols);
}
// A strided Vector (for the uniform BLAS-2 calls) of a row or column view; a column of panel
// storage has no constant increment.
inline Vector as_vector(Matrix const& v) {
    if (v.panel && v.rows != 1) throw std::logic_error("a panel column has no constant increment");
    if (v.cols == 1) return Vector{v.data, v.rows, v.row_major ? v.ld : 1};
    if (v.rows == 1) return Vector{v.data, v.cols, v.panel ? v.panel : (v.row_major ? 1 : v.ld)};
    throw std::invalid_argument("not a vector view");
}

// ---- Ragged batches and panel storage, through the descriptor entry points -------------------
// Every instance of a std::vector<Matrix> batch keeps its own sizes, layout and address. Size
// checks are BLAST's and are made on the host before anything is launched.

// D[i] = alpha*A[i]*B[i] + beta*C[i] (blast::gemm, algorithm/Gemm.hpp:80-97), any layouts.
inline void gemm(double alpha, std::vector<Matrix> const& A, std::vector<Matrix> const& B, double beta,
                 std::vector<Matrix> const& C, std::vector<Matrix> const& D, DescriptorArena& arena,
                 blastgpu_stream_t stream = nullptr) {
    std::size_t const n = A.size();
    detail::same_count(B, n);
    detail::same_count(C, n);
    detail::same_count(D, n);
    std::vector<blastgpu_gemm_desc> d(n);
    int mm = 0, mn = 0, mk = 0;
    for (std::size_t i = 0; i < n; ++i) {
        if (B[i].rows != A[i].cols || C[i].rows != A[i].rows || C[i].cols != B[i].cols || D[i].rows != A[i].rows ||
            D[i].cols != B[i].cols)
            throw std::invalid_argument("Matrix sizes do not match");
        d[i] = blastgpu_gemm_desc{to_mat(A[i]), to_mat(B[i]), to_mat(C[i]), to_mat(D[i]), alpha, beta};
        mm = std::max(mm, A[i].rows);
        mn = std::max(mn, B[i].cols);
        mk = std::max(mk, A[i].cols);
    }
    if (n == 0) return;
    detail::check(blastgpu_dgemm_batched(arena.upload(d, stream), (std::int64_t)n, mm, mn, mk, stream), "gemm");
}

// One instance of any layout, panel storage included (BLAST's panel gemm).
inline void gemm(double alpha, Matrix const& A, Matrix const& B, double beta, Matrix const& C, Matrix const& D,
                 DescriptorArena& arena, blastgpu_stream_t stream = nullptr) {
    gemm(alpha, std::vector<Matrix>{A}, std::vector<Matrix>{B}, beta, std::vector<Matrix>{C}, std::vector<Matrix>{D},
         arena, stream);
}

// L[i] := chol(A[i]) (blast::potrf, dense/Potrf.hpp:66-106 and panel/Potrf.hpp:59-106), M >= N
// trapezoids allowed. All instances column-major, or all panel storage of one panel height
// (4: AVX2 panels, 2: NEON panels). info: optional device array of the batch's length.
inline void potrf(std::vector<Matrix> const& A, std::vector<Matrix> const& L, std::int32_t* info,
                  DescriptorArena& arena, blastgpu_stream_t stream = nullptr) {
    std::size_t const n = A.size();
    detail::same_count(L, n);
    if (n == 0) return;
    int const ps = A[0].panel;
    std::vector<blastgpu_potrf_desc> d(n);
    for (std::size_t i = 0; i < n; ++i) {
        if (A[i].cols > A[i].rows || L[i].rows != A[i].rows || L[i].cols != A[i].cols)
            throw std::invalid_argument("Invalid matrix size");
        if (A[i].panel != ps || L[i].panel != ps || A[i].row_major || L[i].row_major)
            throw std::logic_error("potrf: every instance needs the same storage (column-major or one panel height)");
        d[i] = blastgpu_potrf_desc{to_mat(A[i]), to_mat(L[i])};
    }
    detail::check(blastgpu_dpotrf_batched(arena.upload(d, stream), (std::int64_t)n,
                                          ps ? BLASTGPU_PANEL : BLASTGPU_COL_MAJOR, ps, info, stream),
                  "potrf");
}

inline void potrf(Matrix const& A, Matrix const& L, std::int32_t* info, DescriptorArena& arena,
                  blastgpu_stream_t stream = nullptr) {
    potrf(std::vector<Matrix>{A}, std::vector<Matrix>{L}, info, arena, stream);
}

// A[i]*X[i] = B[i], A[i] triangular as viewed (blast::trsm<UPLO, UNIT>, dense/Trsm.hpp:17-66).
template <UpLo UPLO, bool UNIT>
inline void trsm(std::vector<Matrix> const& A, std::vector<Matrix> const& B, std::vector<Matrix> const& X,
                 DescriptorArena& arena, blastgpu_stream_t stream = nullptr) {
    std::size_t const n = A.size();
    detail::same_count(B, n);
    detail::same_count(X, n);
    std::vector<blastgpu_trsm_desc> d(n);
    for (std::size_t i = 0; i < n; ++i) {
        if (A[i].rows != B[i].rows || A[i].cols != B[i].rows || X[i].rows != B[i].rows || X[i].cols != B[i].cols)
            throw std::invalid_argument("Invalid argument size");
        d[i] = blastgpu_trsm_desc{to_mat(A[i]), to_mat(B[i]), to_mat(X[i])};
    }
    if (n == 0) return;
    detail::check(blastgpu_dtrsm_batched(BLASTGPU_LEFT, static_cast<int>(UPLO), UNIT, arena.upload(d, stream),
                                         (std::int64_t)n, nullptr, stream),
                  "trsm");
}

// D[i]_lower = alpha*A[i]*A[i]^T + beta*C[i]_lower (blast::syrkLower, dense/Syrk.hpp:15-145).
inline void syrkLower(double alpha, std::vector<Matrix> const& A, double beta, std::vector<Matrix> const& C,
                      std::vector<Matrix> const& D, DescriptorArena& arena, blastgpu_stream_t stream = nullptr) {
    std::size_t const n = A.size();
    detail::same_count(C, n);
    detail::same_count(D, n);
    std::vector<blastgpu_syrk_desc> d(n);
    for (std::size_t i = 0; i < n; ++i) {
        int const M = A[i].rows;
        if (C[i].rows != M || C[i].cols != M || D[i].rows != M || D[i].cols != M)
            throw std::invalid_argument("Matrix sizes do not match");
        d[i] = blastgpu_syrk_desc{to_mat(A[i]), to_mat(C[i]), to_mat(D[i]), alpha, beta};
    }
    if (n == 0) return;
    detail::check(blastgpu_dsyrk_lower_batched(arena.upload(d, stream), (std::int64_t)n, nullptr, stream),
                  "syrkLower");
}

// C[i] = alpha*A[i]*B[i], A[i] upper triangular (algorithm/Trmm.hpp:260-283), BLAST's exceptions kept.
inline void trmm(double alpha, std::vector<Matrix> const& A, UpLo uplo, bool diag, std::vector<Matrix> const& B,
                 std::vector<Matrix> const& C, DescriptorArena& arena, blastgpu_stream_t stream = nullptr) {
    if (diag) throw std::logic_error("Unit-triangular matrices support not implemented in trmm()");
    if (uplo != UpLo::Upper)
        throw std::logic_error("Left product with lower-triangular matrices not implemented in trmm()");
    std::size_t const n = A.size();
    detail::same_count(B, n);
    detail::same_count(C, n);
    std::vector<blastgpu_trmm_desc> d(n);
    for (std::size_t i = 0; i < n; ++i) {
        int const M = B[i].rows, N = B[i].cols;
        if (A[i].rows != M || A[i].cols != M || C[i].rows != M || C[i].cols != N)
            throw std::invalid_argument("Matrix sizes do not match");
        d[i] = blastgpu_trmm_desc{to_mat(A[i]), to_mat(B[i]), to_mat(C[i]), alpha};
    }
    if (n == 0) return;
    detail::check(blastgpu_dtrmm_batched(BLASTGPU_LEFT, static_cast<int>(uplo), diag, arena.upload(d, stream),
                                         (std::int64_t)n, nullptr, stream),
                  "trmm");
}

// A[i] = P*L*U in place (blast::getrf, dense/Getrf.hpp:52-119), column-major; ipiv[i]: device
// int32 arrays of min(m, n) entries; info: device array (see check_singular).
inline void getrf(std::vector<Matrix> const& A, std::vector<std::int32_t*> const& ipiv, std::int32_t* info,
                  DescriptorArena& arena, blastgpu_stream_t stream = nullptr) {
    std::size_t const n = A.size();
    detail::same_count(ipiv, n);
    std::vector<blastgpu_getrf_desc> d(n);
    int mx = 0;
    for (std::size_t i = 0; i < n; ++i) {
        if (A[i].row_major || A[i].panel) throw std::logic_error("getrf needs column-major storage");
        blastgpu_mat empty{};
        empty.ld = 1;
        d[i] = blastgpu_getrf_desc{to_mat(A[i]), ipiv[i], empty};
        mx = std::max(mx, std::max(A[i].rows, A[i].cols));
    }
    if (n == 0) return;
    detail::check(blastgpu_dgetrf_batched(arena.upload(d, stream), info, (std::int64_t)n, mx, stream), "getrf");
}

// Throws what BLAST's getf2 throws for a singular pivot (dense/Getf2.hpp:68-69), given the
// per-instance info copied to the host.
inline void check_singular(std::int32_t const* info_host, std::int64_t count) {
    for (std::int64_t i = 0; i < count; ++i)
        if (info_host[i] != 0) throw std::invalid_argument("Matrix is singular");
}

}  // namespace blastgpu

// Shared device/host helpers of the blastgpu library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "../../include/blastgpu.h"

namespace blastgpu {

// Per-thread record of the last CUDA error, and a global launch counter.
void set_cuda_error(cudaError_t e);
void count_launch(int64_t n = 1);

// Checks the launch that was just enqueued; returns a blastgpu status.
inline int check_launch() {
    cudaError_t const e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return BLASTGPU_ERR_CUDA;
    }
    count_launch();
    return BLASTGPU_SUCCESS;
}

inline cudaStream_t as_cuda(blastgpu_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

// Number of SMs of the current device (cached per device).
int sm_count();

// Raises Kernel's dynamic shared-memory limit to at least `bytes` on the current device. The
// attribute belongs to the (kernel, device) pair, so the flag is kept per device: a call on a
// second GPU of the same process sets it there too. Setting it is not a stream operation, so a
// launch captured into a CUDA graph after the first call on that device replays with it set.
constexpr int kMaxDevices = 64;
template <auto Kernel>
cudaError_t ensure_smem(size_t bytes) {
    static std::atomic<size_t> done[kMaxDevices];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices)
        return cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (done[dev].load(std::memory_order_acquire) >= bytes) return cudaSuccess;
    e = cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) done[dev].store(bytes, std::memory_order_release);
    return e;
}

// D_lower = beta*C + alpha*op(A)*op(A)^T on a uniform batch, syrkLower's order (blas3.cu);
// op(A) = A (m x k) or, with trans_a, the transpose of a k x m A.
int launch_syrk_lower(int m, int k, int trans_a, double alpha, const double* A, int lda, int64_t sa,
                      double beta, const double* C, int ldc, int64_t sc, double* D, int ldd, int64_t sd,
                      int64_t batch, cudaStream_t s);

// Uniform batch of Cholesky solves (or factorisations: nrhs = 0; or solves with a given factor:
// A = nullptr) on the CTA-per-matrix kernels of posv_cta.cu, n <= 512. L may equal A, X may equal B.
int launch_posv_cta_strided(int n, int nrhs, const double* A, int lda, int64_t sa, double* L, int ldl,
                            int64_t sl, const double* B, int ldb, int64_t sb, double* X, int ldx, int64_t sx,
                            int32_t* info, int64_t batch, cudaStream_t s);

// Ragged binary64 Cholesky solves with every n <= 128 on the warp-per-matrix kernel of
// posv_warp.cu (descriptors as for blastgpu_dposv_batched).
int launch_posv_warp(const blastgpu_posv_desc* desc, int64_t count, int max_n, int32_t* info, cudaStream_t s);
// Their adjoints (descriptors as for blastgpu_dposv_bwd_batched), one warp per matrix.
int launch_posv_bwd_warp(const blastgpu_posv_bwd_desc* desc, int64_t count, int max_n, int recompute, int32_t* info,
                         cudaStream_t s);

// Kernel-selection parameters set by the autotuner (blastgpu_tune_set); `fallback` if unset.
int tune_get(const char* key, int fallback);

// Size bin of n for per-bin tuning keys: the smallest power of two >= n (at least 8).
inline int size_bin(int n) {
    int b = 8;
    while (b < n && b < (1 << 20)) b <<= 1;
    return b;
}

// tune_get(prefix + ".n" + size_bin(n)), falling back to tune_get(prefix), then to `fallback`.
int tune_get_bin(const char* prefix, int n, int fallback);

// ---------------------------------------------------------------------------------------------
// Matrix views
// ---------------------------------------------------------------------------------------------
struct MatView {
    double* p;
    int32_t ld;
    int32_t layout;
    int32_t ps;

    __device__ __forceinline__ int64_t off(int i, int j) const {
        if (layout == BLASTGPU_COL_MAJOR) return i + (int64_t)j * ld;
        if (layout == BLASTGPU_ROW_MAJOR) return (int64_t)i * ld + j;
        return (int64_t)(i / ps) * ld + i % ps + (int64_t)j * ps;
    }
    __device__ __forceinline__ double& operator()(int i, int j) const { return p[off(i, j)]; }
};

__device__ __forceinline__ MatView view(blastgpu_mat const& m) {
    return MatView{m.data, m.ld, m.layout, m.ps > 0 ? m.ps : 1};
}

// Device-side validation of a view read from a descriptor (the host cannot read device-resident
// descriptors): extents, a data pointer, and a leading dimension that covers the extents.
__device__ __forceinline__ bool view_ok(blastgpu_mat const& m) {
    if (m.rows < 0 || m.cols < 0) return false;
    if (m.rows == 0 || m.cols == 0) return true;
    if (m.data == nullptr) return false;
    switch (m.layout) {
        case BLASTGPU_COL_MAJOR: return m.ld >= m.rows;
        case BLASTGPU_ROW_MAJOR: return m.ld >= m.cols;
        case BLASTGPU_PANEL: return m.ps > 0 && (int64_t)m.ld >= (int64_t)m.ps * m.cols;
        default: return false;
    }
}

// The transpose of a dense view (column-major <-> row-major over the same storage, BLAST's
// trans()); panel storage has no transposed view (returns false).
__device__ __forceinline__ bool transposed(blastgpu_mat const& m, blastgpu_mat& t) {
    if (m.layout == BLASTGPU_PANEL) return false;
    t = m;
    t.rows = m.cols;
    t.cols = m.rows;
    t.layout = m.layout == BLASTGPU_COL_MAJOR ? BLASTGPU_ROW_MAJOR : BLASTGPU_COL_MAJOR;
    return true;
}

// Host-side validation of one descriptor.
inline bool mat_ok(blastgpu_mat const& m) {
    if (m.rows < 0 || m.cols < 0 || m.reserved != 0) return false;
    if (m.rows == 0 || m.cols == 0) return true;
    if (!m.data) return false;
    switch (m.layout) {
        case BLASTGPU_COL_MAJOR: return m.ld >= m.rows;
        case BLASTGPU_ROW_MAJOR: return m.ld >= m.cols;
        case BLASTGPU_PANEL: return m.ps > 0 && m.ld >= (int64_t)m.ps * m.cols;
        default: return false;
    }
}

// ---------------------------------------------------------------------------------------------
// Reciprocal square root in binary64.
// Newton-Raphson iteration for f(y) = 1/y^2 - s, y' = y*(3 - s*y^2)/2, seeded with the binary32
// hardware estimate (about 23 correct bits); two steps give full binary64 accuracy (each step
// roughly doubles the number of correct bits). Outside the binary32 normal range, and for
// non-positive or NaN s, it falls back to the IEEE operations 1/sqrt(s).
// The divisions and square roots this replaces cost about ten FMA issue slots each on GB300,
// where the FP64 pipe is the bottleneck of every plain-FP64 kernel.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ double rsqrt_nr(double s) {
    if (s > 1.0e-36 && s < 1.0e36) {
        double y = (double)rsqrtf((float)s);
        double const h = 0.5 * s;
        y = y * fma(-h * y, y, 1.5);
        y = y * fma(-h * y, y, 1.5);
        return y;
    }
    return 1.0 / sqrt(s);
}

// Reciprocal by Newton-Raphson for f(y) = 1/y - a, y' = y*(2 - a*y), seeded with the binary32
// estimate; same range fallback as rsqrt_nr.
__device__ __forceinline__ double rcp_nr(double a) {
    double const m = fabs(a);
    if (m > 1.0e-36 && m < 1.0e36) {
        double y = (double)__fdividef(1.0f, (float)a);
        y = y * fma(-a, y, 2.0);
        y = y * fma(-a, y, 2.0);
        // One more correction with the residual e = 1 - a*y gives the last bits.
        double const e = fma(-a, y, 1.0);
        return fma(y, e, y);
    }
    return 1.0 / a;
}

}  // namespace blastgpu

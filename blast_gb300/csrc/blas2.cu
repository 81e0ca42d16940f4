// Batched BLAS-2 building blocks of BLAST's LU: ger, iamax, laswp, swap (binary64, sm_103a).
//
// References (each reproduced operation for operation):
//  * blast::ger (dense/Ger.hpp:40-135): B = A + alpha*x*y^T, per element b_ij = fma(alpha*x_i, y_j,
//    a_ij) (RegisterMatrix::load(1, A) then ger(alpha, x, y): ax = alpha*x rounded, fused update).
//  * blast::iamax (dense/Iamax.hpp:82-95): first index of the largest |x_i| (strict '>' scan; a NaN
//    never replaces the running maximum, a leading NaN is never replaced).
//  * blast::laswp (dense/Laswp.hpp:37-43): for k = k0..k1-1, swap rows k and ipiv[k].
//  * blast::swap (dense/Swap.hpp:35-44): exchange two vectors.
// trsvLeftLower / trsvLeftUpper (dense/Trsv.hpp:15-68) are blastgpu_dtrsm_strided with n = 1.
//
// GPU mapping: ger, laswp and swap are elementwise (one warp per instance, lanes over elements or
// columns); iamax is one warp per vector with the shuffle reduction used by getrf.
#include "common.cuh"

namespace blastgpu {
namespace {

__global__ void __launch_bounds__(128) ger_kernel(int m, int n, double alpha, const double* x, int incx,
                                                  int64_t sx, const double* y, int incy, int64_t sy,
                                                  const double* A, int lda, int64_t sa, double* B, int ldb,
                                                  int64_t sb, int64_t batch) {
    int64_t const b = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= batch) return;
    const double* xb = x + b * sx;
    const double* yb = y + b * sy;
    const double* Ab = A + b * sa;
    double* Bb = B + b * sb;
    for (int j = 0; j < n; ++j) {
        double const yj = yb[(int64_t)j * incy];
        for (int i = lane; i < m; i += 32) {
            double const ax = alpha * xb[(int64_t)i * incx];
            Bb[i + (int64_t)j * ldb] = fma(ax, yj, Ab[i + (int64_t)j * lda]);
        }
    }
}

__global__ void __launch_bounds__(128) iamax_kernel(int n, const double* x, int incx, int64_t sx,
                                                    int32_t* result, int64_t batch) {
    int64_t const b = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= batch) return;
    const double* xb = x + b * sx;
    double best = -1.0;
    int idx = 0x7fffffff;
    for (int i = lane; i < n; i += 32) {
        double const v = fabs(xb[(int64_t)i * incx]);
        if (v > best) { best = v; idx = i; }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        double const ob = __shfl_xor_sync(0xffffffffu, best, off);
        int const oi = __shfl_xor_sync(0xffffffffu, idx, off);
        if (ob > best || (ob == best && oi < idx)) { best = ob; idx = oi; }
    }
    if (lane == 0) {
        double const first = xb[0];
        result[b] = (first != first || idx == 0x7fffffff) ? 0 : idx;
    }
}

__global__ void __launch_bounds__(128) laswp_kernel(int ncols, double* A, int lda, int64_t sa, int k0, int k1,
                                                    const int32_t* ipiv, int64_t sp, int64_t batch) {
    int64_t const b = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= batch) return;
    double* Ab = A + b * sa;
    const int32_t* pb = ipiv + b * sp;
    for (int j = lane; j < ncols; j += 32) {
        double* col = Ab + (int64_t)j * lda;
        for (int k = k0; k < k1; ++k) {
            int const q = pb[k];
            if (q != k) {
                double const t = col[k];
                col[k] = col[q];
                col[q] = t;
            }
        }
    }
}

__global__ void __launch_bounds__(128) swap_kernel(int n, double* x, int incx, int64_t sx, double* y, int incy,
                                                   int64_t sy, int64_t batch) {
    int64_t const b = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= batch) return;
    double* xb = x + b * sx;
    double* yb = y + b * sy;
    for (int i = lane; i < n; i += 32) {
        double const t = xb[(int64_t)i * incx];
        xb[(int64_t)i * incx] = yb[(int64_t)i * incy];
        yb[(int64_t)i * incy] = t;
    }
}

inline bool grid_ok(int64_t batch, unsigned& blocks) {
    int64_t const b = (batch + 3) / 4;
    if (b > 0x7fffffff) return false;
    blocks = (unsigned)b;
    return true;
}

}  // namespace
}  // namespace blastgpu

using namespace blastgpu;

extern "C" {

int blastgpu_dger_strided(int m, int n, double alpha, const double* x, int incx, int64_t stride_x,
                          const double* y, int incy, int64_t stride_y, const double* A, int lda,
                          int64_t stride_a, double* B, int ldb, int64_t stride_b, int64_t batch,
                          blastgpu_stream_t stream) {
    if (m < 0) return -1;
    if (n < 0) return -2;
    if (m > 0 && n > 0 && !x) return -4;
    if (incx == 0) return -5;
    if (m > 0 && n > 0 && !y) return -7;
    if (incy == 0) return -8;
    if (m > 0 && n > 0 && !A) return -10;
    if (lda < (m > 0 ? m : 1)) return -11;
    if (m > 0 && n > 0 && !B) return -13;
    if (ldb < (m > 0 ? m : 1)) return -14;
    if (batch < 0) return -16;
    if (batch == 0 || m == 0 || n == 0) return BLASTGPU_SUCCESS;
    unsigned blocks;
    if (!grid_ok(batch, blocks)) return BLASTGPU_ERR_TOO_LARGE;
    ger_kernel<<<blocks, 128, 0, as_cuda(stream)>>>(m, n, alpha, x, incx, stride_x, y, incy, stride_y, A, lda,
                                                    stride_a, B, ldb, stride_b, batch);
    return check_launch();
}

int blastgpu_idamax_strided(int n, const double* x, int incx, int64_t stride_x, int32_t* result,
                            int64_t batch, blastgpu_stream_t stream) {
    if (n <= 0) return -1;  // BLAST asserts a non-empty vector (dense/Iamax.hpp:69)
    if (!x) return -2;
    if (incx == 0) return -3;
    if (!result) return -5;
    if (batch < 0) return -6;
    if (batch == 0) return BLASTGPU_SUCCESS;
    unsigned blocks;
    if (!grid_ok(batch, blocks)) return BLASTGPU_ERR_TOO_LARGE;
    iamax_kernel<<<blocks, 128, 0, as_cuda(stream)>>>(n, x, incx, stride_x, result, batch);
    return check_launch();
}

int blastgpu_dlaswp_strided(int ncols, double* A, int lda, int64_t stride_a, int k0, int k1,
                            const int32_t* ipiv, int64_t stride_ipiv, int64_t batch,
                            blastgpu_stream_t stream) {
    if (ncols < 0) return -1;
    if (ncols > 0 && !A) return -2;
    if (lda < 1) return -3;
    if (k0 < 0) return -5;
    if (k1 < k0) return -6;
    if (k1 > k0 && !ipiv) return -7;
    if (batch < 0) return -9;
    if (batch == 0 || ncols == 0 || k1 == k0) return BLASTGPU_SUCCESS;
    unsigned blocks;
    if (!grid_ok(batch, blocks)) return BLASTGPU_ERR_TOO_LARGE;
    laswp_kernel<<<blocks, 128, 0, as_cuda(stream)>>>(ncols, A, lda, stride_a, k0, k1, ipiv, stride_ipiv, batch);
    return check_launch();
}

int blastgpu_dswap_strided(int n, double* x, int incx, int64_t stride_x, double* y, int incy,
                           int64_t stride_y, int64_t batch, blastgpu_stream_t stream) {
    if (n < 0) return -1;
    if (n > 0 && !x) return -2;
    if (incx == 0) return -3;
    if (n > 0 && !y) return -5;
    if (incy == 0) return -6;
    if (batch < 0) return -8;
    if (batch == 0 || n == 0) return BLASTGPU_SUCCESS;
    unsigned blocks;
    if (!grid_ok(batch, blocks)) return BLASTGPU_ERR_TOO_LARGE;
    swap_kernel<<<blocks, 128, 0, as_cuda(stream)>>>(n, x, incx, stride_x, y, incy, stride_y, batch);
    return check_launch();
}

}  // extern "C"

// Ragged (descriptor) forms of syrkLower, trsm (both sides), trmm, the BLAS-2 operations and the
// trsm / potrf adjoints, binary64, sm_103a.
//
// Every instance is described by its own blastgpu_mat views, so one launch takes a batch of
// matrices of different sizes and layouts: column-major, row-major (BLAST's trans() view of a
// column-major matrix) or panel storage (panel/StaticPanelMatrix.hpp:165-184). The per-element
// order of rounded operations is the one of the strided kernels (blas2.cu, blas3.cu, adjoint.cu),
// so a descriptor call and a strided call on the same data give the same bits:
//  * syrkLower (dense/Syrk.hpp:15-145): v = beta*c_ij; for k ascending v = fma(alpha*a_ik, a_jk, v).
//  * trsm (dense/Trsm.hpp:17-66): per right-hand-side column, lower: i ascending,
//    acc = b_ij, acc = fma(-a_iq, x_qj, acc) for q < i ascending, x_ij = acc / a_ii (unit: acc);
//    upper: i descending, q > i ascending. uplo names the triangle of A as viewed (a row-major
//    view of a lower column-major factor is upper). Right side X*A = B: per row, column
//    substitution in the same pattern (no BLAST counterpart, register_matrix/RegisterMatrix.hpp:
//    592-597 leaves it unimplemented).
//  * trmm (algorithm/Trmm.hpp:93-242): c_ij = sum over the triangle of fma(alpha*a_iq, b_qj, .)
//    (left) or fma(alpha*b_iq, a_qj, .) (right), q ascending from a zero accumulator.
//  * ger (dense/Ger.hpp:40-135): b_ij = fma(alpha*x_i, y_j, a_ij); iamax (dense/Iamax.hpp:82-95):
//    first index of the largest |x_i|; laswp (dense/Laswp.hpp:37-43); swap (dense/Swap.hpp:35-44).
//  * adjoints of trsm and potrf as in adjoint.cu.
//
// A vector operand is a blastgpu_mat with one column (element i at (i, 0)) or one row (element i
// at (0, i)), so a column or a row of a matrix (RowColumnVectorPointer.hpp:179-231) is a view too.
//
// GPU mapping: one warp per instance (128-thread blocks), lanes over output elements (syrk,
// trmm, ger, swap), right-hand-side columns or rows (trsm), or columns (laswp). A descriptor whose
// shapes do not fit together gets status -1 and nothing is written for it.
#include "common.cuh"

namespace blastgpu {
namespace {

constexpr int kWarpsPerBlock = 4;

struct Vec {
    MatView v;
    bool row;
    __device__ __forceinline__ double& operator[](int i) const { return row ? v(0, i) : v(i, 0); }
};

__device__ __forceinline__ int vlen(blastgpu_mat const& m) { return m.cols == 1 ? m.rows : (m.rows == 1 ? m.cols : -1); }
__device__ __forceinline__ Vec vec(blastgpu_mat const& m) { return Vec{view(m), m.rows == 1 && m.cols != 1}; }

__device__ __forceinline__ void put_status(int32_t* status, int64_t b, int lane, int v) {
    if (status && lane == 0) status[b] = v;
}

// ---------------------------------------------------------------------------------------------
// syrkLower
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) syrk_lower_desc_kernel(const blastgpu_syrk_desc* desc, int64_t count,
                                                              int32_t* status) {
    int64_t const b = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= count) return;
    blastgpu_syrk_desc const d = desc[b];
    int const m = d.A.rows, k = d.A.cols;
    bool const ok = view_ok(d.A) && view_ok(d.C) && view_ok(d.D) && d.C.rows == m && d.C.cols == m &&
                    d.D.rows == m && d.D.cols == m;
    put_status(status, b, lane, ok ? 0 : -1);
    if (!ok) return;
    MatView const A = view(d.A), C = view(d.C), D = view(d.D);
    bool const alpha1 = d.alpha == 1.0;
    int const total = m * (m + 1) / 2;
    for (int e = lane; e < total; e += 32) {
        int j = 0, rem = e;
        while (rem >= m - j) { rem -= m - j; ++j; }
        int const i = j + rem;
        double v = d.beta * C(i, j);
        for (int q = 0; q < k; ++q) v = fma(alpha1 ? A(i, q) : d.alpha * A(i, q), A(j, q), v);
        D(i, j) = v;
    }
}

// ---------------------------------------------------------------------------------------------
// trsm, both sides (X may equal B)
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void trsm_left_col(int uplo, int unit, int m, MatView const& A, MatView const& B,
                                              MatView const& X, int j) {
    if (uplo == BLASTGPU_LOWER) {
        for (int i = 0; i < m; ++i) {
            double acc = B(i, j);
            for (int q = 0; q < i; ++q) acc = fma(-A(i, q), X(q, j), acc);
            X(i, j) = unit ? acc : acc / A(i, i);
        }
    } else {
        for (int i = m; i-- > 0;) {
            double acc = B(i, j);
            for (int q = i + 1; q < m; ++q) acc = fma(-A(i, q), X(q, j), acc);
            X(i, j) = unit ? acc : acc / A(i, i);
        }
    }
}

__device__ __forceinline__ void trsm_right_row(int uplo, int unit, int n, MatView const& A, MatView const& B,
                                               MatView const& X, int i) {
    if (uplo == BLASTGPU_UPPER) {
        for (int j = 0; j < n; ++j) {
            double acc = B(i, j);
            for (int q = 0; q < j; ++q) acc = fma(-X(i, q), A(q, j), acc);
            X(i, j) = unit ? acc : acc / A(j, j);
        }
    } else {
        for (int j = n; j-- > 0;) {
            double acc = B(i, j);
            for (int q = j + 1; q < n; ++q) acc = fma(-X(i, q), A(q, j), acc);
            X(i, j) = unit ? acc : acc / A(j, j);
        }
    }
}

__device__ __forceinline__ bool trsm_shapes_ok(int side, blastgpu_mat const& A, blastgpu_mat const& B,
                                               blastgpu_mat const& X) {
    int const ka = side == BLASTGPU_LEFT ? B.rows : B.cols;
    return view_ok(A) && view_ok(B) && view_ok(X) && A.rows == ka && A.cols == ka && X.rows == B.rows &&
           X.cols == B.cols;
}

__global__ void __launch_bounds__(128) trsm_desc_kernel(int side, int uplo, int unit, const blastgpu_trsm_desc* desc,
                                                        int64_t count, int32_t* status) {
    int64_t const b = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= count) return;
    blastgpu_trsm_desc const d = desc[b];
    bool const ok = trsm_shapes_ok(side, d.A, d.B, d.X);
    put_status(status, b, lane, ok ? 0 : -1);
    if (!ok) return;
    MatView const A = view(d.A), B = view(d.B), X = view(d.X);
    if (side == BLASTGPU_LEFT) {
        for (int j = lane; j < d.B.cols; j += 32) trsm_left_col(uplo, unit, d.B.rows, A, B, X, j);
    } else {
        for (int i = lane; i < d.B.rows; i += 32) trsm_right_row(uplo, unit, d.B.cols, A, B, X, i);
    }
}

// ---------------------------------------------------------------------------------------------
// trmm (C must not overlap A or B)
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) trmm_desc_kernel(int side, int uplo, int unit, const blastgpu_trmm_desc* desc,
                                                        int64_t count, int32_t* status) {
    int64_t const b = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= count) return;
    blastgpu_trmm_desc const d = desc[b];
    int const m = d.B.rows, n = d.B.cols;
    int const ka = side == BLASTGPU_LEFT ? m : n;
    bool const ok = view_ok(d.A) && view_ok(d.B) && view_ok(d.C) && d.A.rows == ka && d.A.cols == ka &&
                    d.C.rows == m && d.C.cols == n;
    put_status(status, b, lane, ok ? 0 : -1);
    if (!ok) return;
    MatView const A = view(d.A), B = view(d.B), C = view(d.C);
    bool const upper = uplo == BLASTGPU_UPPER, alpha1 = d.alpha == 1.0;
    auto a = [&](int i, int q) -> double { return (unit && i == q) ? 1.0 : A(i, q); };
    for (int e = lane; e < m * n; e += 32) {
        int const i = e % m, j = e / m;
        double acc = 0.0;
        if (side == BLASTGPU_LEFT) {
            int const q0 = upper ? i : 0, q1 = upper ? m : i + 1;
            for (int q = q0; q < q1; ++q) acc = fma(alpha1 ? a(i, q) : d.alpha * a(i, q), B(q, j), acc);
        } else {
            int const q0 = upper ? 0 : j, q1 = upper ? j + 1 : n;
            for (int q = q0; q < q1; ++q) acc = fma(alpha1 ? B(i, q) : d.alpha * B(i, q), a(q, j), acc);
        }
        C(i, j) = acc;
    }
}

// ---------------------------------------------------------------------------------------------
// BLAS-2
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) ger_desc_kernel(const blastgpu_ger_desc* desc, int64_t count, int32_t* status) {
    int64_t const b = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= count) return;
    blastgpu_ger_desc const d = desc[b];
    int const m = d.A.rows, n = d.A.cols;
    bool const ok = view_ok(d.x) && view_ok(d.y) && view_ok(d.A) && view_ok(d.B) && vlen(d.x) == m &&
                    vlen(d.y) == n && d.B.rows == m && d.B.cols == n;
    put_status(status, b, lane, ok ? 0 : -1);
    if (!ok) return;
    Vec const x = vec(d.x), y = vec(d.y);
    MatView const A = view(d.A), B = view(d.B);
    for (int j = 0; j < n; ++j) {
        double const yj = y[j];
        for (int i = lane; i < m; i += 32) B(i, j) = fma(d.alpha * x[i], yj, A(i, j));
    }
}

// result[b] = first index of the largest |x_i|; -1 for a descriptor that is not a vector.
__global__ void __launch_bounds__(128) iamax_desc_kernel(const blastgpu_mat* xs, int64_t count, int32_t* result) {
    int64_t const b = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= count) return;
    blastgpu_mat const d = xs[b];
    int const n = vlen(d);
    if (!view_ok(d) || n < 0) {
        if (lane == 0) result[b] = -1;
        return;
    }
    if (n == 0) {
        if (lane == 0) result[b] = 0;
        return;
    }
    Vec const x = vec(d);
    double best = -1.0;
    int idx = 0x7fffffff;
    for (int i = lane; i < n; i += 32) {
        double const v = fabs(x[i]);
        if (v > best) { best = v; idx = i; }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        double const ob = __shfl_xor_sync(0xffffffffu, best, off);
        int const oi = __shfl_xor_sync(0xffffffffu, idx, off);
        if (ob > best || (ob == best && oi < idx)) { best = ob; idx = oi; }
    }
    if (lane == 0) {
        double const first = x[0];
        result[b] = (first != first || idx == 0x7fffffff) ? 0 : idx;
    }
}

__global__ void __launch_bounds__(128) laswp_desc_kernel(const blastgpu_laswp_desc* desc, int64_t count,
                                                         int32_t* status) {
    int64_t const b = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= count) return;
    blastgpu_laswp_desc const d = desc[b];
    bool ok = view_ok(d.A) && d.k0 >= 0 && d.k0 <= d.k1 && d.k1 <= d.A.rows && (d.k1 == d.k0 || d.ipiv != nullptr);
    // every pivot row must lie inside A (BLAST does not check; here nothing is swapped otherwise)
    if (ok) {
        bool bad = false;
        for (int k = d.k0 + lane; k < d.k1; k += 32) bad |= d.ipiv[k] < 0 || d.ipiv[k] >= d.A.rows;
        ok = !__any_sync(0xffffffffu, bad);
    }
    put_status(status, b, lane, ok ? 0 : -1);
    if (!ok) return;
    MatView const A = view(d.A);
    for (int j = lane; j < d.A.cols; j += 32) {
        for (int k = d.k0; k < d.k1; ++k) {
            int const q = d.ipiv[k];
            if (q != k) {
                double const t = A(k, j);
                A(k, j) = A(q, j);
                A(q, j) = t;
            }
        }
    }
}

__global__ void __launch_bounds__(128) swap_desc_kernel(const blastgpu_swap_desc* desc, int64_t count, int32_t* status) {
    int64_t const b = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= count) return;
    blastgpu_swap_desc const d = desc[b];
    int const n = vlen(d.x);
    bool const ok = view_ok(d.x) && view_ok(d.y) && n >= 0 && vlen(d.y) == n;
    put_status(status, b, lane, ok ? 0 : -1);
    if (!ok) return;
    Vec const x = vec(d.x), y = vec(d.y);
    for (int i = lane; i < n; i += 32) {
        double const t = x[i];
        x[i] = y[i];
        y[i] = t;
    }
}

// ---------------------------------------------------------------------------------------------
// Adjoints of trsm and potrf
// ---------------------------------------------------------------------------------------------
// trsm op(A) X = B (A as viewed, uplo of that view): Bbar = A^{-T} Xbar (a left solve with the
// transposed view, whose triangle is the other one), then Abar -= Bbar X^T on A's triangle
// (strictly, for a unit diagonal). Abar is a view in A's own orientation.
__global__ void __launch_bounds__(128) trsm_bwd_desc_kernel(int uplo, int unit, const blastgpu_trsm_bwd_desc* desc,
                                                            int64_t count, int32_t* status) {
    int64_t const b = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= count) return;
    blastgpu_trsm_bwd_desc const d = desc[b];
    int const m = d.Xbar.rows, n = d.Xbar.cols;
    blastgpu_mat At;
    bool ok = transposed(d.A, At) && view_ok(d.A) && view_ok(d.Xbar) && view_ok(d.Bbar) && d.A.rows == m &&
              d.A.cols == m && d.Bbar.rows == m && d.Bbar.cols == n;
    bool const want_a = d.Abar.data != nullptr;
    if (want_a)
        ok = ok && view_ok(d.X) && view_ok(d.Abar) && d.X.rows == m && d.X.cols == n && d.Abar.rows == m &&
             d.Abar.cols == m;
    put_status(status, b, lane, ok ? 0 : -1);
    if (!ok) return;
    MatView const AT = view(At), Xb = view(d.Xbar), Bb = view(d.Bbar);
    int const tuplo = uplo == BLASTGPU_LOWER ? BLASTGPU_UPPER : BLASTGPU_LOWER;
    for (int j = lane; j < n; j += 32) trsm_left_col(tuplo, unit, m, AT, Xb, Bb, j);
    if (!want_a) return;
    __syncwarp();
    MatView const X = view(d.X), Ab = view(d.Abar);
    for (int e = lane; e < m * m; e += 32) {
        int const i = e % m, j = e / m;
        bool const in = uplo == BLASTGPU_LOWER ? (unit ? i > j : i >= j) : (unit ? i < j : i <= j);
        if (!in) continue;
        double v = 0.0;
        for (int r = 0; r < n; ++r) v = fma(Bb(i, r), X(j, r), v);
        Ab(i, j) -= v;
    }
}

// potrf A = L L^T: Abar = (S + S^T)/2, S = L^{-T} Phi(L^T Lbar) L^{-1} (I. Murray, 2016), all in
// Abar: Phi into Abar, the left solve with the transposed view of L, the right solve with L, and
// the symmetrisation, one warp per instance throughout.
__global__ void __launch_bounds__(128) potrf_bwd_desc_kernel(const blastgpu_potrf_bwd_desc* desc, int64_t count,
                                                             int32_t* status) {
    int64_t const b = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= count) return;
    blastgpu_potrf_bwd_desc const d = desc[b];
    int const n = d.L.rows;
    blastgpu_mat Lt;
    bool const ok = transposed(d.L, Lt) && view_ok(d.L) && view_ok(d.Lbar) && view_ok(d.Abar) && d.L.cols == n &&
                    d.Lbar.rows == n && d.Lbar.cols == n && d.Abar.rows == n && d.Abar.cols == n;
    put_status(status, b, lane, ok ? 0 : -1);
    if (!ok) return;
    MatView const L = view(d.L), Lb = view(d.Lbar), W = view(d.Abar), LT = view(Lt);
    for (int e = lane; e < n * n; e += 32) {
        int const i = e % n, j = e / n;
        double s = 0.0;
        if (i >= j) {
            for (int k = i; k < n; ++k) s = fma(L(k, i), Lb(k, j), s);
            if (i == j) s *= 0.5;
        }
        W(i, j) = s;
    }
    __syncwarp();
    for (int j = lane; j < n; j += 32) trsm_left_col(BLASTGPU_UPPER, 0, n, LT, W, W, j);  // W := L^{-T} W
    __syncwarp();
    for (int i = lane; i < n; i += 32) trsm_right_row(BLASTGPU_LOWER, 0, n, L, W, W, i);  // W := W L^{-1}
    __syncwarp();
    for (int e = lane; e < n * n; e += 32) {
        int const i = e % n, j = e / n;
        if (i > j) {
            double const s = 0.5 * (W(i, j) + W(j, i));
            W(i, j) = s;
            W(j, i) = s;
        }
    }
}

inline int warp_blocks(int64_t batch, unsigned& blocks) {
    int64_t const g = (batch + kWarpsPerBlock - 1) / kWarpsPerBlock;
    if (g > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    blocks = (unsigned)g;
    return BLASTGPU_SUCCESS;
}

}  // namespace
}  // namespace blastgpu

using namespace blastgpu;

extern "C" {

#define BLASTGPU_DESC_PROLOGUE                         \
    if (batch < 0) return -2;                          \
    if (batch == 0) return BLASTGPU_SUCCESS;           \
    if (!desc) return -1;                              \
    unsigned blocks = 0;                               \
    if (warp_blocks(batch, blocks) != BLASTGPU_SUCCESS) return BLASTGPU_ERR_TOO_LARGE;

int blastgpu_dsyrk_lower_batched(const blastgpu_syrk_desc* desc, int64_t batch, int32_t* status,
                                 blastgpu_stream_t stream) {
    BLASTGPU_DESC_PROLOGUE
    syrk_lower_desc_kernel<<<blocks, 128, 0, as_cuda(stream)>>>(desc, batch, status);
    return check_launch();
}

int blastgpu_dtrsm_batched(int side, int uplo, int unit, const blastgpu_trsm_desc* desc, int64_t batch,
                           int32_t* status, blastgpu_stream_t stream) {
    if (side != BLASTGPU_LEFT && side != BLASTGPU_RIGHT) return -1;
    if (uplo != BLASTGPU_LOWER && uplo != BLASTGPU_UPPER) return -2;
    if (unit != 0 && unit != 1) return -3;
    if (batch < 0) return -5;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (!desc) return -4;
    unsigned blocks = 0;
    if (warp_blocks(batch, blocks) != BLASTGPU_SUCCESS) return BLASTGPU_ERR_TOO_LARGE;
    trsm_desc_kernel<<<blocks, 128, 0, as_cuda(stream)>>>(side, uplo, unit, desc, batch, status);
    return check_launch();
}

int blastgpu_dtrmm_batched(int side, int uplo, int unit, const blastgpu_trmm_desc* desc, int64_t batch,
                           int32_t* status, blastgpu_stream_t stream) {
    if (side != BLASTGPU_LEFT && side != BLASTGPU_RIGHT) return -1;
    if (uplo != BLASTGPU_LOWER && uplo != BLASTGPU_UPPER) return -2;
    if (unit != 0 && unit != 1) return -3;
    if (batch < 0) return -5;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (!desc) return -4;
    unsigned blocks = 0;
    if (warp_blocks(batch, blocks) != BLASTGPU_SUCCESS) return BLASTGPU_ERR_TOO_LARGE;
    trmm_desc_kernel<<<blocks, 128, 0, as_cuda(stream)>>>(side, uplo, unit, desc, batch, status);
    return check_launch();
}

int blastgpu_dger_batched(const blastgpu_ger_desc* desc, int64_t batch, int32_t* status, blastgpu_stream_t stream) {
    BLASTGPU_DESC_PROLOGUE
    ger_desc_kernel<<<blocks, 128, 0, as_cuda(stream)>>>(desc, batch, status);
    return check_launch();
}

int blastgpu_idamax_batched(const blastgpu_mat* desc, int64_t batch, int32_t* result, blastgpu_stream_t stream) {
    if (batch < 0) return -2;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (!desc) return -1;
    if (!result) return -3;
    unsigned blocks = 0;
    if (warp_blocks(batch, blocks) != BLASTGPU_SUCCESS) return BLASTGPU_ERR_TOO_LARGE;
    iamax_desc_kernel<<<blocks, 128, 0, as_cuda(stream)>>>(desc, batch, result);
    return check_launch();
}

int blastgpu_dlaswp_batched(const blastgpu_laswp_desc* desc, int64_t batch, int32_t* status,
                            blastgpu_stream_t stream) {
    BLASTGPU_DESC_PROLOGUE
    laswp_desc_kernel<<<blocks, 128, 0, as_cuda(stream)>>>(desc, batch, status);
    return check_launch();
}

int blastgpu_dswap_batched(const blastgpu_swap_desc* desc, int64_t batch, int32_t* status, blastgpu_stream_t stream) {
    BLASTGPU_DESC_PROLOGUE
    swap_desc_kernel<<<blocks, 128, 0, as_cuda(stream)>>>(desc, batch, status);
    return check_launch();
}

int blastgpu_dtrsm_bwd_batched(int uplo, int unit, const blastgpu_trsm_bwd_desc* desc, int64_t batch,
                               int32_t* status, blastgpu_stream_t stream) {
    if (uplo != BLASTGPU_LOWER && uplo != BLASTGPU_UPPER) return -1;
    if (unit != 0 && unit != 1) return -2;
    if (batch < 0) return -4;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (!desc) return -3;
    unsigned blocks = 0;
    if (warp_blocks(batch, blocks) != BLASTGPU_SUCCESS) return BLASTGPU_ERR_TOO_LARGE;
    trsm_bwd_desc_kernel<<<blocks, 128, 0, as_cuda(stream)>>>(uplo, unit, desc, batch, status);
    return check_launch();
}

int blastgpu_dpotrf_bwd_batched(const blastgpu_potrf_bwd_desc* desc, int64_t batch, int32_t* status,
                                blastgpu_stream_t stream) {
    BLASTGPU_DESC_PROLOGUE
    potrf_bwd_desc_kernel<<<blocks, 128, 0, as_cuda(stream)>>>(desc, batch, status);
    return check_launch();
}

#undef BLASTGPU_DESC_PROLOGUE

}  // extern "C"

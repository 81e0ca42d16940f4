// Reverse-mode adjoints of gemm, trsm and potrf for uniform batches (binary64, sm_103a).
// BLAST has no derivatives; these follow the standard matrix calculus of the forward operations
// the library implements (gemm: algorithm/Gemm.hpp:80-97; trsm: dense/Trsm.hpp:17-66; potrf:
// dense/Potrf.hpp:66-106), and each entry point composes the library's own batched kernels with
// a few elementwise ones.
//
//  * gemm, D = alpha*op(A)*op(B) + beta*C:  op(A)bar = alpha*Dbar*op(B)^T,
//    op(B)bar = alpha*op(A)^T*Dbar, Cbar = beta*Dbar. Two gemm launches with beta = 1 accumulate
//    into Abar and Bbar in their own storage orientation; one axpy accumulates Cbar.
//  * trsm, op(A)*X = B:  Bbar = op(A)^{-T}*Xbar (a trsm with the transpose flipped, so the
//    triangle flips too), op(A)bar = -Bbar*X^T on op(A)'s triangle (strictly, for a unit
//    diagonal), accumulated into Abar in A's storage orientation.
//  * potrf, A = L*L^T:  Abar = (S + S^T)/2 with S = L^{-T} Phi(L^T*Lbar) L^{-1}, Phi the lower
//    triangle with the diagonal halved (I. Murray, "Differentiation of the Cholesky
//    decomposition", 2016): the gradient of a symmetric A, written in full, the same convention as
//    blastgpu_dposv_bwd_batched. Phi(L^T*Lbar) is formed in Abar, the two triangular solves run in
//    place there (blastgpu_dtrsm_strided, blastgpu_dtrsm_right_strided), then Abar is symmetrised.
//
// The elementwise kernels run one warp per instance (128-thread blocks), lanes over elements.
#include "common.cuh"

namespace blastgpu {
namespace {

struct ColMat {
    double* p;
    int ld;
    int64_t stride;
    __device__ __forceinline__ double& at(int64_t b, int i, int j) const { return p[b * stride + i + (int64_t)j * ld]; }
};

// Y += alpha * X, m x n per instance.
__global__ void __launch_bounds__(128) mat_axpy_kernel(int m, int n, double alpha, ColMat X, ColMat Y, int64_t batch) {
    int64_t const b = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= batch) return;
    for (int e = lane; e < m * n; e += 32) {
        int const i = e % m, j = e / m;
        Y.at(b, i, j) = fma(alpha, X.at(b, i, j), Y.at(b, i, j));
    }
}

// Abar += -P*Q^T on op(A)'s triangle (uplo of op(A); strict when unit), stored transposed when
// trans_a. P and Q are m x n; element (i, j) of op(A) sums over r = 0..n-1 in ascending order.
__global__ void __launch_bounds__(128) tri_outer_acc_kernel(int uplo, int trans_a, int unit, int m, int n, ColMat P,
                                                            ColMat Q, ColMat Abar, int64_t batch) {
    int64_t const b = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= batch) return;
    for (int e = lane; e < m * m; e += 32) {
        int const i = e % m, j = e / m;
        bool const in = uplo == BLASTGPU_LOWER ? (unit ? i > j : i >= j) : (unit ? i < j : i <= j);
        if (!in) continue;
        double v = 0.0;
        for (int r = 0; r < n; ++r) v = fma(P.at(b, i, r), Q.at(b, j, r), v);
        double& dst = trans_a ? Abar.at(b, j, i) : Abar.at(b, i, j);
        dst -= v;
    }
}

// W = Phi(L^T * Lbar): element (i, j), i >= j, is sum_{k = i}^{n-1} l_ki * lbar_kj (both lower
// triangles; k ascending), halved on the diagonal; the strictly upper part of W is zeroed.
__global__ void __launch_bounds__(128) chol_bwd_phi_kernel(int n, ColMat L, ColMat Lbar, ColMat W, int64_t batch) {
    int64_t const b = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= batch) return;
    for (int e = lane; e < n * n; e += 32) {
        int const i = e % n, j = e / n;
        double s = 0.0;
        if (i >= j) {
            for (int k = i; k < n; ++k) s = fma(L.at(b, k, i), Lbar.at(b, k, j), s);
            if (i == j) s *= 0.5;
        }
        W.at(b, i, j) = s;
    }
}

// W = (W + W^T) / 2 in place; each off-diagonal pair is owned by one lane.
__global__ void __launch_bounds__(128) symmetrize_kernel(int n, ColMat W, int64_t batch) {
    int64_t const b = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= batch) return;
    for (int e = lane; e < n * n; e += 32) {
        int const i = e % n, j = e / n;
        if (i > j) {
            double const s = 0.5 * (W.at(b, i, j) + W.at(b, j, i));
            W.at(b, i, j) = s;
            W.at(b, j, i) = s;
        }
    }
}

inline bool warp_grid(int64_t batch, unsigned& blocks) {
    int64_t const g = (batch + 3) / 4;
    if (g > 0x7fffffff) return false;
    blocks = (unsigned)g;
    return true;
}

}  // namespace
}  // namespace blastgpu

using namespace blastgpu;

extern "C" {

int blastgpu_dgemm_bwd_strided(int trans_a, int trans_b, int m, int n, int k, double alpha, const double* A,
                               int lda, int64_t stride_a, const double* B, int ldb, int64_t stride_b, double beta,
                               const double* Dbar, int lddb, int64_t stride_db, double* Abar, int ldab,
                               int64_t stride_ab, double* Bbar, int ldbb, int64_t stride_bb, double* Cbar, int ldcb,
                               int64_t stride_cb, int64_t batch, blastgpu_stream_t stream) {
    if (trans_a != 0 && trans_a != 1) return -1;
    if (trans_b != 0 && trans_b != 1) return -2;
    if (m < 0) return -3;
    if (n < 0) return -4;
    if (k < 0) return -5;
    int const arows = trans_a ? k : m, brows = trans_b ? n : k;
    if (Bbar && m > 0 && k > 0 && !A) return -7;
    if (lda < (arows > 0 ? arows : 1)) return -8;
    if (Abar && k > 0 && n > 0 && !B) return -10;
    if (ldb < (brows > 0 ? brows : 1)) return -11;
    if (m > 0 && n > 0 && !Dbar) return -14;
    if (lddb < (m > 0 ? m : 1)) return -15;
    if (Abar && ldab < (arows > 0 ? arows : 1)) return -18;
    if (Bbar && ldbb < (brows > 0 ? brows : 1)) return -21;
    if (Cbar && ldcb < (m > 0 ? m : 1)) return -24;
    if (batch < 0) return -26;
    // instances accumulate concurrently: a shared (stride 0) output would race
    if (batch > 1 && Abar && stride_ab == 0) return -19;
    if (batch > 1 && Bbar && stride_bb == 0) return -22;
    if (batch > 1 && Cbar && stride_cb == 0) return -25;
    if (batch == 0) return BLASTGPU_SUCCESS;
    int st = BLASTGPU_SUCCESS;
    if (Abar && m > 0 && k > 0) {
        if (!trans_a)  // Abar (m x k) += alpha * Dbar * op(B)^T
            st = blastgpu_dgemm_strided(0, !trans_b, m, k, n, alpha, Dbar, lddb, stride_db, B, ldb, stride_b, 1.0,
                                        Abar, ldab, stride_ab, Abar, ldab, stride_ab, batch, stream);
        else  // A is stored k x m: Abar += alpha * op(B) * Dbar^T
            st = blastgpu_dgemm_strided(trans_b, 1, k, m, n, alpha, B, ldb, stride_b, Dbar, lddb, stride_db, 1.0,
                                        Abar, ldab, stride_ab, Abar, ldab, stride_ab, batch, stream);
        if (st != BLASTGPU_SUCCESS) return st;
    }
    if (Bbar && k > 0 && n > 0) {
        if (!trans_b)  // Bbar (k x n) += alpha * op(A)^T * Dbar
            st = blastgpu_dgemm_strided(!trans_a, 0, k, n, m, alpha, A, lda, stride_a, Dbar, lddb, stride_db, 1.0,
                                        Bbar, ldbb, stride_bb, Bbar, ldbb, stride_bb, batch, stream);
        else  // B is stored n x k: Bbar += alpha * Dbar^T * op(A)
            st = blastgpu_dgemm_strided(1, trans_a, n, k, m, alpha, Dbar, lddb, stride_db, A, lda, stride_a, 1.0,
                                        Bbar, ldbb, stride_bb, Bbar, ldbb, stride_bb, batch, stream);
        if (st != BLASTGPU_SUCCESS) return st;
    }
    if (Cbar && m > 0 && n > 0) {
        unsigned blocks;
        if (!warp_grid(batch, blocks)) return BLASTGPU_ERR_TOO_LARGE;
        mat_axpy_kernel<<<blocks, 128, 0, as_cuda(stream)>>>(m, n, beta, ColMat{const_cast<double*>(Dbar), lddb, stride_db},
                                                            ColMat{Cbar, ldcb, stride_cb}, batch);
        st = check_launch();
    }
    return st;
}

int blastgpu_dtrsm_bwd_strided(int uplo, int trans_a, int unit, int m, int n, const double* A, int lda,
                               int64_t stride_a, const double* X, int ldx, int64_t stride_x, const double* Xbar,
                               int ldxb, int64_t stride_xb, double* Bbar, int ldbb, int64_t stride_bb, double* Abar,
                               int ldab, int64_t stride_ab, int64_t batch, blastgpu_stream_t stream) {
    if (uplo != BLASTGPU_LOWER && uplo != BLASTGPU_UPPER) return -1;
    if (trans_a != 0 && trans_a != 1) return -2;
    if (unit != 0 && unit != 1) return -3;
    if (m < 0) return -4;
    if (n < 0) return -5;
    if (m > 0 && !A) return -6;
    if (lda < (m > 0 ? m : 1)) return -7;
    if (Abar && m > 0 && n > 0 && !X) return -9;
    if (ldx < (m > 0 ? m : 1)) return -10;
    if (m > 0 && n > 0 && !Xbar) return -12;
    if (ldxb < (m > 0 ? m : 1)) return -13;
    if (m > 0 && n > 0 && !Bbar) return -15;
    if (ldbb < (m > 0 ? m : 1)) return -16;
    if (Abar && ldab < (m > 0 ? m : 1)) return -19;
    if (batch < 0) return -21;
    if (batch > 1 && stride_bb == 0) return -17;  // outputs of different instances would race
    if (batch > 1 && Abar && stride_ab == 0) return -20;
    if (batch == 0 || m == 0 || n == 0) return BLASTGPU_SUCCESS;
    // Bbar = op(A)^{-T} Xbar: op(A)^T is A read with the transpose flipped, and its triangle is the
    // other one.
    int st = blastgpu_dtrsm_strided(uplo == BLASTGPU_LOWER ? BLASTGPU_UPPER : BLASTGPU_LOWER, !trans_a, unit, m, n,
                                    A, lda, stride_a, Xbar, ldxb, stride_xb, Bbar, ldbb, stride_bb, batch, stream);
    if (st != BLASTGPU_SUCCESS || !Abar) return st;
    unsigned blocks;
    if (!warp_grid(batch, blocks)) return BLASTGPU_ERR_TOO_LARGE;
    tri_outer_acc_kernel<<<blocks, 128, 0, as_cuda(stream)>>>(uplo, trans_a, unit, m, n, ColMat{Bbar, ldbb, stride_bb},
                                                             ColMat{const_cast<double*>(X), ldx, stride_x},
                                                             ColMat{Abar, ldab, stride_ab}, batch);
    return check_launch();
}

int blastgpu_dpotrf_bwd_strided(int n, const double* L, int ldl, int64_t stride_l, const double* Lbar, int ldlb,
                                int64_t stride_lb, double* Abar, int ldab, int64_t stride_ab, int64_t batch,
                                blastgpu_stream_t stream) {
    if (n < 0) return -1;
    if (n > 0 && !L) return -2;
    if (ldl < (n > 0 ? n : 1)) return -3;
    if (n > 0 && !Lbar) return -5;
    if (ldlb < (n > 0 ? n : 1)) return -6;
    if (n > 0 && !Abar) return -8;
    if (ldab < (n > 0 ? n : 1)) return -9;
    if (batch < 0) return -11;
    if (batch > 1 && stride_ab == 0) return -10;  // outputs of different instances would race
    if (batch == 0 || n == 0) return BLASTGPU_SUCCESS;
    unsigned blocks;
    if (!warp_grid(batch, blocks)) return BLASTGPU_ERR_TOO_LARGE;
    cudaStream_t const s = as_cuda(stream);
    ColMat const W{Abar, ldab, stride_ab};
    chol_bwd_phi_kernel<<<blocks, 128, 0, s>>>(n, ColMat{const_cast<double*>(L), ldl, stride_l},
                                               ColMat{const_cast<double*>(Lbar), ldlb, stride_lb}, W, batch);
    int st = check_launch();
    if (st != BLASTGPU_SUCCESS) return st;
    // W := L^{-T} W  (op(L) = L^T is upper triangular)
    st = blastgpu_dtrsm_strided(BLASTGPU_UPPER, 1, 0, n, n, L, ldl, stride_l, Abar, ldab, stride_ab, Abar, ldab,
                                stride_ab, batch, stream);
    if (st != BLASTGPU_SUCCESS) return st;
    // W := W L^{-1}  (solves X L = W)
    st = blastgpu_dtrsm_right_strided(BLASTGPU_LOWER, 0, 0, n, n, L, ldl, stride_l, Abar, ldab, stride_ab, Abar,
                                      ldab, stride_ab, batch, stream);
    if (st != BLASTGPU_SUCCESS) return st;
    symmetrize_kernel<<<blocks, 128, 0, s>>>(n, W, batch);
    return check_launch();
}

}  // extern "C"

// Batched gemm D = alpha*A*B + beta*C, binary64, sm_103a.
//
// Reference: blast::gemm (algorithm/Gemm.hpp:41-118) tiles D with register matrices
// (algorithm/arch/avx2/Tile.hpp:45-139) and runs, per tile, the rank-1 loop of
// register_matrix/Gemm.hpp:64-124:  acc = 0; for k: acc += a_k * b_k^T (fused); acc *= alpha;
// acc = fma(beta, C, acc); store.
//
// GPU mapping: one warp per instance. The warp's 32 lanes form a 4 x 8 grid; each lane owns an
// RM x RN register tile (BLAST's RegisterMatrix), so a warp tile is (4*RM) x (8*RN) (24 x 24 for
// RM = 6, RN = 3: every lane holds 18 accumulators and no lane idles). Operand panels of K_CHUNK
// columns of A and rows of B are staged in shared memory with coalesced loads; every lane then
// performs the same per-element sequence of fused multiply-adds as BLAST (ascending k, alpha
// scaling, fma(beta, c, .)), so the results are bit-identical to the oracle restatement.
// GB300's binary64 pipe (~1.2 TFLOP/s measured) bounds this kernel; the staging and shared-memory
// traffic are far below their own limits.
#include <cstdio>

#include "common.cuh"

namespace blastgpu {
namespace {

constexpr int kWarps = 4;    // warps (instances) per CTA
constexpr int kKChunk = 16;  // K columns staged per pass (static shared memory stays under 48 KB)

struct StridedGemm {
    int m, n, k;
    double alpha, beta;
    MatView A, B, C, D;
    int64_t sa, sb, sc, sd;
    __device__ void get(int64_t b, int& mm, int& nn, int& kk, double& al, double& be, MatView& a,
                        MatView& bm, MatView& c, MatView& d) const {
        mm = m; nn = n; kk = k; al = alpha; be = beta;
        a = A; a.p += b * sa;
        bm = B; bm.p += b * sb;
        c = C; c.p += b * sc;
        d = D; d.p += b * sd;
    }
};

struct DescGemm {
    const blastgpu_gemm_desc* desc;
    __device__ void get(int64_t b, int& mm, int& nn, int& kk, double& al, double& be, MatView& a,
                        MatView& bm, MatView& c, MatView& d) const {
        blastgpu_gemm_desc const& g = desc[b];
        mm = g.D.rows; nn = g.D.cols; kk = g.A.cols; al = g.alpha; be = g.beta;
        a = view(g.A); bm = view(g.B); c = view(g.C); d = view(g.D);
    }
};

// Adjoint of D = alpha*A*B + beta*C over descriptors (A, B as views, so op() is the view):
// which = 0 forms Abar += alpha*Dbar*B^T in A's orientation, which = 1 forms Bbar += alpha*A^T*Dbar
// in B's; both are gemms with beta = 1 on transposed views, in place. An instance whose shapes
// do not fit (gemm_bwd_ok) or whose gradient is not wanted (null data) gets m = 0.
__device__ __forceinline__ bool gemm_bwd_ok(blastgpu_gemm_bwd_desc const& g) {
    int const m = g.Dbar.rows, n = g.Dbar.cols, k = g.A.cols;
    blastgpu_mat t;
    if (!view_ok(g.Dbar) || g.A.rows != m || g.B.rows != k || g.B.cols != n) return false;
    if (g.Abar.data && !(view_ok(g.B) && transposed(g.B, t) && view_ok(g.Abar) && g.Abar.rows == m && g.Abar.cols == k))
        return false;
    if (g.Bbar.data && !(view_ok(g.A) && transposed(g.A, t) && view_ok(g.Bbar) && g.Bbar.rows == k && g.Bbar.cols == n))
        return false;
    if (g.Cbar.data && !(view_ok(g.Cbar) && g.Cbar.rows == m && g.Cbar.cols == n)) return false;
    return true;
}

struct GemmBwdBatch {
    const blastgpu_gemm_bwd_desc* desc;
    int which;
    __device__ void get(int64_t b, int& mm, int& nn, int& kk, double& al, double& be, MatView& a, MatView& bm,
                        MatView& c, MatView& d) const {
        blastgpu_gemm_bwd_desc const& g = desc[b];
        mm = nn = kk = 0;
        al = g.alpha;
        be = 1.0;
        if (!gemm_bwd_ok(g)) return;
        blastgpu_mat t;
        if (which == 0) {
            if (!g.Abar.data) return;
            transposed(g.B, t);
            mm = g.Abar.rows; nn = g.Abar.cols; kk = g.Dbar.cols;
            a = view(g.Dbar); bm = view(t); c = view(g.Abar);
        } else {
            if (!g.Bbar.data) return;
            transposed(g.A, t);
            mm = g.Bbar.rows; nn = g.Bbar.cols; kk = g.Dbar.rows;
            a = view(t); bm = view(g.Dbar); c = view(g.Bbar);
        }
        d = c;
    }
};

// Cbar += beta*Dbar (fma(beta, dbar, cbar), as the strided adjoint) and the status of every instance.
__global__ void __launch_bounds__(128) gemm_bwd_c_kernel(const blastgpu_gemm_bwd_desc* desc, int64_t count,
                                                         int32_t* status) {
    int64_t const b = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= count) return;
    blastgpu_gemm_bwd_desc const& g = desc[b];
    bool const ok = gemm_bwd_ok(g);
    if (status && lane == 0) status[b] = ok ? 0 : -1;
    if (!ok || !g.Cbar.data) return;
    MatView const Db = view(g.Dbar), Cb = view(g.Cbar);
    int const m = g.Dbar.rows, n = g.Dbar.cols;
    for (int e = lane; e < m * n; e += 32) {
        int const i = e % m, j = e / m;
        Cb(i, j) = fma(g.beta, Db(i, j), Cb(i, j));
    }
}

template <int RM, int RN, class Batch>
__global__ void __launch_bounds__(kWarps * 32) gemm_warp_kernel(Batch batch, int64_t count) {
    constexpr int WM = 4 * RM, WN = 8 * RN;
    __shared__ double sA[kWarps][kKChunk][WM];
    __shared__ double sB[kWarps][kKChunk][WN];

    int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t const b = (int64_t)blockIdx.x * kWarps + warp;
    if (b >= count) return;

    int M, N, K;
    double alpha, beta;
    MatView A, B, C, D;
    batch.get(b, M, N, K, alpha, beta, A, B, C, D);

    int const lr = lane & 3, lc = lane >> 2;
    double (*a_s)[WM] = sA[warp];
    double (*b_s)[WN] = sB[warp];

    for (int ti = 0; ti < M; ti += WM) {
        for (int tj = 0; tj < N; tj += WN) {
            double acc[RM][RN];
#pragma unroll
            for (int r = 0; r < RM; ++r)
#pragma unroll
                for (int c = 0; c < RN; ++c) acc[r][c] = 0.0;

            for (int kc = 0; kc < K; kc += kKChunk) {
                int const kn = min(kKChunk, K - kc);
                __syncwarp();
                // Stage A(ti:ti+WM, kc:kc+kn): consecutive lanes take consecutive rows.
                for (int idx = lane; idx < WM * kn; idx += 32) {
                    int const r = idx % WM, q = idx / WM;
                    a_s[q][r] = (ti + r < M) ? A(ti + r, kc + q) : 0.0;
                }
                // Stage B(kc:kc+kn, tj:tj+WN): consecutive lanes take consecutive k.
                for (int idx = lane; idx < WN * kn; idx += 32) {
                    int const q = idx % kn, c = idx / kn;
                    b_s[q][c] = (tj + c < N) ? B(kc + q, tj + c) : 0.0;
                }
                __syncwarp();
                for (int q = 0; q < kn; ++q) {
                    double av[RM], bv[RN];
#pragma unroll
                    for (int r = 0; r < RM; ++r) av[r] = a_s[q][lr * RM + r];
#pragma unroll
                    for (int c = 0; c < RN; ++c) bv[c] = b_s[q][lc * RN + c];
#pragma unroll
                    for (int c = 0; c < RN; ++c)
#pragma unroll
                        for (int r = 0; r < RM; ++r) acc[r][c] = fma(av[r], bv[c], acc[r][c]);
                }
            }
            // Epilogue: acc *= alpha; d = fma(beta, c, acc).
#pragma unroll
            for (int c = 0; c < RN; ++c) {
                int const j = tj + lc * RN + c;
                if (j < N) {
#pragma unroll
                    for (int r = 0; r < RM; ++r) {
                        int const i = ti + lr * RM + r;
                        if (i < M) D(i, j) = fma(beta, C(i, j), acc[r][c] * alpha);
                    }
                }
            }
        }
    }
}

template <class Batch>
int launch_gemm(Batch const& batch, int64_t count, int max_m, int max_n, cudaStream_t stream) {
    if (count == 0) return BLASTGPU_SUCCESS;
    int64_t const blocks64 = (count + kWarps - 1) / kWarps;
    if (blocks64 > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    dim3 const grid((unsigned)blocks64), block(kWarps * 32);
    // Warp-tile shape per size bin: by default the smallest tile that covers the instance
    // without idle lanes where possible (24 x 24 is covered exactly by RM = 6, RN = 3); the
    // autotuner may override it per bin (0 = 8x8, 1 = 16x16, 2 = 24x24, 3 = 32x32 warp tiles).
    int const mx = max_m > max_n ? max_m : max_n;
    int const dflt = (max_m <= 8 && max_n <= 8) ? 0 : (max_m <= 16 && max_n <= 16) ? 1
                   : (max_m <= 24 && max_n <= 24) ? 2 : 3;
    // gemm tiles change every 8 rows/columns, so its bins are multiples of 8 ("gemm.shape.m24").
    char key[32];
    snprintf(key, sizeof(key), "gemm.shape.m%d", ((mx + 7) / 8) * 8);
    switch (tune_get(key, dflt)) {
        case 0: gemm_warp_kernel<2, 1><<<grid, block, 0, stream>>>(batch, count); break;
        case 1: gemm_warp_kernel<4, 2><<<grid, block, 0, stream>>>(batch, count); break;
        case 2: gemm_warp_kernel<6, 3><<<grid, block, 0, stream>>>(batch, count); break;
        default: gemm_warp_kernel<8, 4><<<grid, block, 0, stream>>>(batch, count); break;
    }
    return check_launch();
}

}  // namespace
}  // namespace blastgpu

using namespace blastgpu;

extern "C" {

int blastgpu_dgemm_strided(int trans_a, int trans_b, int m, int n, int k, double alpha,
                           const double* A, int lda, int64_t stride_a,
                           const double* B, int ldb, int64_t stride_b, double beta,
                           const double* C, int ldc, int64_t stride_c,
                           double* D, int ldd, int64_t stride_d,
                           int64_t batch, blastgpu_stream_t stream) {
    if (trans_a != 0 && trans_a != 1) return -1;
    if (trans_b != 0 && trans_b != 1) return -2;
    if (m < 0) return -3;
    if (n < 0) return -4;
    if (k < 0) return -5;
    // Leading dimensions bound the stored arrays: A is m x k (k x m when trans_a), B k x n.
    if (lda < (trans_a ? (k > 0 ? k : 1) : (m > 0 ? m : 1)) && m > 0 && k > 0) return -8;
    if (ldb < (trans_b ? (n > 0 ? n : 1) : (k > 0 ? k : 1)) && n > 0 && k > 0) return -11;
    if (ldc < (m > 0 ? m : 1) && m > 0 && n > 0) return -15;
    if (ldd < (m > 0 ? m : 1) && m > 0 && n > 0) return -18;
    if (batch < 0) return -20;
    if (batch == 0 || m == 0 || n == 0) return BLASTGPU_SUCCESS;
    if (k > 0 && (!A || !B)) return !A ? -7 : -10;
    if (!C) return -14;
    if (!D) return -17;
    StridedGemm g;
    g.m = m; g.n = n; g.k = k; g.alpha = alpha; g.beta = beta;
    g.A = MatView{const_cast<double*>(A), lda, trans_a ? BLASTGPU_ROW_MAJOR : BLASTGPU_COL_MAJOR, 1};
    g.B = MatView{const_cast<double*>(B), ldb, trans_b ? BLASTGPU_ROW_MAJOR : BLASTGPU_COL_MAJOR, 1};
    g.C = MatView{const_cast<double*>(C), ldc, BLASTGPU_COL_MAJOR, 1};
    g.D = MatView{D, ldd, BLASTGPU_COL_MAJOR, 1};
    g.sa = stride_a; g.sb = stride_b; g.sc = stride_c; g.sd = stride_d;
    return launch_gemm(g, batch, m, n, as_cuda(stream));
}

int blastgpu_dgemm_bwd_batched(const blastgpu_gemm_bwd_desc* desc, int64_t batch, int max_dim, int32_t* status,
                               blastgpu_stream_t stream) {
    if (batch < 0) return -2;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (!desc) return -1;
    if (max_dim < 0) return -3;
    int64_t const blocks = (batch + 3) / 4;
    if (blocks > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    cudaStream_t const s = as_cuda(stream);
    gemm_bwd_c_kernel<<<(unsigned)blocks, 128, 0, s>>>(desc, batch, status);
    int st = check_launch();
    if (st != BLASTGPU_SUCCESS) return st;
    st = launch_gemm(GemmBwdBatch{desc, 0}, batch, max_dim, max_dim, s);
    if (st != BLASTGPU_SUCCESS) return st;
    return launch_gemm(GemmBwdBatch{desc, 1}, batch, max_dim, max_dim, s);
}

int blastgpu_dgemm_batched(const blastgpu_gemm_desc* desc, int64_t batch, int max_m, int max_n,
                           int max_k, blastgpu_stream_t stream) {
    if (batch < 0) return -2;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (!desc) return -1;
    if (max_m < 0) return -3;
    if (max_n < 0) return -4;
    if (max_k < 0) return -5;
    DescGemm g{desc};
    return launch_gemm(g, batch, max_m, max_n, as_cuda(stream));
}

}  // extern "C"

// Ragged Cholesky solves for small n (n <= 128), binary64: one warp per matrix.
//
// Reference: blast::potrf (dense/Potrf.hpp:66-106), left-looking in strips of 4 columns: each
// element of a strip first takes the fused products of all earlier columns in ascending order
// (the ger(-1, ...) loop), then RegisterMatrix::potrf / ::trsm (RegisterMatrix.hpp:566-602,
// 710-739) finish the strip column by column. The solves follow dense/Trsm.hpp:39-65.
//
// Mapping: lane l owns rows l, l + 32, ... of its matrix (MAXT row blocks), so each strip's
// register tile is MAXT x 4 per lane, the earlier columns are read coalesced (a warp reads 32
// consecutive rows of a column), and the strip's own rows are broadcast loads. The diagonal 4 x 4
// block lives in 4 consecutive lanes; its entries reach the other lanes by shuffles. Every element
// sees the same fused multiply-adds, in the same order, as the thread-per-matrix kernel
// (potrf_tile: the products of column l before those of column l + 1; then, for column c of the
// strip, the terms of the strip's columns j < c, and the scaling by the reciprocal square root of
// the pivot), so the factor and the solutions are the same bits. A thread per matrix needs far
// more matrices than a ragged batch of small n has to fill the chip, and a CTA per matrix spends
// its time on barriers; a warp per matrix has neither problem.
//
// Solves, one right-hand side at a time: the forward substitution is a column sweep (once x_l is
// final, every row below takes its term), which keeps each row's ascending order. The backward
// substitution keeps the thread-per-matrix kernel's order for row i of the 4-row block i0 .. i0+3:
// first the rows below the block in ascending order, then the block's own later rows. It runs
// one block at a time from the bottom: four lanes take the rows below, then lane 0 finishes the
// block.
#include "common.cuh"

namespace blastgpu {
namespace {

constexpr int kWarpsPerCta = 4;

// Column C of the strip at k: the terms of the strip's columns j < C (their final, scaled
// values), then the scaling by y = rsqrt_nr(pivot). The strip's rows k .. k+3 are in block T0;
// blocks above it hold no rows at or below k and are left out at compile time, rows above k + C
// in block T0 by a predicate.
template <int MAXT, int T0, int C>
__device__ __forceinline__ void strip_column(double (&acc)[MAXT][4], int k, int n, int lane, int& info) {
    int const owner = (k + C) & 31;
#pragma unroll
    for (int j = 0; j < C; ++j) {
        // l_{k+C, k+j}: row k + C's final value in column j, from the lane that holds it
        double const lcj = __shfl_sync(0xffffffffu, acc[T0][j], owner);
#pragma unroll
        for (int t = T0; t < MAXT; ++t) {
            int const i = lane + 32 * t;
            if (i - k >= C && i < n) acc[t][C] = fma(-lcj, acc[t][j], acc[t][C]);
        }
    }
    double const s = __shfl_sync(0xffffffffu, acc[T0][C], owner);
    if (!(s > 0.0) && info == 0) info = k + C + 1;
    double const y = rsqrt_nr(s);
#pragma unroll
    for (int t = T0; t < MAXT; ++t) {
        int const i = lane + 32 * t;
        if (i - k >= C && i < n) acc[t][C] *= y;
    }
}

// One strip (columns k .. k+nc-1) of the left-looking Cholesky, its rows in blocks T0 .. MAXT-1.
template <int MAXT, int T0>
__device__ __forceinline__ void warp_strip(int n, int k, const double* A, int lda, double* L, int ldl, int lane,
                                           int& info) {
    int const nc = min(4, n - k);
    double acc[MAXT][4];
#pragma unroll
    for (int t = T0; t < MAXT; ++t)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            int const i = lane + 32 * t;
            acc[t][c] = (c < nc && i < n && i - k >= c) ? A[i + (int64_t)(k + c) * lda] : 0.0;
        }
    // the earlier columns in ascending order, the next column's loads issued first
    if (k > 0) {
        double a[MAXT], b[4];
#pragma unroll
        for (int t = T0; t < MAXT; ++t) {
            int const i = lane + 32 * t;
            a[t] = (i < n && i >= k) ? L[i] : 0.0;
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) b[c] = c < nc ? L[k + c] : 0.0;
        for (int l = 0; l < k; ++l) {
            double an[MAXT], bn[4];
            int const ln = l + 1 < k ? l + 1 : l;
            double const* col = L + (int64_t)ln * ldl;
#pragma unroll
            for (int t = T0; t < MAXT; ++t) {
                int const i = lane + 32 * t;
                an[t] = (i < n && i >= k) ? col[i] : 0.0;
            }
#pragma unroll
            for (int c = 0; c < 4; ++c) bn[c] = c < nc ? col[k + c] : 0.0;
#pragma unroll
            for (int t = T0; t < MAXT; ++t) {
                int const i = lane + 32 * t;
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    if (t > T0 || i - k >= c) acc[t][c] = fma(-a[t], b[c], acc[t][c]);
            }
#pragma unroll
            for (int t = T0; t < MAXT; ++t) a[t] = an[t];
#pragma unroll
            for (int c = 0; c < 4; ++c) b[c] = bn[c];
        }
    }
    strip_column<MAXT, T0, 0>(acc, k, n, lane, info);
    if (nc > 1) strip_column<MAXT, T0, 1>(acc, k, n, lane, info);
    if (nc > 2) strip_column<MAXT, T0, 2>(acc, k, n, lane, info);
    if (nc > 3) strip_column<MAXT, T0, 3>(acc, k, n, lane, info);
#pragma unroll
    for (int t = T0; t < MAXT; ++t)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            int const i = lane + 32 * t;
            if (c < nc && i < n && i - k >= c) L[i + (int64_t)(k + c) * ldl] = acc[t][c];
        }
}

// Left-looking Cholesky of the n x n matrix A (lower triangle read) into L (lower triangle
// written), one warp. Returns 0 or the first bad pivot + 1, the same in every lane.
template <int MAXT>
__device__ int warp_potrf(int n, const double* A, int lda, double* L, int ldl, int lane) {
    int info = 0;
    for (int k = 0; k < n; k += 4) {
        switch (k >> 5) {  // the block holding rows k .. k+3 (k is a multiple of 4)
            case 0: warp_strip<MAXT, 0>(n, k, A, lda, L, ldl, lane, info); break;
            case 1: if constexpr (MAXT > 1) warp_strip<MAXT, (MAXT > 1 ? 1 : 0)>(n, k, A, lda, L, ldl, lane, info); break;
            case 2: if constexpr (MAXT > 2) warp_strip<MAXT, (MAXT > 2 ? 2 : 0)>(n, k, A, lda, L, ldl, lane, info); break;
            default: if constexpr (MAXT > 3) warp_strip<MAXT, (MAXT > 3 ? 3 : 0)>(n, k, A, lda, L, ldl, lane, info); break;
        }
        __syncwarp();  // the strip's columns are read by every lane from the next strip on
    }
    return info;
}

// Columns l of the forward sweep with l in block TL (32 TL <= l < 32 TL + 32): rows in blocks
// below TL all take the term; block TL only below l.
template <int MAXT, int TL>
__device__ __forceinline__ void fwd_sweep_block(int n, const double* L, int ldl, double (&acc)[MAXT],
                                                double const (&d)[MAXT], int lane) {
    int const l1 = min(n, 32 * TL + 32);
    for (int l = 32 * TL; l < l1; ++l) {
        double col[MAXT];
        double const* cl = L + (int64_t)l * ldl;
#pragma unroll
        for (int t = TL; t < MAXT; ++t) {
            int const i = lane + 32 * t;
            col[t] = (i > l && i < n) ? cl[i] : 0.0;
        }
        double const xl = __shfl_sync(0xffffffffu, acc[TL] * d[TL], l & 31);
#pragma unroll
        for (int t = TL; t < MAXT; ++t) {
            int const i = lane + 32 * t;
            if (i == l) acc[t] = xl;
            else if (i > l && i < n) acc[t] = fma(-col[t], xl, acc[t]);
        }
    }
}

// X(:, j) = A^{-1} B(:, j) from the factor L, one warp; xs: n doubles of shared memory.
template <int MAXT>
__device__ void warp_potrs_column(int n, const double* L, int ldl, const double* bcol, double* xcol, double* xs,
                                  int lane) {
    // forward: L y = b, column sweep
    double acc[MAXT], d[MAXT];
#pragma unroll
    for (int t = 0; t < MAXT; ++t) {
        int const i = lane + 32 * t;
        acc[t] = i < n ? bcol[i] : 0.0;
        d[t] = i < n ? rcp_nr(L[i + (int64_t)i * ldl]) : 0.0;
    }
    fwd_sweep_block<MAXT, 0>(n, L, ldl, acc, d, lane);
    if constexpr (MAXT > 1) fwd_sweep_block<MAXT, (MAXT > 1 ? 1 : 0)>(n, L, ldl, acc, d, lane);
    if constexpr (MAXT > 2) fwd_sweep_block<MAXT, (MAXT > 2 ? 2 : 0)>(n, L, ldl, acc, d, lane);
    if constexpr (MAXT > 3) fwd_sweep_block<MAXT, (MAXT > 3 ? 3 : 0)>(n, L, ldl, acc, d, lane);
#pragma unroll
    for (int t = 0; t < MAXT; ++t) {
        int const i = lane + 32 * t;
        if (i < n) xs[i] = acc[t];
    }
    __syncwarp();
    // backward: L^T x = y, 4-row blocks from the bottom
    __shared__ double part[kWarpsPerCta][4];
    int const w = threadIdx.x >> 5;
    for (int i0 = ((n - 1) / 4) * 4; i0 >= 0; i0 -= 4) {
        int const ni = min(4, n - i0);
        if (lane < ni) {
            int const i = i0 + lane;
            double const* li = L + (int64_t)i * ldl;  // column i of L: L(l, i) for l > i
            double s = xs[i];
            int l = i0 + 4;
            for (; l + 8 <= n; l += 8) {
                double v[8], x[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    v[u] = li[l + u];
                    x[u] = xs[l + u];
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) s = fma(-v[u], x[u], s);
            }
            for (; l < n; ++l) s = fma(-li[l], xs[l], s);
            part[w][lane] = s;
        }
        __syncwarp();
        if (lane == 0) {
            double xb[4];
            for (int r = ni - 1; r >= 0; --r) {
                int const i = i0 + r;
                double s = part[w][r];
                for (int q = r + 1; q < ni; ++q) s = fma(-L[(i0 + q) + (int64_t)i * ldl], xb[q], s);
                xb[r] = s * rcp_nr(L[i + (int64_t)i * ldl]);
                xs[i] = xb[r];
            }
        }
        __syncwarp();
    }
    for (int i = lane; i < n; i += 32) xcol[i] = xs[i];
    __syncwarp();
}

// One instance with n <= 32 NB: its row blocks (NB of them) fix the register tiles, so the
// blocks past its last row cost nothing.
template <int NB>
__device__ __forceinline__ void warp_posv(blastgpu_posv_desc const& dsc, int n, double* xs, int lane, int32_t* info_b) {
    if (dsc.A.data != nullptr) {  // A == nullptr: solves with the given factor L only
        int const r = warp_potrf<NB>(n, dsc.A.data, dsc.A.ld, dsc.L.data, dsc.L.ld, lane);
        if (info_b && lane == 0) *info_b = r;
    }
    for (int j = 0; j < dsc.B.cols; ++j)
        warp_potrs_column<NB>(n, dsc.L.data, dsc.L.ld, dsc.B.data + (int64_t)j * dsc.B.ld,
                              dsc.X.data + (int64_t)j * dsc.X.ld, xs, lane);
}

template <int MAXT>
__global__ void __launch_bounds__(kWarpsPerCta * 32) posv_warp_kernel(const blastgpu_posv_desc* desc, int64_t count,
                                                                     int32_t* info) {
    __shared__ double xs_all[kWarpsPerCta][32 * MAXT];
    int const w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t const b = (int64_t)blockIdx.x * kWarpsPerCta + w;
    if (b >= count) return;
    blastgpu_posv_desc const& dsc = desc[b];
    int const n = dsc.A.rows;
    if (n > 32 * MAXT) return;  // the launch's max_n bounds every instance
    int32_t* const info_b = info ? info + b : nullptr;
    switch ((n + 31) >> 5) {
        case 0:
        case 1: warp_posv<1>(dsc, n, xs_all[w], lane, info_b); break;
        case 2: if constexpr (MAXT >= 2) warp_posv<(MAXT >= 2 ? 2 : 1)>(dsc, n, xs_all[w], lane, info_b); break;
        case 3: if constexpr (MAXT >= 3) warp_posv<(MAXT >= 3 ? 3 : 1)>(dsc, n, xs_all[w], lane, info_b); break;
        default: if constexpr (MAXT >= 4) warp_posv<(MAXT >= 4 ? 4 : 1)>(dsc, n, xs_all[w], lane, info_b); break;
    }
}

// Adjoint of X = A^{-1} B for one instance, one warp (as posv_bwd_kernel, which runs a CTA per
// matrix): the factor kept in L or recomputed from A, dl/dB = A^{-1} dl/dX with the warp's solve,
// dl/dA = -(dl/dB X^T + X dl/dB^T)/2 written by lanes over rows, a column at a time.
template <int NB>
__device__ __forceinline__ void warp_posv_bwd(blastgpu_posv_bwd_desc const& d, int n, int recompute, double* xs,
                                              int lane, int32_t* info_b) {
    if (recompute) {
        int const r = warp_potrf<NB>(n, d.A.data, d.A.ld, d.L.data, d.L.ld, lane);
        if (info_b && lane == 0) *info_b = r;
    } else if (info_b && lane == 0) {
        *info_b = 0;
    }
    int const nrhs = d.X.cols;
    for (int c = 0; c < nrhs; ++c)
        warp_potrs_column<NB>(n, d.L.data, d.L.ld, d.Xbar.data + (int64_t)c * d.Xbar.ld,
                              d.Bbar.data + (int64_t)c * d.Bbar.ld, xs, lane);
    if (nrhs == 1) {  // dl/dB is still in xs
        double xi[NB], gi[NB];
#pragma unroll
        for (int t = 0; t < NB; ++t) {
            int const i = lane + 32 * t;
            xi[t] = i < n ? d.X.data[i] : 0.0;
            gi[t] = i < n ? xs[i] : 0.0;
        }
        for (int j = 0; j < n; ++j) {
            double const xj = d.X.data[j], gj = xs[j];
            double* ga = d.Abar.data + (int64_t)j * d.Abar.ld;
#pragma unroll
            for (int t = 0; t < NB; ++t) {
                int const i = lane + 32 * t;
                if (i < n) ga[i] = -0.5 * fma(xi[t], gj, gi[t] * xj);
            }
        }
        return;
    }
    __syncwarp();  // dl/dB columns are complete in memory
    for (int j = 0; j < n; ++j)
        for (int i = lane; i < n; i += 32) {
            double acc = 0.0;
            for (int c = 0; c < nrhs; ++c) {
                acc = fma(d.Bbar.data[i + (int64_t)c * d.Bbar.ld], d.X.data[j + (int64_t)c * d.X.ld], acc);
                acc = fma(d.X.data[i + (int64_t)c * d.X.ld], d.Bbar.data[j + (int64_t)c * d.Bbar.ld], acc);
            }
            d.Abar.data[i + (int64_t)j * d.Abar.ld] = -0.5 * acc;
        }
}

template <int MAXT>
__global__ void __launch_bounds__(kWarpsPerCta * 32) posv_bwd_warp_kernel(const blastgpu_posv_bwd_desc* desc,
                                                                         int64_t count, int recompute, int32_t* info) {
    __shared__ double xs_all[kWarpsPerCta][32 * MAXT];
    int const w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t const b = (int64_t)blockIdx.x * kWarpsPerCta + w;
    if (b >= count) return;
    blastgpu_posv_bwd_desc const& d = desc[b];
    int const n = d.A.rows;
    if (n > 32 * MAXT) return;  // the launch's max_n bounds every instance
    int32_t* const info_b = info ? info + b : nullptr;
    switch ((n + 31) >> 5) {
        case 0:
        case 1: warp_posv_bwd<1>(d, n, recompute, xs_all[w], lane, info_b); break;
        case 2: if constexpr (MAXT >= 2) warp_posv_bwd<(MAXT >= 2 ? 2 : 1)>(d, n, recompute, xs_all[w], lane, info_b); break;
        case 3: if constexpr (MAXT >= 3) warp_posv_bwd<(MAXT >= 3 ? 3 : 1)>(d, n, recompute, xs_all[w], lane, info_b); break;
        default: if constexpr (MAXT >= 4) warp_posv_bwd<(MAXT >= 4 ? 4 : 1)>(d, n, recompute, xs_all[w], lane, info_b); break;
    }
}

}  // namespace

// Adjoints of ragged binary64 Cholesky solves with every n <= 128, one warp per matrix
// (blastgpu_dposv_bwd_batched routes such launches here unless "posv.warp_bwd.n<bin>" is 0).
int launch_posv_bwd_warp(const blastgpu_posv_bwd_desc* desc, int64_t count, int max_n, int recompute, int32_t* info,
                         cudaStream_t s) {
    if (count == 0) return BLASTGPU_SUCCESS;
    int64_t const blocks = (count + kWarpsPerCta - 1) / kWarpsPerCta;
    if (blocks > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    unsigned const g = (unsigned)blocks, t = kWarpsPerCta * 32;
    if (max_n <= 32) posv_bwd_warp_kernel<1><<<g, t, 0, s>>>(desc, count, recompute, info);
    else if (max_n <= 64) posv_bwd_warp_kernel<2><<<g, t, 0, s>>>(desc, count, recompute, info);
    else if (max_n <= 128) posv_bwd_warp_kernel<4><<<g, t, 0, s>>>(desc, count, recompute, info);
    else return BLASTGPU_ERR_TOO_LARGE;
    return check_launch();
}

// Ragged binary64 Cholesky solves with every n <= 128, one warp per matrix (blastgpu_dposv_batched
// routes such launches here unless "posv.warp.n<bin>" is 0).
int launch_posv_warp(const blastgpu_posv_desc* desc, int64_t count, int max_n, int32_t* info, cudaStream_t s) {
    if (count == 0) return BLASTGPU_SUCCESS;
    int64_t const blocks = (count + kWarpsPerCta - 1) / kWarpsPerCta;
    if (blocks > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    unsigned const g = (unsigned)blocks, t = kWarpsPerCta * 32;
    if (max_n <= 32) posv_warp_kernel<1><<<g, t, 0, s>>>(desc, count, info);
    else if (max_n <= 64) posv_warp_kernel<2><<<g, t, 0, s>>>(desc, count, info);
    else if (max_n <= 128) posv_warp_kernel<4><<<g, t, 0, s>>>(desc, count, info);
    else return BLASTGPU_ERR_TOO_LARGE;
    return check_launch();
}

}  // namespace blastgpu

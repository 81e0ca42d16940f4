// Batched LU with partial pivoting (getrf), row interchanges (laswp) and the LU solve (getrs),
// binary64, sm_103a.
//
// Reference: blast::getrf (dense/Getrf.hpp:52-119), right-looking with NB = TileSize<double> = 4:
//   getf2 on the (M-k) x 4 panel (dense/Getf2.hpp:52-77: iamax pivot, swap within the panel,
//   singular check, scale by the pivot, rank-1 update), pivot adjustment, laswp of the other
//   columns (dense/Laswp.hpp:37-43), U12 := L11^{-1} A12 (trsm<Lower, unit>, dense/Trsm.hpp),
//   A22 := A22 - A21*U12 through gemm (K = 4: acc = sum of fused products from 0, d = c - acc);
//   unblocked getf2 on the remainder; laswp of the left columns.
// BLAST has no getrs: it is laswp(b), trsm<Lower, unit>, trsm<Upper> (scalar loops, dense/Trsm.hpp).
//
// GPU mapping:
//  * getrf: one warp per matrix, the matrix in global memory (L1/L2 resident while its warp works
//    on it). Lanes split every step: the pivot search is a warp-shuffle argmax that keeps the
//    first maximum (BLAST's strict '>' scan, dense/Iamax.hpp:82-95), swaps and laswp go lane per
//    column, scaling and rank-1 updates lane per row, the trailing update lane per element.
//    Every element sees exactly BLAST's sequence of rounded operations (the pivot scaling is an
//    IEEE division, as in BLAST), so factors and pivot sequences are bit-identical to the oracle.
//  * getrs: one thread per matrix. The backward substitution is a chain of dependent dot
//    products in BLAST's order (each x_i starts from x_{i+1}); running whole solves per thread
//    keeps every lane busy while preserving that order.
#include "common.cuh"

namespace blastgpu {
namespace {

constexpr int kWarps = 4;  // matrices (warps) per CTA of the getrf kernel

struct GetrfItem {
    double* a;
    int m, n, lda;
    int32_t* ipiv;
};

struct StridedGetrf {
    int m, n, lda;
    double* A;
    int64_t sa;
    int32_t* ipiv;
    int64_t sp;
    __device__ GetrfItem get(int64_t b) const { return {A + b * sa, m, n, lda, ipiv + b * sp}; }
};

struct DescGetrf {
    const blastgpu_getrf_desc* desc;
    __device__ GetrfItem get(int64_t b) const {
        blastgpu_getrf_desc const& d = desc[b];
        return {d.A.data, d.A.rows, d.A.cols, d.A.ld, d.ipiv};
    }
};

// First index of the largest |x|, rows [r0, r1) of column j, as BLAST's scalar scan would find:
// a value replaces the running maximum only if strictly larger, so the first maximum wins and
// NaN never wins unless it is the first element (then nothing replaces it).
__device__ __forceinline__ int warp_iamax(const double* a, int lda, int r0, int r1, int j, int lane) {
    double best = -1.0;
    int idx = 0x7fffffff;
    for (int r = r0 + lane; r < r1; r += 32) {
        double const v = fabs(a[r + (int64_t)j * lda]);
        if (v > best) { best = v; idx = r; }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        double const ob = __shfl_xor_sync(0xffffffffu, best, off);
        int const oi = __shfl_xor_sync(0xffffffffu, idx, off);
        if (ob > best || (ob == best && oi < idx)) { best = ob; idx = oi; }
    }
    double const first = a[r0 + (int64_t)j * lda];
    if (first != first || idx == 0x7fffffff) idx = r0;  // NaN first element, or all NaN
    return idx - r0;
}

// getf2 (dense/Getf2.hpp:52-77) on the m x n block at (r0, c0); swaps cover the block's columns.
// ipiv receives block-relative pivots. Returns the block-relative k+1 of a zero pivot, or 0.
__device__ int warp_getf2(double* a, int lda, int r0, int c0, int m, int n, int32_t* ipiv, int lane) {
    for (int k = 0; k < m && k < n; ++k) {
        int const ip = warp_iamax(a, lda, r0 + k, r0 + m, c0 + k, lane) + k;
        if (lane == 0) ipiv[k] = ip;
        if (ip != k) {
            for (int j = lane; j < n; j += 32) {
                double* p = a + (int64_t)(c0 + j) * lda;
                double const t = p[r0 + k];
                p[r0 + k] = p[r0 + ip];
                p[r0 + ip] = t;
            }
        }
        __syncwarp();
        double const piv = a[(r0 + k) + (int64_t)(c0 + k) * lda];
        if (piv == 0.0) return k + 1;
        double* col = a + (int64_t)(c0 + k) * lda;
        for (int i = k + 1 + lane; i < m; i += 32) col[r0 + i] = col[r0 + i] / piv;
        __syncwarp();
        for (int j = k + 1; j < n; ++j) {
            double* cj = a + (int64_t)(c0 + j) * lda;
            double const y = cj[r0 + k];
            for (int i = k + 1 + lane; i < m; i += 32) cj[r0 + i] = fma(-col[r0 + i], y, cj[r0 + i]);
        }
        __syncwarp();
    }
    return 0;
}

// laswp on columns [c0, c1) with pivots ipiv[k0..k1) (dense/Laswp.hpp:37-43), lane per column.
__device__ __forceinline__ void warp_laswp(double* a, int lda, int c0, int c1, int k0, int k1,
                                           const int32_t* ipiv, int lane) {
    for (int j = c0 + lane; j < c1; j += 32) {
        double* p = a + (int64_t)j * lda;
        for (int k = k0; k < k1; ++k) {
            int const q = ipiv[k];
            if (q != k) {
                double const t = p[k];
                p[k] = p[q];
                p[q] = t;
            }
        }
    }
}

__device__ int warp_getrf(GetrfItem it, int lane) {
    constexpr int NB = 4;
    int const M = it.m, N = it.n, lda = it.lda;
    double* a = it.a;
    int32_t* ipiv = it.ipiv;
    int k = 0;
    for (; k + NB < M && k + NB < N; k += NB) {
        int const r = warp_getf2(a, lda, k, k, M - k, NB, ipiv + k, lane);
        __syncwarp();
        if (lane < NB) ipiv[k + lane] += k;
        __syncwarp();
        if (r) return k + r;
        warp_laswp(a, lda, 0, k, k, k + NB, ipiv, lane);
        warp_laswp(a, lda, k + NB, N, k, k + NB, ipiv, lane);
        __syncwarp();
        // U12 := L11^{-1} A12, lane per column (trsm<Lower, unit>, scalar order).
        for (int j = k + NB + lane; j < N; j += 32) {
            double* cj = a + (int64_t)j * lda;
            double x[NB];
#pragma unroll
            for (int i = 0; i < NB; ++i) {
                double acc = cj[k + i];
#pragma unroll
                for (int q = 0; q < i; ++q) acc = fma(-a[(k + i) + (int64_t)(k + q) * lda], x[q], acc);
                x[i] = acc;
                cj[k + i] = acc;
            }
        }
        __syncwarp();
        // A22 := A22 - A21 * U12 (gemm with K = 4, alpha = -1, beta = 1), lane per element.
        int const mr = M - k - NB, nr = N - k - NB;
        int const total = mr * nr;
        for (int e = lane; e < total; e += 32) {
            int const i = k + NB + e % mr, j = k + NB + e / mr;
            double acc = 0.0;
#pragma unroll
            for (int q = 0; q < NB; ++q) acc = fma(a[i + (int64_t)(k + q) * lda], a[(k + q) + (int64_t)j * lda], acc);
            double* c = a + i + (int64_t)j * lda;
            *c = fma(1.0, *c, -acc);
        }
        __syncwarp();
    }
    if (k < M && k < N) {
        int const r = warp_getf2(a, lda, k, k, M - k, N - k, ipiv + k, lane);
        __syncwarp();
        for (int i = k + lane; i < M && i < N; i += 32) ipiv[i] += k;
        __syncwarp();
        if (r) return k + r;
    }
    warp_laswp(a, lda, 0, k, k, min(M, N), ipiv, lane);
    __syncwarp();
    return 0;
}

// CTA-per-matrix getrf for larger n: the same steps as warp_getrf, with the panel factorised by
// warp 0 and the swaps, U12 solve and trailing update spread over the whole CTA. In the trailing
// update each thread owns rows, keeps the row's four A21 entries in registers and reads U12
// (the same for all threads) from L1, so one fused chain per element costs one load and one
// store; fewer matrices in flight keep the working set in L2.
constexpr int kCtaThreads = 256;

constexpr int kPanelRows = 512;  // panels up to this height are factored in shared memory

__device__ int cta_getrf(GetrfItem it, int* s_ret, double* sp) {
    constexpr int NB = 4;
    int const M = it.m, N = it.n, lda = it.lda;
    double* a = it.a;
    int32_t* ipiv = it.ipiv;
    int const tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int k = 0;
    for (; k + NB < M && k + NB < N; k += NB) {
        int const mk = M - k;
        if (mk <= kPanelRows) {
            // The (M-k) x 4 panel goes to shared memory, is factored there by warp 0 (same
            // operations, shared-memory latency instead of global), and is written back.
            for (int idx = tid; idx < NB * mk; idx += kCtaThreads) {
                int const c = idx / mk, r = idx - c * mk;
                sp[c * kPanelRows + r] = a[(k + r) + (int64_t)(k + c) * lda];
            }
            __syncthreads();
            if (warp == 0) {
                int const r = warp_getf2(sp, kPanelRows, 0, 0, mk, NB, ipiv + k, lane);
                __syncwarp();
                if (lane < NB) ipiv[k + lane] += k;
                if (lane == 0) *s_ret = r;
            }
            __syncthreads();
            for (int idx = tid; idx < NB * mk; idx += kCtaThreads) {
                int const c = idx / mk, r = idx - c * mk;
                a[(k + r) + (int64_t)(k + c) * lda] = sp[c * kPanelRows + r];
            }
        } else if (warp == 0) {
            int const r = warp_getf2(a, lda, k, k, M - k, NB, ipiv + k, lane);
            __syncwarp();
            if (lane < NB) ipiv[k + lane] += k;
            if (lane == 0) *s_ret = r;
        }
        __syncthreads();
        if (*s_ret) return k + *s_ret;
        // laswp on the other columns, thread per column
        for (int j = tid; j < N; j += kCtaThreads) {
            if (j >= k && j < k + NB) continue;
            double* p = a + (int64_t)j * lda;
            for (int q = k; q < k + NB; ++q) {
                int const pr = ipiv[q];
                if (pr != q) {
                    double const t = p[q];
                    p[q] = p[pr];
                    p[pr] = t;
                }
            }
        }
        __syncthreads();
        // U12 := L11^{-1} A12, thread per column
        for (int j = k + NB + tid; j < N; j += kCtaThreads) {
            double* cj = a + (int64_t)j * lda;
            double x[NB];
#pragma unroll
            for (int i = 0; i < NB; ++i) {
                double acc = cj[k + i];
#pragma unroll
                for (int q = 0; q < i; ++q) acc = fma(-a[(k + i) + (int64_t)(k + q) * lda], x[q], acc);
                x[i] = acc;
                cj[k + i] = acc;
            }
        }
        __syncthreads();
        // A22 := A22 - A21 * U12, thread per row
        for (int i = k + NB + tid; i < M; i += kCtaThreads) {
            double l[NB];
#pragma unroll
            for (int q = 0; q < NB; ++q) l[q] = a[i + (int64_t)(k + q) * lda];
            for (int j = k + NB; j < N; ++j) {
                double const* u = a + k + (int64_t)j * lda;
                double acc = 0.0;
#pragma unroll
                for (int q = 0; q < NB; ++q) acc = fma(l[q], u[q], acc);
                double* c = a + i + (int64_t)j * lda;
                *c = fma(1.0, *c, -acc);
            }
        }
        __syncthreads();
    }
    if (k < M && k < N) {
        if (warp == 0) {
            int const r = warp_getf2(a, lda, k, k, M - k, N - k, ipiv + k, lane);
            __syncwarp();
            for (int i = k + lane; i < M && i < N; i += 32) ipiv[i] += k;
            if (lane == 0) *s_ret = r;
        }
        __syncthreads();
        if (*s_ret) return k + *s_ret;
    }
    for (int j = tid; j < k; j += kCtaThreads) {
        double* p = a + (int64_t)j * lda;
        for (int q = k; q < min(M, N); ++q) {
            int const pr = ipiv[q];
            if (pr != q) {
                double const t = p[q];
                p[q] = p[pr];
                p[pr] = t;
            }
        }
    }
    __syncthreads();
    return 0;
}

template <class Batch>
__global__ void __launch_bounds__(kCtaThreads) getrf_cta_kernel(Batch batch, int64_t count, int32_t* info) {
    __shared__ int s_ret;
    __shared__ double s_panel[4 * kPanelRows];
    int64_t const b = blockIdx.x;
    if (b >= count) return;
    GetrfItem const it = batch.get(b);
    int const r = cta_getrf(it, &s_ret, s_panel);
    if (info && threadIdx.x == 0) info[b] = r;
}

template <class Batch>
__global__ void __launch_bounds__(kWarps * 32) getrf_warp_kernel(Batch batch, int64_t count, int32_t* info) {
    int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t const b = (int64_t)blockIdx.x * kWarps + warp;
    if (b >= count) return;
    GetrfItem const it = batch.get(b);
    int const r = warp_getrf(it, lane);
    if (info && lane == 0) info[b] = r;
}

// getrs for one matrix and its right-hand sides, in BLAST's scalar order (dense/Trsm.hpp:39-65):
// laswp(b) with ipiv[0..n), x_i = b_i - sum_{k<i} l_ik x_k (unit lower), then
// x_i = (x_i - sum_{k>i, ascending} u_ik x_k) / u_ii.
__device__ void getrs_thread(int n, int nrhs, const double* a, int lda, const int32_t* ipiv,
                             double* x, int ldx) {
    for (int j = 0; j < nrhs; ++j) {
        double* xj = x + (int64_t)j * ldx;
        for (int k = 0; k < n; ++k) {
            int const q = ipiv[k];
            if (q != k) {
                double const t = xj[k];
                xj[k] = xj[q];
                xj[q] = t;
            }
        }
        // The dot products keep BLAST's ascending order; each pass of 16 issues its 32 loads before
        // the 16 dependent fused multiply-adds, so the thread waits for memory once per 16 terms.
        for (int i = 0; i < n; ++i) {
            double acc = xj[i];
            int k = 0;
            for (; k + 16 <= i; k += 16) {
                double av[16], xv[16];
#pragma unroll
                for (int u = 0; u < 16; ++u) {
                    av[u] = a[i + (int64_t)(k + u) * lda];
                    xv[u] = xj[k + u];
                }
#pragma unroll
                for (int u = 0; u < 16; ++u) acc = fma(-av[u], xv[u], acc);
            }
            for (; k < i; ++k) acc = fma(-a[i + (int64_t)k * lda], xj[k], acc);
            xj[i] = acc;
        }
        for (int i = n; i-- > 0;) {
            double acc = xj[i];
            int k = i + 1;
            for (; k + 16 <= n; k += 16) {
                double av[16], xv[16];
#pragma unroll
                for (int u = 0; u < 16; ++u) {
                    av[u] = a[i + (int64_t)(k + u) * lda];
                    xv[u] = xj[k + u];
                }
#pragma unroll
                for (int u = 0; u < 16; ++u) acc = fma(-av[u], xv[u], acc);
            }
            for (; k < n; ++k) acc = fma(-a[i + (int64_t)k * lda], xj[k], acc);
            xj[i] = acc / a[i + (int64_t)i * lda];
        }
    }
}

struct GetrsItem {
    const double* a;
    int n, lda;
    const int32_t* ipiv;
    double* x;
    int nrhs, ldx;
};

struct StridedGetrs {
    int n, nrhs, lda, ldx;
    const double* A;
    int64_t sa;
    const int32_t* ipiv;
    int64_t sp;
    double* X;
    int64_t sx;
    __device__ GetrsItem get(int64_t b) const {
        return {A + b * sa, n, lda, ipiv + b * sp, X + b * sx, nrhs, ldx};
    }
};

struct DescGetrs {
    const blastgpu_getrf_desc* desc;
    __device__ GetrsItem get(int64_t b) const {
        blastgpu_getrf_desc const& d = desc[b];
        return {d.A.data, d.A.rows, d.A.ld, d.ipiv, d.B.data, d.B.cols, d.B.ld};
    }
};

template <class Batch>
__global__ void __launch_bounds__(128) getrs_thread_kernel(Batch batch, int64_t count, const int32_t* info) {
    int64_t const b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= count) return;
    if (info && info[b] != 0) return;  // singular factor: BLAST would have thrown in getrf
    GetrsItem const it = batch.get(b);
    getrs_thread(it.n, it.nrhs, it.a, it.lda, it.ipiv, it.x, it.ldx);
}

// Lane-interleaved getrs. Thread-per-matrix solves read a different matrix in every lane, so each
// load instruction touches 32 unrelated sectors and the chains stall on memory. The interleaved
// path first copies each group of 32 consecutive instances into a workspace region where element
// (i, k) of instance 32w + l sits at off_w + (k * nmax_w + i) * 32 + l (nmax_w: the group's largest
// n), then solves with the same per-thread chains in BLAST's order, now reading 256 contiguous
// bytes per warp load. The right-hand sides follow at off_w + 32 nmax_w^2 + (j * nmax_w + k) * 32 + l.
__device__ __forceinline__ int group_nmax(DescGetrs const& batch, int64_t count, int64_t b0, int lane, int& n_own,
                                          int& r_max) {
    int n = 0, r = 0;
    if (b0 + lane < count) {
        blastgpu_getrf_desc const& d = batch.desc[b0 + lane];
        n = d.A.rows;
        r = d.B.cols;
    }
    n_own = n;
    int nm = n;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        nm = max(nm, __shfl_xor_sync(0xffffffffu, nm, off));
        r = max(r, __shfl_xor_sync(0xffffffffu, r, off));
    }
    r_max = r;
    return nm;
}

// One CTA (8 warps) per group of 32 instances: warp w copies rows i = w, w+8, ... of every column,
// lane l taking instance 32g + l (the 8 warps together read 8 consecutive rows of a column, so the
// sectors are shared through L1); stores are 256 contiguous bytes per warp.
__global__ void __launch_bounds__(256) getrs_interleave_kernel(DescGetrs batch, int64_t count, const int64_t* offsets,
                                                               double* ws) {
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t const b0 = (int64_t)blockIdx.x * 32;
    int n_own, r_max;
    int const nmax = group_nmax(batch, count, b0, lane, n_own, r_max);
    double* dst = ws + offsets[blockIdx.x];
    const double* a = nullptr;
    int lda = 1;
    if (n_own > 0) {
        blastgpu_getrf_desc const& d = batch.desc[b0 + lane];
        a = d.A.data;
        lda = d.A.ld;
    }
    for (int k = 0; k < nmax; ++k)
        for (int i = warp; i < nmax; i += 8)
            dst[((int64_t)k * nmax + i) * 32 + lane] = (i < n_own && k < n_own) ? a[i + (int64_t)k * lda] : 0.0;
}

// Thread per instance on the interleaved copy: laswp, unit-lower and upper substitution in
// BLAST's order (identical chains to getrs_thread), 16 loads issued ahead of their FMAs.
__global__ void __launch_bounds__(32) getrs_interleaved_kernel(DescGetrs batch, int64_t count, const int32_t* info,
                                                               const int64_t* offsets, double* ws) {
    int const lane = threadIdx.x;
    int64_t const b0 = (int64_t)blockIdx.x * 32;
    int n, r_max;
    int const nmax = group_nmax(batch, count, b0, lane, n, r_max);
    if (n == 0) return;
    if (info && info[b0 + lane] != 0) return;  // singular factor: BLAST would have thrown in getrf
    GetrsItem const it = batch.get(b0 + lane);
    const double* A = ws + offsets[blockIdx.x];
    double* X = ws + offsets[blockIdx.x] + (int64_t)32 * nmax * nmax;
    auto a = [&](int i, int k) -> double { return A[((int64_t)k * nmax + i) * 32 + lane]; };
    for (int j = 0; j < it.nrhs; ++j) {
        double* x = X + (int64_t)j * nmax * 32 + lane;  // x[k * 32]
        const double* bj = it.x + (int64_t)j * it.ldx;
        for (int k = 0; k < n; ++k) x[k * 32] = bj[k];
        for (int k = 0; k < n; ++k) {
            int const q = it.ipiv[k];
            if (q != k) {
                double const t = x[k * 32];
                x[k * 32] = x[q * 32];
                x[q * 32] = t;
            }
        }
        for (int i = 0; i < n; ++i) {
            double acc = x[i * 32];
            int k = 0;
            for (; k + 16 <= i; k += 16) {
                double av[16], xv[16];
#pragma unroll
                for (int u = 0; u < 16; ++u) {
                    av[u] = a(i, k + u);
                    xv[u] = x[(k + u) * 32];
                }
#pragma unroll
                for (int u = 0; u < 16; ++u) acc = fma(-av[u], xv[u], acc);
            }
            for (; k < i; ++k) acc = fma(-a(i, k), x[k * 32], acc);
            x[i * 32] = acc;
        }
        for (int i = n; i-- > 0;) {
            double acc = x[i * 32];
            int k = i + 1;
            for (; k + 16 <= n; k += 16) {
                double av[16], xv[16];
#pragma unroll
                for (int u = 0; u < 16; ++u) {
                    av[u] = a(i, k + u);
                    xv[u] = x[(k + u) * 32];
                }
#pragma unroll
                for (int u = 0; u < 16; ++u) acc = fma(-av[u], xv[u], acc);
            }
            for (; k < n; ++k) acc = fma(-a(i, k), x[k * 32], acc);
            x[i * 32] = acc / a(i, i);
        }
        double* out = it.x + (int64_t)j * it.ldx;
        for (int k = 0; k < n; ++k) out[k] = x[k * 32];
    }
}

// "getrf.cta.n<bin>" = 1 selects the CTA-per-matrix kernel for that size bin; by default it is
// used above n = 64, the warp-per-matrix kernel below.
template <class Batch>
int launch_getrf(Batch const& batch, int64_t count, int max_n, int32_t* info, cudaStream_t s) {
    bool const cta = tune_get_bin("getrf.cta", max_n, max_n > 64 ? 1 : 0) != 0;
    if (cta) {
        if (count > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
        getrf_cta_kernel<<<(unsigned)count, kCtaThreads, 0, s>>>(batch, count, info);
    } else {
        int64_t const blocks = (count + kWarps - 1) / kWarps;
        if (blocks > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
        getrf_warp_kernel<<<(unsigned)blocks, kWarps * 32, 0, s>>>(batch, count, info);
    }
    return check_launch();
}

template <class Batch>
int launch_getrs(Batch const& batch, int64_t count, const int32_t* info, cudaStream_t s) {
    int64_t const blocks = (count + 127) / 128;
    if (blocks > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    getrs_thread_kernel<<<(unsigned)blocks, 128, 0, s>>>(batch, count, info);
    return check_launch();
}

}  // namespace
}  // namespace blastgpu

using namespace blastgpu;

extern "C" {

int blastgpu_dgetrf_strided(int m, int n, double* A, int lda, int64_t stride_a, int32_t* ipiv,
                            int64_t stride_ipiv, int32_t* info, int64_t batch, blastgpu_stream_t stream) {
    if (m < 0) return -1;
    if (n < 0) return -2;
    if (m > 0 && n > 0 && !A) return -3;
    if (lda < (m > 0 ? m : 1)) return -4;
    if (m > 0 && n > 0 && !ipiv) return -6;
    if (batch < 0) return -9;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (m == 0 || n == 0) {
        if (info) {
            cudaError_t const e = cudaMemsetAsync(info, 0, sizeof(int32_t) * batch, as_cuda(stream));
            if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
        }
        return BLASTGPU_SUCCESS;
    }
    StridedGetrf g{m, n, lda, A, stride_a, ipiv, stride_ipiv};
    return launch_getrf(g, batch, m > n ? m : n, info, as_cuda(stream));
}

int blastgpu_dgetrf_batched(const blastgpu_getrf_desc* desc, int32_t* info, int64_t batch,
                            int max_n, blastgpu_stream_t stream) {
    if (batch < 0) return -3;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (!desc) return -1;
    if (max_n < 0) return -4;
    return launch_getrf(DescGetrf{desc}, batch, max_n, info, as_cuda(stream));
}

int64_t blastgpu_dgetrs_interleave_plan(const int32_t* n, const int32_t* nrhs, int64_t batch, int64_t* offsets) {
    if (batch < 0 || (batch > 0 && (!n || !nrhs))) return -1;
    int64_t const groups = (batch + 31) / 32;
    int64_t total = 0;
    for (int64_t g = 0; g < groups; ++g) {
        int64_t nm = 0, rm = 0;
        for (int64_t b = 32 * g; b < batch && b < 32 * g + 32; ++b) {
            if (n[b] < 0 || nrhs[b] < 0) return -1;
            nm = n[b] > nm ? n[b] : nm;
            rm = nrhs[b] > rm ? nrhs[b] : rm;
        }
        if (offsets) offsets[g] = total;
        total += 32 * (nm * nm + nm * rm);
    }
    if (offsets) offsets[groups] = total;
    return total * (int64_t)sizeof(double);
}

int blastgpu_dgetrs_batched_ws(const blastgpu_getrf_desc* desc, const int32_t* info, int64_t batch,
                               const int64_t* offsets, double* workspace, blastgpu_stream_t stream) {
    if (batch < 0) return -3;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (!desc) return -1;
    if (!offsets) return -4;
    if (!workspace) return -5;
    int64_t const groups = (batch + 31) / 32;
    if (groups > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    cudaStream_t const s = as_cuda(stream);
    DescGetrs const d{desc};
    getrs_interleave_kernel<<<(unsigned)groups, 256, 0, s>>>(d, batch, offsets, workspace);
    int st = check_launch();
    if (st != BLASTGPU_SUCCESS) return st;
    getrs_interleaved_kernel<<<(unsigned)groups, 32, 0, s>>>(d, batch, info, offsets, workspace);
    return check_launch();
}

int blastgpu_dgetrs_strided(int n, int nrhs, const double* LU, int lda, int64_t stride_a,
                            const int32_t* ipiv, int64_t stride_ipiv, double* X, int ldx,
                            int64_t stride_x, const int32_t* info, int64_t batch,
                            blastgpu_stream_t stream) {
    if (n < 0) return -1;
    if (nrhs < 0) return -2;
    if (n > 0 && !LU) return -3;
    if (lda < (n > 0 ? n : 1)) return -4;
    if (n > 0 && !ipiv) return -6;
    if (n > 0 && nrhs > 0 && !X) return -8;
    if (ldx < (n > 0 ? n : 1)) return -9;
    if (batch < 0) return -12;
    if (batch == 0 || n == 0 || nrhs == 0) return BLASTGPU_SUCCESS;
    StridedGetrs g{n, nrhs, lda, ldx, LU, stride_a, ipiv, stride_ipiv, X, stride_x};
    return launch_getrs(g, batch, info, as_cuda(stream));
}

int blastgpu_dgetrs_batched(const blastgpu_getrf_desc* desc, const int32_t* info, int64_t batch,
                            blastgpu_stream_t stream) {
    if (batch < 0) return -3;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (!desc) return -1;
    return launch_getrs(DescGetrs{desc}, batch, info, as_cuda(stream));
}

int blastgpu_dgesv_batched(const blastgpu_getrf_desc* desc, int32_t* info, int64_t batch,
                           int max_n, blastgpu_stream_t stream) {
    int st = blastgpu_dgetrf_batched(desc, info, batch, max_n, stream);
    if (st != BLASTGPU_SUCCESS) return st;
    return blastgpu_dgetrs_batched(desc, info, batch, stream);
}

}  // extern "C"

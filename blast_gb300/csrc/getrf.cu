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
//  * getrs: the forward half (laswp(b), unit-lower solve) one warp per matrix for n <= 256, lanes
//    over rows in a column sweep that keeps every row's ascending order; the backward half one
//    thread per matrix. The backward substitution is a chain of dependent dot products in BLAST's
//    order (each x_i starts from x_{i+1}); running it per thread keeps every lane busy while
//    preserving that order.
#include <math_constants.h>

#include <atomic>

#include "common.cuh"

namespace blastgpu {
namespace {

constexpr int kWarps = 4;  // matrices (warps) per CTA of the getrf kernel

template <typename T>
struct GetrfItemT {
    T* a;
    int m, n, lda;
    int32_t* ipiv;
};
using GetrfItem = GetrfItemT<double>;

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
template <typename T>
__device__ __forceinline__ int warp_iamax(const T* a, int lda, int r0, int r1, int j, int lane) {
    T best = (T)-1;
    int idx = 0x7fffffff;
    for (int r = r0 + lane; r < r1; r += 32) {
        T const v = fabs(a[r + (int64_t)j * lda]);
        if (v > best) { best = v; idx = r; }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        T const ob = __shfl_xor_sync(0xffffffffu, best, off);
        int const oi = __shfl_xor_sync(0xffffffffu, idx, off);
        if (ob > best || (ob == best && oi < idx)) { best = ob; idx = oi; }
    }
    T const first = a[r0 + (int64_t)j * lda];
    if (first != first || idx == 0x7fffffff) idx = r0;  // NaN first element, or all NaN
    return idx - r0;
}

// getf2 (dense/Getf2.hpp:52-77) on the m x n block at (r0, c0); swaps cover the block's columns.
// ipiv receives block-relative pivots. Returns the block-relative k+1 of a zero pivot, or 0.
template <typename T>
__device__ int warp_getf2(T* a, int lda, int r0, int c0, int m, int n, int32_t* ipiv, int lane) {
    for (int k = 0; k < m && k < n; ++k) {
        int const ip = warp_iamax(a, lda, r0 + k, r0 + m, c0 + k, lane) + k;
        if (lane == 0) ipiv[k] = ip;
        if (ip != k) {
            for (int j = lane; j < n; j += 32) {
                T* p = a + (int64_t)(c0 + j) * lda;
                T const t = p[r0 + k];
                p[r0 + k] = p[r0 + ip];
                p[r0 + ip] = t;
            }
        }
        __syncwarp();
        T const piv = a[(r0 + k) + (int64_t)(c0 + k) * lda];
        if (piv == (T)0) return k + 1;
        T* col = a + (int64_t)(c0 + k) * lda;
        for (int i = k + 1 + lane; i < m; i += 32) col[r0 + i] = col[r0 + i] / piv;
        __syncwarp();
        for (int j = k + 1; j < n; ++j) {
            T* cj = a + (int64_t)(c0 + j) * lda;
            T const y = cj[r0 + k];
            for (int i = k + 1 + lane; i < m; i += 32) cj[r0 + i] = fma(-col[r0 + i], y, cj[r0 + i]);
        }
        __syncwarp();
    }
    return 0;
}

// laswp on columns [c0, c1) with pivots ipiv[k0..k1) (dense/Laswp.hpp:37-43), lane per column.
template <typename T>
__device__ __forceinline__ void warp_laswp(T* a, int lda, int c0, int c1, int k0, int k1,
                                           const int32_t* ipiv, int lane) {
    for (int j = c0 + lane; j < c1; j += 32) {
        T* p = a + (int64_t)j * lda;
        for (int k = k0; k < k1; ++k) {
            int const q = ipiv[k];
            if (q != k) {
                T const t = p[k];
                p[k] = p[q];
                p[q] = t;
            }
        }
    }
}

template <typename T>
__device__ int warp_getrf(GetrfItemT<T> it, int lane) {
    constexpr int NB = 4;
    int const M = it.m, N = it.n, lda = it.lda;
    T* a = it.a;
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
            T* cj = a + (int64_t)j * lda;
            T x[NB];
#pragma unroll
            for (int i = 0; i < NB; ++i) {
                T acc = cj[k + i];
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
            T acc = (T)0;
#pragma unroll
            for (int q = 0; q < NB; ++q) acc = fma(a[i + (int64_t)(k + q) * lda], a[(k + q) + (int64_t)j * lda], acc);
            T* c = a + i + (int64_t)j * lda;
            *c = fma((T)1, *c, -acc);
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

template <typename T>
__device__ int cta_getrf(GetrfItemT<T> it, int* s_ret, T* sp) {
    constexpr int NB = 4;
    int const M = it.m, N = it.n, lda = it.lda;
    T* a = it.a;
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
            T* p = a + (int64_t)j * lda;
            for (int q = k; q < k + NB; ++q) {
                int const pr = ipiv[q];
                if (pr != q) {
                    T const t = p[q];
                    p[q] = p[pr];
                    p[pr] = t;
                }
            }
        }
        __syncthreads();
        // U12 := L11^{-1} A12, thread per column
        for (int j = k + NB + tid; j < N; j += kCtaThreads) {
            T* cj = a + (int64_t)j * lda;
            T x[NB];
#pragma unroll
            for (int i = 0; i < NB; ++i) {
                T acc = cj[k + i];
#pragma unroll
                for (int q = 0; q < i; ++q) acc = fma(-a[(k + i) + (int64_t)(k + q) * lda], x[q], acc);
                x[i] = acc;
                cj[k + i] = acc;
            }
        }
        __syncthreads();
        // A22 := A22 - A21 * U12, thread per row. Column j + 1's operands (U12, final in this
        // phase, and this thread's own element) are loaded before column j's store, which they
        // would otherwise wait behind (the compiler cannot tell the addresses apart).
        for (int i = k + NB + tid; i < M; i += kCtaThreads) {
            T l[NB];
#pragma unroll
            for (int q = 0; q < NB; ++q) l[q] = a[i + (int64_t)(k + q) * lda];
            int j = k + NB;
            T u[NB], cv = (T)0;
#pragma unroll
            for (int q = 0; q < NB; ++q) u[q] = (T)0;
            if (j < N) {
#pragma unroll
                for (int q = 0; q < NB; ++q) u[q] = a[k + q + (int64_t)j * lda];
                cv = a[i + (int64_t)j * lda];
            }
            for (; j < N; ++j) {
                T un[NB], cn = (T)0;
#pragma unroll
                for (int q = 0; q < NB; ++q) un[q] = (T)0;
                if (j + 1 < N) {
#pragma unroll
                    for (int q = 0; q < NB; ++q) un[q] = a[k + q + (int64_t)(j + 1) * lda];
                    cn = a[i + (int64_t)(j + 1) * lda];
                }
                T acc = (T)0;
#pragma unroll
                for (int q = 0; q < NB; ++q) acc = fma(l[q], u[q], acc);
                a[i + (int64_t)j * lda] = fma((T)1, cv, -acc);
#pragma unroll
                for (int q = 0; q < NB; ++q) u[q] = un[q];
                cv = cn;
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
        T* p = a + (int64_t)j * lda;
        for (int q = k; q < min(M, N); ++q) {
            int const pr = ipiv[q];
            if (pr != q) {
                T const t = p[q];
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

// Left-looking schedule of BLAST's blocked LU for square matrices (the CTA kernel's default for
// n <= 512). BLAST's getrf is right-looking: after each 4-column panel every later column takes its
// row swaps, its 4 rows of U (trsm with the unit-lower 4 x 4 block) and a rank-4 update of the rows
// below. Each element of a column sees these operations in step order, and a step only reads the
// column itself, the panel's L columns and the pivots. So a column may receive all its updates
// late, step after step, as long as L stays in the row order of its own step; the swaps that
// BLAST applies to the columns left of a later panel therefore wait until the end (they only move
// finished values). Every element then sees exactly BLAST's rounded operations, in BLAST's order,
// and factors and pivots are bit-identical to the right-looking kernels.
//
// Mapping: the matrix is processed in super-panels of 32 columns held in shared memory (n x 32
// doubles, leading dimension n | 1 so that a warp's column accesses spread over the banks). Warp
// w owns the super-panel's columns c with c % 8 == w. First each warp applies every earlier step
// to its own columns, all of them (up to 4) at once: swaps, the 4-row solve and the rank-4 update,
// lanes over rows, the L block of the step read from global memory once per row for all the
// warp's columns (all warps read the same rows, so L1 serves them); the columns are independent,
// so this phase has no barrier. Then the super-panel is factored with BLAST's
// inner steps: warp 0 runs getf2 on the 4-column panel in shared memory, and after a barrier every
// warp applies the step to its own columns right of the panel. The super-panel goes back to global
// memory, and at the end every column left of a step takes that step's swaps, in step order.
constexpr int kLazyCols = 32;

template <typename T>
__device__ __forceinline__ T sel4(T const (&v)[4], int q) {
    return q == 0 ? v[0] : q == 1 ? v[1] : q == 2 ? v[2] : v[3];
}

// Step k (columns k..k+3 of L, Lk[r + q * ldl] = L(r, k + q)) applied to nc <= 4 columns of the
// super-panel, c0 + j * cstride for j < nc, by one warp: the columns share the loads of L, and
// each column's operations are those of BLAST's step in BLAST's order.
template <typename T>
__device__ __forceinline__ void lazy_apply_step_cols(T* sp, int ld, int n, int k, int c0, int cstride, int nc,
                                                     const T* Lk, int ldl, const int32_t* ipiv, int lane) {
    // swaps of step k (rows k..k+3): lane j < nc swaps column j
    if (lane < nc) {
        T* col = sp + (int64_t)(c0 + lane * cstride) * ld;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            int const pr = ipiv[k + q];
            if (pr != k + q) {
                T const t = col[k + q];
                col[k + q] = col[pr];
                col[pr] = t;
            }
        }
    }
    __syncwarp();
    // rows k..k+3 of U (trsm<Lower, unit> with L(k:k+4, k:k+4)), every lane for every column
    T const l10 = Lk[(k + 1)], l20 = Lk[(k + 2)], l30 = Lk[(k + 3)];
    T const l21 = Lk[(k + 2) + (int64_t)ldl], l31 = Lk[(k + 3) + (int64_t)ldl];
    T const l32 = Lk[(k + 3) + 2 * (int64_t)ldl];
    T x[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (j < nc) {
            T const* col = sp + (int64_t)(c0 + j * cstride) * ld;
            x[j][0] = col[k];
            x[j][1] = fma(-l10, x[j][0], col[k + 1]);
            x[j][2] = fma(-l21, x[j][1], fma(-l20, x[j][0], col[k + 2]));
            x[j][3] = fma(-l32, x[j][2], fma(-l31, x[j][1], fma(-l30, x[j][0], col[k + 3])));
        } else {
            x[j][0] = x[j][1] = x[j][2] = x[j][3] = (T)0;
        }
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (j < nc && lane < 4) sp[(int64_t)(c0 + j * cstride) * ld + k + lane] = sel4(x[j], lane);
    // rank-4 update of the rows below, lanes over rows; the next row's L values are loaded before
    // this row's stores to the super-panel (which the loads could otherwise be held behind)
    int i = k + 4 + lane;
    T m0 = (T)0, m1 = (T)0, m2 = (T)0, m3 = (T)0;
    if (i < n) m0 = Lk[i], m1 = Lk[i + (int64_t)ldl], m2 = Lk[i + 2 * (int64_t)ldl], m3 = Lk[i + 3 * (int64_t)ldl];
    for (; i < n; i += 32) {
        int const in = i + 32;
        T p0 = (T)0, p1 = (T)0, p2 = (T)0, p3 = (T)0;
        if (in < n)
            p0 = Lk[in], p1 = Lk[in + (int64_t)ldl], p2 = Lk[in + 2 * (int64_t)ldl], p3 = Lk[in + 3 * (int64_t)ldl];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (j < nc) {
                T* col = sp + (int64_t)(c0 + j * cstride) * ld;
                T acc = (T)0;
                acc = fma(m0, x[j][0], acc);
                acc = fma(m1, x[j][1], acc);
                acc = fma(m2, x[j][2], acc);
                acc = fma(m3, x[j][3], acc);
                col[i] = fma((T)1, col[i], -acc);
            }
        }
        m0 = p0, m1 = p1, m2 = p2, m3 = p3;
    }
    __syncwarp();
}

template <typename T>
__device__ int cta_getrf_lazy(GetrfItemT<T> it, int* s_ret, T* sp) {
    constexpr int NB = 4;
    int const n = it.n, lda = it.lda, ld = n | 1;
    T* a = it.a;
    int32_t* ipiv = it.ipiv;
    int const tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int const nwarps = kCtaThreads / 32;
    int const kend = ((n - 1) / NB) * NB;  // first column of the unblocked remainder (BLAST: k + NB < n)
    for (int J = 0; J < n; J += kLazyCols) {
        int const w = min(kLazyCols, n - J);
        // the super-panel into shared memory
        for (int e = tid; e < w * n; e += kCtaThreads) {
            int const c = e / n, r = e - c * n;
            sp[(int64_t)c * ld + r] = a[r + (int64_t)(J + c) * lda];
        }
        __syncthreads();
        // every earlier step on this warp's columns warp, warp + 8, ... (no barrier: the columns
        // are independent)
        {
            int const nc = (w - warp + nwarps - 1) / nwarps;
            if (nc > 0)
                for (int k = 0; k < J; k += NB)
                    lazy_apply_step_cols(sp, ld, n, k, warp, nwarps, nc, a + (int64_t)k * lda, lda, ipiv, lane);
        }
        __syncthreads();
        // the super-panel's own steps
        for (int kk = J; kk < J + w; kk += NB) {
            int const kc = kk - J;
            bool const last = kk >= kend;  // the unblocked remainder: getf2 on all remaining columns
            if (warp == 0) {
                int const cols = last ? n - kk : NB;
                int const r = warp_getf2(sp, ld, kk, kc, n - kk, cols, ipiv + kk, lane);
                __syncwarp();
                for (int q = lane; q < cols && q < n - kk; q += 32) ipiv[kk + q] += kk;
                if (lane == 0) *s_ret = r ? kk + r : 0;
            }
            __syncthreads();
            if (*s_ret) return *s_ret;
            if (last) break;
            {
                int const c0 = kc + NB + warp;
                int const nc = c0 < w ? (w - c0 + nwarps - 1) / nwarps : 0;
                if (nc > 0) lazy_apply_step_cols(sp, ld, n, kk, c0, nwarps, nc, sp + (int64_t)kc * ld, ld, ipiv, lane);
            }
            __syncthreads();
        }
        // back to global memory
        for (int e = tid; e < w * n; e += kCtaThreads) {
            int const c = e / n, r = e - c * n;
            a[r + (int64_t)(J + c) * lda] = sp[(int64_t)c * ld + r];
        }
        __syncthreads();
    }
    // the swaps of every step on the columns left of it, in step order (BLAST's laswp of the
    // left columns at each step, and the final one after the remainder)
    for (int c = tid; c < n; c += kCtaThreads) {
        T* col = a + (int64_t)c * lda;
        for (int k = (c / NB + 1) * NB; k < n; ++k) {
            int const pr = ipiv[k];
            if (pr != k) {
                T const t = col[k];
                col[k] = col[pr];
                col[pr] = t;
            }
        }
    }
    __syncthreads();
    return 0;
}

// Square matrices with n <= kLazyMaxN (the super-panel's n x 32 doubles in shared memory).
constexpr int kLazyMaxN = 512;

template <class Batch>
__global__ void __launch_bounds__(kCtaThreads) getrf_cta_lazy_kernel(Batch batch, int64_t count, int32_t* info) {
    extern __shared__ double sp_dyn[];
    __shared__ int s_ret;
    int64_t const b = blockIdx.x;
    if (b >= count) return;
    GetrfItem const it = batch.get(b);
    int r;
    if (it.m == it.n && it.n <= kLazyMaxN) {
        r = cta_getrf_lazy(it, &s_ret, sp_dyn);
    } else {
        // rectangular or larger: the right-looking schedule (its panel buffer aliases the
        // dynamic shared memory, which holds at least 4 * kPanelRows doubles at every launch)
        r = cta_getrf(it, &s_ret, sp_dyn);
    }
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

// getrs, one thread per instance, in BLAST's scalar order (dense/Trsm.hpp:39-65): laswp(b) with
// ipiv[0..n), x_i = b_i - sum_{k<i} l_ik x_k (unit lower), x_i = (x_i - sum_{k>i} u_ik x_k) / u_ii,
// every sum in ascending k. The solution vector lives in shared memory (x[k * 32 + lane], max_n * 32
// doubles per warp). The forward solve runs four rows' chains side by side (each still in ascending
// k), so every x_k read serves four rows and a pass keeps 32 factor loads in flight; the backward
// chain is serial in BLAST's order (row i starts from x_{i+1}). Factor terms are loaded a pass
// ahead of the FMAs that use them (forward: 4 rows x 8 terms; backward: 16 terms along the row,
// the next row's first pass and diagonal included), so memory latency overlaps the chain. On
// GB300 a warp's DFMA occupies its sub-partition's binary64 pipe for 64 cycles, so the largest
// instances' n^2 chained FMAs bound the kernel. A short pass reads zeros past the row's end and
// skips their FMAs.
struct FactorView {
    const double* p;
    int64_t ld;
    __device__ __forceinline__ double operator()(int i, int k) const { return p[i + k * ld]; }
};

__device__ __forceinline__ void load_pass(FactorView const& A, int i, int k0, int k1, double (&av)[16]) {
#pragma unroll
    for (int u = 0; u < 16; ++u) av[u] = k0 + u < k1 ? A(i, k0 + u) : 0.0;
}

// The forward half of getrs with one warp per instance, for n <= 32 * MAXT: the row interchanges
// of b in ipiv order (lane 0, in shared memory), then y_i = b_i - sum_{l<i} l_il y_l as a column
// sweep with lanes over rows: once y_l is final its owner lane broadcasts it and every row below
// takes its term. Each row's sum still runs in ascending l with the same fused multiply-adds as the
// thread kernel's (and BLAST's) order, so y is the same bits; the rows advance together, and the
// factor's columns are read coalesced, four columns ahead of their use. y overwrites b; the
// backward half then runs one thread per instance (getrs_kernel with fwd = 0), whose chain is
// serial in BLAST's order.
// One pass of the backward substitution: row i, terms k0 .. k0+15 (row i's first pass starts at
// k0 = i + 1 and also loads the diagonal u_ii). Passes run bottom row first; i < 0 ends the
// sequence.
struct BwdPass {
    int i, k0;
    __device__ __forceinline__ BwdPass next(int n) const {
        if (i < 0) return *this;
        return k0 + 16 < n ? BwdPass{i, k0 + 16} : BwdPass{i - 1, i};
    }
    __device__ __forceinline__ void load(FactorView const& A, int n, double (&av)[16], double& d) const {
        load_pass(A, i, k0, n, av);
        if (k0 == i + 1) d = A(i, i);
    }
};

template <int MAXT>
struct FwdCols {
    double v[4][MAXT];
    __device__ __forceinline__ void load(FactorView const& A, int s, int l, int n, int lane) {
#pragma unroll
        for (int t = 0; t < MAXT; ++t) {
            int const i = lane + 32 * t;
            v[s][t] = (l < n && i > l && i < n) ? A(i, l) : 0.0;
        }
    }
};

template <int MAXT, class Batch>
__global__ void __launch_bounds__(kWarps * 32) getrs_fwd_warp_kernel(Batch batch, int64_t count, const int32_t* info) {
    __shared__ double ys[kWarps][32 * MAXT];
    int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t const b = (int64_t)blockIdx.x * kWarps + warp;
    if (b >= count) return;
    if (info && info[b] != 0) return;
    GetrsItem const it = batch.get(b);
    int const n = it.n;
    FactorView const A{it.a, it.lda};
    double* y = ys[warp];
    for (int j = 0; j < it.nrhs; ++j) {
        double* bj = it.x + (int64_t)j * it.ldx;
        __syncwarp();
        for (int k = lane; k < n; k += 32) y[k] = bj[k];
        __syncwarp();
        if (lane == 0) {
            for (int k = 0; k < n; ++k) {
                int const q = it.ipiv[k];
                if (q != k) {
                    double const t = y[k];
                    y[k] = y[q];
                    y[q] = t;
                }
            }
        }
        __syncwarp();
        double acc[MAXT];
#pragma unroll
        for (int t = 0; t < MAXT; ++t) acc[t] = lane + 32 * t < n ? y[lane + 32 * t] : 0.0;
        FwdCols<MAXT> c;
#pragma unroll
        for (int s = 0; s < 4; ++s) c.load(A, s, s, n, lane);
        for (int l0 = 0; l0 < n - 1; l0 += 4) {
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                int const l = l0 + s;
                if (l < n - 1) {
                    int const tl = l >> 5;
                    double own = 0.0;
#pragma unroll
                    for (int t = 0; t < MAXT; ++t)
                        if (t == tl) own = acc[t];
                    double const yl = __shfl_sync(0xffffffffu, own, l & 31);
#pragma unroll
                    for (int t = 0; t < MAXT; ++t) {
                        int const i = lane + 32 * t;
                        if (t >= tl && i > l && i < n) acc[t] = fma(-c.v[s][t], yl, acc[t]);
                    }
                }
                c.load(A, s, l + 4, n, lane);
            }
        }
#pragma unroll
        for (int t = 0; t < MAXT; ++t)
            if (lane + 32 * t < n) bj[lane + 32 * t] = acc[t];
    }
}

template <class Batch>
__global__ void __launch_bounds__(32) getrs_kernel(Batch batch, int64_t count, const int32_t* info, int fwd) {
    extern __shared__ double xs[];
    int const lane = threadIdx.x;
    int64_t const b = (int64_t)blockIdx.x * 32 + lane;
    if (b >= count) return;
    if (info && info[b] != 0) return;  // singular factor: BLAST would have thrown in getrf
    GetrsItem const it = batch.get(b);
    int const n = it.n;
    FactorView const A{it.a, it.lda};
    double* x = xs + lane;  // x[k * 32]
    for (int j = 0; j < it.nrhs; ++j) {
        const double* bj = it.x + (int64_t)j * it.ldx;
        for (int k = 0; k < n; ++k) x[k * 32] = bj[k];
        for (int k = 0; k < n && fwd; ++k) {
            int const q = it.ipiv[k];
            if (q != k) {
                double const t = x[k * 32];
                x[k * 32] = x[q * 32];
                x[q * 32] = t;
            }
        }
        for (int i0 = 0; i0 < n && fwd; i0 += 4) {
            double acc[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[r] = i0 + r < n ? x[(i0 + r) * 32] : 0.0;
            double av[4][8];
            auto load8 = [&](int k0, double (&dst)[4][8]) {
#pragma unroll
                for (int r = 0; r < 4; ++r)
#pragma unroll
                    for (int u = 0; u < 8; ++u) dst[r][u] = (i0 + r < n && k0 + u < i0) ? A(i0 + r, k0 + u) : 0.0;
            };
            if (i0 > 0) load8(0, av);
            for (int k0 = 0; k0 < i0; k0 += 8) {
                double an[4][8];
                if (k0 + 8 < i0) load8(k0 + 8, an);
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    if (k0 + u < i0) {
                        double const xk = x[(k0 + u) * 32];
#pragma unroll
                        for (int r = 0; r < 4; ++r) acc[r] = fma(-av[r][u], xk, acc[r]);
                    }
                }
#pragma unroll
                for (int r = 0; r < 4; ++r)
#pragma unroll
                    for (int u = 0; u < 8; ++u) av[r][u] = an[r][u];
            }
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                int const i = i0 + r;
                if (i < n) {
#pragma unroll
                    for (int q = 0; q < r; ++q) acc[r] = fma(-A(i, i0 + q), x[(i0 + q) * 32], acc[r]);
                    x[i * 32] = acc[r];
                }
            }
        }
        {
            // Passes of 16 terms along each row, bottom row first, with kSlots passes in flight:
            // the loop is unrolled over kSlots register slots, and a slot is reloaded with the pass
            // kSlots ahead right after its FMAs, so no load result is ever copied (a copy would
            // wait for it) and each load has kSlots - 1 passes of FMAs to arrive.
            constexpr int kSlots = 3;
            BwdPass p[kSlots];
            double a[kSlots][16], dg[kSlots];
            p[0] = BwdPass{n - 1, n};
#pragma unroll
            for (int s = 1; s < kSlots; ++s) p[s] = p[s - 1].next(n);
#pragma unroll
            for (int s = 0; s < kSlots; ++s) {
                dg[s] = 0.0;
                if (p[s].i >= 0) p[s].load(A, n, a[s], dg[s]);
            }
            BwdPass nxt = p[kSlots - 1].next(n);
            double acc = 0.0, drow = 0.0;
            bool done = false;
            while (!done) {
#pragma unroll
                for (int s = 0; s < kSlots; ++s) {
                    if (!done) {
                        BwdPass const cur = p[s];
                        if (cur.i < 0) {
                            done = true;
                        } else {
                            if (cur.k0 == cur.i + 1) {
                                acc = x[cur.i * 32];
                                drow = dg[s];
                            }
#pragma unroll
                            for (int u = 0; u < 16; ++u)
                                if (cur.k0 + u < n) acc = fma(-a[s][u], x[(cur.k0 + u) * 32], acc);
                            if (p[(s + 1) % kSlots].i != cur.i) x[cur.i * 32] = acc / drow;
                            p[s] = nxt;
                            if (nxt.i >= 0) nxt.load(A, n, a[s], dg[s]);
                            nxt = nxt.next(n);
                        }
                    }
                }
            }
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
    // "getrf.lazy" (default 0): the CTA kernel's left-looking schedule for square n <= 512. On the
    // ragged LU batch (20,000 x n log-uniform in [4, 256]) it took 42.4 ms per step against 33.9 ms
    // for the right-looking kernel, so the autotuner enables it per size bin only where it wins.
    bool const lazy = tune_get_bin("getrf.lazy", max_n, 0) != 0 && max_n <= kLazyMaxN;
    if (cta && lazy) {
        if (count > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
        size_t const rows = (size_t)(max_n | 1);
        size_t smem = sizeof(double) * rows * kLazyCols;
        if (smem < sizeof(double) * 4 * kPanelRows) smem = sizeof(double) * 4 * kPanelRows;
        cudaError_t const e = ensure_smem<getrf_cta_lazy_kernel<Batch>>(smem);
        if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
        getrf_cta_lazy_kernel<<<(unsigned)count, kCtaThreads, smem, s>>>(batch, count, info);
    } else if (cta) {
        if (count > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
        getrf_cta_kernel<<<(unsigned)count, kCtaThreads, 0, s>>>(batch, count, info);
    } else {
        int64_t const blocks = (count + kWarps - 1) / kWarps;
        if (blocks > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
        getrf_warp_kernel<<<(unsigned)blocks, kWarps * 32, 0, s>>>(batch, count, info);
    }
    return check_launch();
}

// max_n bounds every instance's n; the solution vectors of a warp's 32 instances take
// 32 * max_n doubles of shared memory (n up to 800).
template <class Batch>
int launch_getrs(Batch const& batch, int64_t count, int max_n, const int32_t* info, cudaStream_t s) {
    if (count == 0 || max_n == 0) return BLASTGPU_SUCCESS;
    int64_t const blocks = (count + 31) / 32;
    if (blocks > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    size_t const smem = sizeof(double) * 32 * (size_t)max_n;
    if (smem > 200 * 1024) return BLASTGPU_ERR_TOO_LARGE;
    if (smem > 48 * 1024) {
        cudaError_t const e = ensure_smem<getrs_kernel<Batch>>(200 * 1024);
        if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
    }
    // "getrs.warp_fwd" (default 1): the forward half one warp per instance for n <= 256, then
    // the backward half one thread per instance; 0: both halves one thread per instance.
    int const maxt = (max_n + 31) / 32;
    if (max_n <= 256 && tune_get("getrs.warp_fwd", 1) != 0) {
        int64_t const wblocks = (count + kWarps - 1) / kWarps;
        if (wblocks > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
        switch (maxt) {
            case 1: getrs_fwd_warp_kernel<1, Batch><<<(unsigned)wblocks, kWarps * 32, 0, s>>>(batch, count, info); break;
            case 2: getrs_fwd_warp_kernel<2, Batch><<<(unsigned)wblocks, kWarps * 32, 0, s>>>(batch, count, info); break;
            case 3:
            case 4: getrs_fwd_warp_kernel<4, Batch><<<(unsigned)wblocks, kWarps * 32, 0, s>>>(batch, count, info); break;
            default: getrs_fwd_warp_kernel<8, Batch><<<(unsigned)wblocks, kWarps * 32, 0, s>>>(batch, count, info); break;
        }
        getrs_kernel<Batch><<<(unsigned)blocks, 32, smem, s>>>(batch, count, info, 0);
    } else {
        getrs_kernel<Batch><<<(unsigned)blocks, 32, smem, s>>>(batch, count, info, 1);
    }
    return check_launch();
}

// ---------------------------------------------------------------------------------------------
// Mixed-precision LU solve (blastgpu_dgesv_mixed_batched): binary32 factor, binary64 refinement.

struct GesvMixedItems {
    const blastgpu_gesv_mixed_desc* desc;
    char* ws;
    __device__ GetrfItemT<float> get(int64_t b) const {
        blastgpu_gesv_mixed_desc const& d = desc[b];
        int const n = d.A.rows;
        return {reinterpret_cast<float*>(ws + d.ws_offset), n, n, n, d.ipiv};
    }
};

// A (binary64) rounded to binary32 into the instance's scratch (leading dimension n), one CTA of
// 256 threads per instance, consecutive threads on consecutive elements of a column.
__global__ void __launch_bounds__(kCtaThreads) gesv_mixed_round_kernel(GesvMixedItems items, int64_t count) {
    int64_t const b = blockIdx.x;
    if (b >= count) return;
    blastgpu_gesv_mixed_desc const& d = items.desc[b];
    int const n = d.A.rows, nn = n * n;
    float* f = reinterpret_cast<float*>(items.ws + d.ws_offset);
    for (int e = threadIdx.x; e < nn; e += kCtaThreads) {
        int const j = e / n, i = e - j * n;
        f[e] = (float)d.A.data[i + (int64_t)j * d.A.ld];
    }
}

__global__ void __launch_bounds__(kWarps * 32) getrf_warp_f32_kernel(GesvMixedItems items, int64_t count,
                                                                      int32_t* info) {
    int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t const b = (int64_t)blockIdx.x * kWarps + warp;
    if (b >= count) return;
    int const r = warp_getrf(items.get(b), lane);
    if (info && lane == 0) info[b] = r;
}

__global__ void __launch_bounds__(kCtaThreads) getrf_cta_f32_kernel(GesvMixedItems items, int64_t count,
                                                                    int32_t* info) {
    __shared__ int s_ret;
    __shared__ float s_panel[4 * kPanelRows];
    int64_t const b = blockIdx.x;
    if (b >= count) return;
    int const r = cta_getrf(items.get(b), &s_ret, s_panel);
    if (info && threadIdx.x == 0) info[b] = r;
}

// The left-looking schedule in binary32 (super-panels of 32 columns, n x 32 floats of dynamic
// shared memory): far less traffic to L2 than the right-looking kernel's read-modify-write of the
// trailing matrix at every step.
__global__ void __launch_bounds__(kCtaThreads) getrf_cta_lazy_f32_kernel(GesvMixedItems items, int64_t count,
                                                                         int32_t* info) {
    extern __shared__ float spf[];
    __shared__ int s_ret;
    int64_t const b = blockIdx.x;
    if (b >= count) return;
    int const r = cta_getrf_lazy(items.get(b), &s_ret, spf);
    if (info && threadIdx.x == 0) info[b] = r;
}

template <int MAXT>
__device__ __forceinline__ double warp_max_abs(double const (&v)[MAXT], int n, int lane) {
    double m = 0.0;
#pragma unroll
    for (int t = 0; t < MAXT; ++t) {
        double const a = fabs(v[t]);
        if (lane + 32 * t < n) m = (a > m || a != a) ? a : m;  // NaN-propagating
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        double const o = __shfl_xor_sync(0xffffffffu, m, off);
        m = (o > m || o != o) ? o : m;
    }
    return m;
}

// v := U^{-1} L^{-1} P v with the binary32 factor F (leading dimension n) of one instance, one warp,
// lanes over rows (row lane + 32 t in v[t]). perm[i] is the row of v that row i of P v takes
// (the pivots' interchanges composed), buf: n floats of shared memory. Both substitutions are
// column sweeps: once an entry is final its lane broadcasts it, and every remaining row takes its
// term. The sweeps run block by block of 32 steps with the block index a compile-time constant
// (the broadcast entry is v[TL], and the row blocks above or below need no test), and the factor's
// columns are read coalesced into four register slots, each reloaded with the column four steps
// ahead right after use.
template <int MAXT>
struct ColSlots {
    float v[4][MAXT];
    // rows i < n of column c, clamped into the matrix (a column outside it is never used)
    __device__ __forceinline__ void load(int s, const float* F, int n, int c, int lane) {
        int const cc = c < 0 ? 0 : (c >= n ? n - 1 : c);
#pragma unroll
        for (int t = 0; t < MAXT; ++t) {
            int const i = lane + 32 * t;
            v[s][t] = i < n ? F[i + (int64_t)cc * n] : 0.f;
        }
    }
};

template <int MAXT, int TL>
__device__ __forceinline__ void lu_fwd_block(float (&v)[MAXT], ColSlots<MAXT>& cs, const float* F, int n, int lane) {
    int const lend = min(n - 1, 32 * TL + 32);
    for (int l0 = 32 * TL; l0 < lend; l0 += 4) {
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            int const l = l0 + s;
            if (l < lend) {
                float const vl = __shfl_sync(0xffffffffu, v[TL], l & 31);
#pragma unroll
                for (int t = TL; t < MAXT; ++t)
                    if (t > TL || lane > (l & 31)) v[t] = fmaf(-cs.v[s][t], vl, v[t]);
            }
            cs.load(s, F, n, l + 4, lane);
        }
    }
}

template <int MAXT, int TL>
__device__ __forceinline__ void lu_bwd_block(float (&v)[MAXT], ColSlots<MAXT>& cs, const float* F, int n, int lane,
                                             int& l0) {
    // groups of 4 steps l = l0, l0-1, l0-2, l0-3 with l0 = 3 mod 4 (so that a group never straddles
    // a 32-step block), down to 32 TL; steps past n - 1 (the top group's) are left out
    int const lstop = 32 * TL;
    for (; l0 >= lstop; l0 -= 4) {
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            int const l = l0 - s;
            if (l < n) {
                if (lane == (l & 31)) v[TL] = v[TL] / cs.v[s][TL];
                float const xl = __shfl_sync(0xffffffffu, v[TL], l & 31);
#pragma unroll
                for (int t = 0; t <= TL; ++t)
                    if (t < TL || lane < (l & 31)) v[t] = fmaf(-cs.v[s][t], xl, v[t]);
            }
            cs.load(s, F, n, l - 4, lane);
        }
    }
}

template <int MAXT>
__device__ void warp_lu_solve_f32(float (&v)[MAXT], const float* F, int n, const int* perm, float* buf, int lane) {
#pragma unroll
    for (int t = 0; t < MAXT; ++t)
        if (lane + 32 * t < n) buf[lane + 32 * t] = v[t];
    __syncwarp();
#pragma unroll
    for (int t = 0; t < MAXT; ++t) v[t] = lane + 32 * t < n ? buf[perm[lane + 32 * t]] : 0.f;
    __syncwarp();
    ColSlots<MAXT> cs;
    // forward: unit lower; step l uses column l (rows below l take its term)
#pragma unroll
    for (int s = 0; s < 4; ++s) cs.load(s, F, n, s, lane);
    lu_fwd_block<MAXT, 0>(v, cs, F, n, lane);
    if constexpr (MAXT > 1) lu_fwd_block<MAXT, (MAXT > 1 ? 1 : 0)>(v, cs, F, n, lane);
    if constexpr (MAXT > 2) lu_fwd_block<MAXT, (MAXT > 2 ? 2 : 0)>(v, cs, F, n, lane);
    if constexpr (MAXT > 3) lu_fwd_block<MAXT, (MAXT > 3 ? 3 : 0)>(v, cs, F, n, lane);
    if constexpr (MAXT > 4) lu_fwd_block<MAXT, (MAXT > 4 ? 4 : 0)>(v, cs, F, n, lane);
    if constexpr (MAXT > 5) lu_fwd_block<MAXT, (MAXT > 5 ? 5 : 0)>(v, cs, F, n, lane);
    if constexpr (MAXT > 6) lu_fwd_block<MAXT, (MAXT > 6 ? 6 : 0)>(v, cs, F, n, lane);
    if constexpr (MAXT > 7) lu_fwd_block<MAXT, (MAXT > 7 ? 7 : 0)>(v, cs, F, n, lane);
    // backward: upper, dividing by the diagonal; step l uses column l (rows above l take its term)
    int l0 = ((n - 1) / 4) * 4 + 3;
#pragma unroll
    for (int s = 0; s < 4; ++s) cs.load(s, F, n, l0 - s, lane);
    if constexpr (MAXT > 7) lu_bwd_block<MAXT, (MAXT > 7 ? 7 : 0)>(v, cs, F, n, lane, l0);
    if constexpr (MAXT > 6) lu_bwd_block<MAXT, (MAXT > 6 ? 6 : 0)>(v, cs, F, n, lane, l0);
    if constexpr (MAXT > 5) lu_bwd_block<MAXT, (MAXT > 5 ? 5 : 0)>(v, cs, F, n, lane, l0);
    if constexpr (MAXT > 4) lu_bwd_block<MAXT, (MAXT > 4 ? 4 : 0)>(v, cs, F, n, lane, l0);
    if constexpr (MAXT > 3) lu_bwd_block<MAXT, (MAXT > 3 ? 3 : 0)>(v, cs, F, n, lane, l0);
    if constexpr (MAXT > 2) lu_bwd_block<MAXT, (MAXT > 2 ? 2 : 0)>(v, cs, F, n, lane, l0);
    if constexpr (MAXT > 1) lu_bwd_block<MAXT, (MAXT > 1 ? 1 : 0)>(v, cs, F, n, lane, l0);
    lu_bwd_block<MAXT, 0>(v, cs, F, n, lane, l0);
}

// Refinement, one warp per instance (n <= 32 MAXT): x0 from the binary32 factor, then r = b - A x
// in binary64 (A read by columns, coalesced; |A|_inf from the same pass the first time), the
// backward error, and corrections d = (U^{-1} L^{-1} P (r / |r|_inf)) |r|_inf until the error is at
// most tol or max_iter corrections are spent. X overwrites B at the end.
// One instance with n <= 32 MAXT (its own row-block count, so that blocks past its last row
// cost nothing); xs, buf, perm: n doubles, floats and ints of the warp's shared memory.
template <int MAXT>
__device__ void gesv_mixed_ir(GesvMixedItems const& items, int64_t b, double tol, int max_iter, const int32_t* info,
                              int32_t* iters, double* berr, double* xs, float* buf, int* perm, int lane) {
    // the descriptor's fields, read once
    blastgpu_gesv_mixed_desc const& d = items.desc[b];
    int const n = d.A.rows, nrhs = d.B.cols, lda = d.A.ld, ldb = d.B.ld;
    const double* const A = d.A.data;
    double* const B = d.B.data;
    const int32_t* const ipiv = d.ipiv;
    const float* F = reinterpret_cast<const float*>(items.ws + d.ws_offset);
    if (info && info[b] != 0) {  // a zero binary32 pivot: no factor to refine with
        for (int c = 0; c < nrhs; ++c)
            for (int i = lane; i < n; i += 32) B[i + (int64_t)c * ldb] = CUDART_NAN;
        if (lane == 0) {
            if (iters) iters[b] = 0;
            if (berr) berr[b] = CUDART_NAN;
        }
        return;
    }
    // P as a permutation: the pivots' interchanges applied in order to the identity
    for (int i = lane; i < n; i += 32) perm[i] = i;
    __syncwarp();
    if (lane == 0) {
        for (int k = 0; k < n; ++k) {
            int const q = ipiv[k];
            if (q != k) {
                int const t = perm[k];
                perm[k] = perm[q];
                perm[q] = t;
            }
        }
    }
    __syncwarp();
    double anorm = -1.0, worst = 0.0;
    int total_iters = 0;
    for (int c = 0; c < nrhs; ++c) {
        double* bc = B + (int64_t)c * ldb;
        double bv[MAXT], x[MAXT], r[MAXT];
#pragma unroll
        for (int t = 0; t < MAXT; ++t) bv[t] = lane + 32 * t < n ? bc[lane + 32 * t] : 0.0;
        double const bnorm = warp_max_abs<MAXT>(bv, n, lane);
        float w[MAXT];
#pragma unroll
        for (int t = 0; t < MAXT; ++t) w[t] = (float)bv[t];
        warp_lu_solve_f32<MAXT>(w, F, n, perm, buf, lane);
#pragma unroll
        for (int t = 0; t < MAXT; ++t) x[t] = (double)w[t];
        double be = CUDART_NAN;
        int it = 0;
        while (true) {
            // r = b - A x
#pragma unroll
            for (int t = 0; t < MAXT; ++t)
                if (lane + 32 * t < n) xs[lane + 32 * t] = x[t];
            __syncwarp();
            double rs[MAXT];
#pragma unroll
            for (int t = 0; t < MAXT; ++t) {
                r[t] = bv[t];
                rs[t] = 0.0;
            }
            bool const first = anorm < 0.0;
            // columns of A in four register slots, each reloaded with the column four ahead
            double acol[4][MAXT];
            auto load_col = [&](int s, int j) {
#pragma unroll
                for (int t = 0; t < MAXT; ++t)
                    acol[s][t] = (j < n && lane + 32 * t < n) ? A[lane + 32 * t + (int64_t)j * lda] : 0.0;
            };
#pragma unroll
            for (int s = 0; s < 4; ++s) load_col(s, s);
            for (int j0 = 0; j0 < n; j0 += 4) {
#pragma unroll
                for (int s = 0; s < 4; ++s) {
                    int const j = j0 + s;
                    if (j < n) {
                        double const xj = xs[j];
#pragma unroll
                        for (int t = 0; t < MAXT; ++t) {
                            r[t] = fma(-acol[s][t], xj, r[t]);
                            if (first) rs[t] += fabs(acol[s][t]);
                        }
                    }
                    load_col(s, j + 4);
                }
            }
            __syncwarp();
            if (first) anorm = warp_max_abs<MAXT>(rs, n, lane);
            double const rm = warp_max_abs<MAXT>(r, n, lane);
            double const xm = warp_max_abs<MAXT>(x, n, lane);
            double const den = anorm * xm + bnorm;
            be = den > 0.0 ? rm / den : (rm == 0.0 ? 0.0 : CUDART_INF);
            if (!(be > tol) || it >= max_iter) break;
#pragma unroll
            for (int t = 0; t < MAXT; ++t) w[t] = (float)(r[t] / rm);
            warp_lu_solve_f32<MAXT>(w, F, n, perm, buf, lane);
#pragma unroll
            for (int t = 0; t < MAXT; ++t) x[t] += (double)w[t] * rm;
            ++it;
        }
#pragma unroll
        for (int t = 0; t < MAXT; ++t)
            if (lane + 32 * t < n) bc[lane + 32 * t] = x[t];
        total_iters = max(total_iters, it);
        worst = (be > worst || be != be) ? be : worst;
    }
    if (lane == 0) {
        if (iters) iters[b] = total_iters;
        if (berr) berr[b] = worst;
    }
}

template <int MAXT>
__global__ void __launch_bounds__(kWarps * 32) gesv_mixed_ir_kernel(GesvMixedItems items, int64_t count, double tol,
                                                                   int max_iter, const int32_t* info, int32_t* iters,
                                                                   double* berr) {
    __shared__ double xs_all[kWarps][32 * MAXT];
    __shared__ float buf_all[kWarps][32 * MAXT];
    __shared__ int perm_all[kWarps][32 * MAXT];
    int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t const b = (int64_t)blockIdx.x * kWarps + warp;
    if (b >= count) return;
    int const n = items.desc[b].A.rows;
    if (n > 32 * MAXT) return;  // the launch's max_n bounds every instance
    double* xs = xs_all[warp];
    float* buf = buf_all[warp];
    int* perm = perm_all[warp];
    switch ((n + 31) >> 5) {
        case 0:
        case 1: gesv_mixed_ir<1>(items, b, tol, max_iter, info, iters, berr, xs, buf, perm, lane); break;
        case 2:
            if constexpr (MAXT >= 2) gesv_mixed_ir<(MAXT >= 2 ? 2 : 1)>(items, b, tol, max_iter, info, iters, berr, xs, buf, perm, lane);
            break;
        case 3:
        case 4:
            if constexpr (MAXT >= 4) gesv_mixed_ir<(MAXT >= 4 ? 4 : 1)>(items, b, tol, max_iter, info, iters, berr, xs, buf, perm, lane);
            break;
        case 5:
        case 6:
            if constexpr (MAXT >= 8) gesv_mixed_ir<(MAXT >= 8 ? 6 : 1)>(items, b, tol, max_iter, info, iters, berr, xs, buf, perm, lane);
            break;
        default:
            if constexpr (MAXT >= 8) gesv_mixed_ir<(MAXT >= 8 ? 8 : 1)>(items, b, tol, max_iter, info, iters, berr, xs, buf, perm, lane);
            break;
    }
}

int launch_gesv_mixed(GesvMixedItems items, int64_t count, int max_n, double tol, int max_iter, int32_t* info,
                      int32_t* iters, double* berr, cudaStream_t s) {
    if (count == 0) return BLASTGPU_SUCCESS;
    int64_t const wblocks = (count + kWarps - 1) / kWarps;
    if (wblocks > 0x7fffffff || count > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    unsigned const wg = (unsigned)wblocks;
    gesv_mixed_round_kernel<<<(unsigned)count, kCtaThreads, 0, s>>>(items, count);
    // n > 64: the CTA kernel, left-looking ("gesv_mixed.lazy" = 1, default) or right-looking
    if (max_n > 64 && tune_get_bin("gesv_mixed.lazy", max_n, 1) != 0) {
        size_t const smem = sizeof(float) * (size_t)(max_n | 1) * kLazyCols;
        cudaError_t const e = ensure_smem<getrf_cta_lazy_f32_kernel>(smem);
        if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
        getrf_cta_lazy_f32_kernel<<<(unsigned)count, kCtaThreads, smem, s>>>(items, count, info);
    } else if (max_n > 64) {
        getrf_cta_f32_kernel<<<(unsigned)count, kCtaThreads, 0, s>>>(items, count, info);
    } else {
        getrf_warp_f32_kernel<<<wg, kWarps * 32, 0, s>>>(items, count, info);
    }
    int const maxt = (max_n + 31) / 32;
    if (maxt <= 1) gesv_mixed_ir_kernel<1><<<wg, kWarps * 32, 0, s>>>(items, count, tol, max_iter, info, iters, berr);
    else if (maxt <= 2) gesv_mixed_ir_kernel<2><<<wg, kWarps * 32, 0, s>>>(items, count, tol, max_iter, info, iters, berr);
    else if (maxt <= 4) gesv_mixed_ir_kernel<4><<<wg, kWarps * 32, 0, s>>>(items, count, tol, max_iter, info, iters, berr);
    else gesv_mixed_ir_kernel<8><<<wg, kWarps * 32, 0, s>>>(items, count, tol, max_iter, info, iters, berr);
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
    return launch_getrs(g, batch, n, info, as_cuda(stream));
}

int blastgpu_dgetrs_batched(const blastgpu_getrf_desc* desc, const int32_t* info, int64_t batch, int max_n,
                            blastgpu_stream_t stream) {
    if (batch < 0) return -3;
    if (max_n < 0) return -4;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (!desc) return -1;
    return launch_getrs(DescGetrs{desc}, batch, max_n, info, as_cuda(stream));
}

int blastgpu_dgesv_batched(const blastgpu_getrf_desc* desc, int32_t* info, int64_t batch,
                           int max_n, blastgpu_stream_t stream) {
    int st = blastgpu_dgetrf_batched(desc, info, batch, max_n, stream);
    if (st != BLASTGPU_SUCCESS) return st;
    return blastgpu_dgetrs_batched(desc, info, batch, max_n, stream);
}

size_t blastgpu_dgesv_mixed_workspace_bytes(int n) {
    if (n <= 0) return 0;
    return (((size_t)n * n * sizeof(float)) + 255) / 256 * 256;
}

int blastgpu_dgesv_mixed_batched(const blastgpu_gesv_mixed_desc* desc, int64_t batch, int max_n, void* workspace,
                                 double tol, int max_iter, int32_t* info, int32_t* iters, double* berr,
                                 blastgpu_stream_t stream) {
    if (batch < 0) return -2;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (!desc) return -1;
    if (max_n < 0) return -3;
    if (max_n > 256) return BLASTGPU_ERR_TOO_LARGE;
    if (!workspace) return -4;
    if (!(tol >= 0.0)) return -5;
    if (max_iter < 0) return -6;
    if (!info) return -7;  // the refinement reads the factorisation's info
    return launch_gesv_mixed(GesvMixedItems{desc, static_cast<char*>(workspace)}, batch, max_n, tol, max_iter,
                             info, iters, berr, as_cuda(stream));
}

}  // extern "C"

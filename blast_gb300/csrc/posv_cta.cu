// Ragged batched Cholesky solve for medium sizes (one CTA per matrix), binary64 and
// mixed precision (binary32 factorisation + binary64 iterative refinement), sm_103a.
//
// Reference: blast::potrf (dense/Potrf.hpp:66-106) is left-looking: each column strip is first
// updated with all previous columns (the ger(-1, ...) loop, a gemm), then factored on the
// diagonal and solved below it (RegisterMatrix::potrf / ::trsm). The solves are BLAST's trsm
// (dense/Trsm.hpp:17-66). BLAST has no mixed precision and no refinement; that part is new.
//
// GPU mapping: one CTA of 256 threads (8 warps) per matrix, the whole solve in one launch.
//  * Factorisation, left-looking with panels of 32 columns. Warp w owns panel columns
//    4w..4w+3, lane l owns rows l, l+32, ..., so each thread keeps an MAXR x 4 register tile
//    (BLAST's RegisterMatrix, 32 times wider). The update of a panel with all previous columns
//    streams those columns through shared memory with cp.async, 16 at a time and double-buffered
//    (the next 16 are in flight while the current ones are applied); every thread performs RA*4
//    fused multiply-adds per column (RA = 32-row blocks still below the diagonal, fixed at
//    compile time per panel) with operands read conflict-free from shared memory (rows:
//    consecutive lanes; panel columns: a warp-uniform broadcast).
//  * The 32 x 32 diagonal block is factored in place in shared memory: binary64 column at a time
//    by all threads with warp 0 finishing each pivot column, binary32 in sub-panels of 8 columns
//    factored by warp 0 in registers. The rows below are then solved against it (one thread per
//    row), and the panel is written to the factor.
//  * Forward and backward substitution run blockwise with look-ahead: once a 32-row block is
//    solved, warp 0 applies it to the next block and solves that block's triangle from registers
//    with shuffles while the other warps apply it to everything beyond; one barrier per block.
//  * Mixed precision: the factor is binary32 (in the caller's workspace); the residual
//    r = b - A*x is computed in binary64 from A's lower triangle, the correction solve uses the
//    binary32 factor on the scaled residual, and each matrix iterates until its normwise
//    backward error |r|_inf / (|A|_inf |x|_inf + |b|_inf) reaches the tolerance.
// On GB300 binary32 FMAs issue ~58x faster than binary64 (70 vs 1.2 TFLOP/s measured), which is
// what the mixed path turns into matrices per second.
#include <math_constants.h>

#include <atomic>
#include <mutex>
#include <type_traits>

#include "common.cuh"

namespace blastgpu {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kNB = 32;  // panel width = 4 columns per warp
constexpr int kKC = 32;  // previous columns staged at once by the panel update, as two chunks of 16
                         // (= panel width, so the staging buffer fits in the panel buffer's space)

struct CtaItem {
    int n;
    const double* A; int lda;
    double* L; int ldl;       // binary64 factor output (plain path) or nullptr
    const double* B; int ldb;
    double* X; int ldx;
    int nrhs;
    char* ws;                 // per-instance workspace (mixed path)
};

// Uniform batch: instance b at base + b * stride (A = nullptr: solves only, with the given L).
struct StridedPosv {
    int n, nrhs;
    const double* A; int lda; int64_t sa;
    double* L; int ldl; int64_t sl;
    const double* B; int ldb; int64_t sb;
    double* X; int ldx; int64_t sx;
    __device__ CtaItem get(int64_t b) const {
        return {n, A ? A + b * sa : nullptr, lda, L + b * sl, ldl, nrhs ? B + b * sb : nullptr, ldb,
                nrhs ? X + b * sx : nullptr, ldx, nrhs, nullptr};
    }
};

// capacity > 0: the workspace is a fixed array of that many bytes (the allocation-free entry
// point); an instance whose scratch range [ws_offset, ws_offset + n*n*4) is not inside it, or whose
// offset is not 4-byte aligned, comes back with n = -1 and is not solved.
struct DescPosv {
    const blastgpu_posv_desc* desc;
    char* workspace;
    int64_t capacity = 0;
    __device__ CtaItem get(int64_t b) const {
        blastgpu_posv_desc const& d = desc[b];
        int n = d.A.rows;
        if (capacity > 0) {
            int64_t const need = (int64_t)sizeof(float) * n * n;
            if (d.ws_offset < 0 || (d.ws_offset & 3) != 0 || d.ws_offset > capacity - need) n = -1;
        }
        return {n, d.A.data, d.A.ld, d.L.data, d.L.ld, d.B.data, d.B.ld,
                d.X.data, d.X.ld, d.B.cols, workspace && n >= 0 ? workspace + d.ws_offset : nullptr};
    }
};

// Asynchronous global -> shared copies (cp.async, completed by cp.async.wait_group + a barrier):
// every thread issues all of its copies back to back instead of waiting for each load.
__device__ __forceinline__ void cp_async(float* dst, const float* src) {
    unsigned const d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async(double* dst, const double* src) {
    unsigned const d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}

template <typename T>
__device__ __forceinline__ T rsqrt_t(T s);
template <>
__device__ __forceinline__ double rsqrt_t<double>(double s) { return rsqrt_nr(s); }
template <>
__device__ __forceinline__ float rsqrt_t<float>(float s) { return 1.0f / sqrtf(s); }

template <typename T>
__device__ __forceinline__ T rcp_t(T s);
template <>
__device__ __forceinline__ double rcp_t<double>(double s) { return rcp_nr(s); }
template <>
__device__ __forceinline__ float rcp_t<float>(float s) { return 1.0f / s; }

// Shared-memory layout (T = factor precision):
//   union { stage[kKC][NMAX] (panel update) ; panel[kNB][NMAX] (diag + trsm) }
//   vecs: 4 * NMAX doubles (b/x, r, work) + reductions
template <typename T, int MAXR>
struct Smem {
    static constexpr int NMAX = 32 * MAXR;
    static constexpr int kPanelElems = kNB * NMAX;
    static constexpr int kStageElems = kKC * NMAX;
    static constexpr int kBufElems = kPanelElems > kStageElems ? kPanelElems : kStageElems;
    static constexpr size_t kBytes =
        sizeof(T) * kBufElems + sizeof(double) * (4 * NMAX + 64);
};

// Update of the panel's register tiles with all previous columns: acc -= F(k0:n, kk) * F(k0+c, kk)
// for kk < k0, the columns streamed through shared memory in chunks of kKC / 2, double-buffered:
// the next chunk's asynchronous copies are in flight while the current chunk is applied. RA = row
// blocks still below the diagonal (ceil(m / 32)), fixed at compile time so that the inner loop is
// RA x 4 fused multiply-adds with no per-row guards. Rows past m and columns past nb pick up
// stale shared-memory values; they are never stored.
template <typename T, int MAXR>
__device__ __forceinline__ void panel_stage(const T* F, int ldf, T* buf, int k0, int m, int ch) {
    constexpr int NMAX = 32 * MAXR, KH = kKC / 2;
    int const kk = ch * KH, kc = min(KH, k0 - kk);
    T* dst = buf + (ch & 1) * KH * NMAX;
    for (int q = 0; q < kc; ++q) {
        T const* src = F + k0 + (int64_t)(kk + q) * ldf;
        for (int r = threadIdx.x; r < m; r += kThreads) cp_async(dst + q * NMAX + r, src + r);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

template <typename T, int RA, int MAXR>
__device__ __forceinline__ void panel_update(T (&acc)[MAXR][4], const T* F, int ldf, T* buf, int k0, int m,
                                             int c0) {
    constexpr int NMAX = 32 * MAXR, KH = kKC / 2;
    int const lane = threadIdx.x & 31;
    int const nch = (k0 + KH - 1) / KH;
    if (nch == 0) return;
    __syncthreads();  // the buffer's earlier contents are no longer read
    panel_stage<T, MAXR>(F, ldf, buf, k0, m, 0);
    for (int ch = 0; ch < nch; ++ch) {
        if (ch + 1 < nch) {
            panel_stage<T, MAXR>(F, ldf, buf, k0, m, ch + 1);  // into the half chunk ch - 1 used
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        }
        __syncthreads();
        int const kc = min(KH, k0 - ch * KH);
        T const* base = buf + (ch & 1) * KH * NMAX;
#pragma unroll 2
        for (int q = 0; q < kc; ++q) {
            T const* col = base + q * NMAX;
            T b[4];
            // the warp's 4 panel columns in one (binary32) or two (binary64) 16-byte broadcast
            // loads: NMAX and c0 are multiples of 4 elements and the buffer is 16-byte aligned
            if constexpr (sizeof(T) == 4) {
                float4 const v = *reinterpret_cast<float4 const*>(col + c0);
                b[0] = v.x, b[1] = v.y, b[2] = v.z, b[3] = v.w;
            } else {
                double2 const v0 = *reinterpret_cast<double2 const*>(col + c0);
                double2 const v1 = *reinterpret_cast<double2 const*>(col + c0 + 2);
                b[0] = v0.x, b[1] = v0.y, b[2] = v1.x, b[3] = v1.y;
            }
#pragma unroll
            for (int i = 0; i < RA; ++i) {
                T const a = col[lane + 32 * i];
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(-a, b[j], acc[i][j]);
            }
        }
        __syncthreads();  // every thread is done with this half before chunk ch + 2 is staged into it
    }
}

template <typename T, int MAXR>
__device__ __forceinline__ void panel_update_dispatch(T (&acc)[MAXR][4], const T* F, int ldf, T* buf, int k0,
                                                      int m, int c0) {
    switch ((m + 31) / 32) {
#define BLASTGPU_PANEL_CASE(R) \
    case R:                    \
        if constexpr (R <= MAXR) panel_update<T, R, MAXR>(acc, F, ldf, buf, k0, m, c0); \
        break;
        BLASTGPU_PANEL_CASE(1) BLASTGPU_PANEL_CASE(2) BLASTGPU_PANEL_CASE(3) BLASTGPU_PANEL_CASE(4)
        BLASTGPU_PANEL_CASE(5) BLASTGPU_PANEL_CASE(6) BLASTGPU_PANEL_CASE(7) BLASTGPU_PANEL_CASE(8)
        BLASTGPU_PANEL_CASE(9) BLASTGPU_PANEL_CASE(10) BLASTGPU_PANEL_CASE(11) BLASTGPU_PANEL_CASE(12)
        BLASTGPU_PANEL_CASE(13) BLASTGPU_PANEL_CASE(14) BLASTGPU_PANEL_CASE(15) BLASTGPU_PANEL_CASE(16)
#undef BLASTGPU_PANEL_CASE
        default: break;
    }
}

// Cholesky of the nb x nb diagonal block held in shared memory (column j at blk + j * NMAX),
// column at a time, all threads (used for binary64, where warp 0's dependent reciprocal square
// roots cost 64 cycles per step and the sub-panel version below is slower). Column j is final
// (scaled) before step j: step j updates the trailing block a_il = fma(-l_ij, l_lj, a_il) (warp w:
// columns l = j+1+w, j+1+w+8, ...; lane: row l + lane), and warp 0, which owns column j+1,
// finishes it in the same step: the new pivot
// d = a_{j+1,j+1} comes from lane 0 by a shuffle, y = 1/sqrt(d), and the column is stored as
// a_{i,j+1} * y. Every element is then a single fused multiply-add per step, the reciprocal
// square root is taken by one warp, and there is one barrier per column. The products equal
// RegisterMatrix::potrf's (the pivot column scaled by 1/sqrt(d) once, then used unrounded).
// rinv[j] = 1/l_jj. Records the first bad pivot (k0 + j + 1) in *s_info.
template <typename T, int NMAX>
__device__ __forceinline__ void cta_chol_block_cols(T* blk, int nb, int k0, T* rinv, int* s_info) {
    int const tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (warp == 0) {
        T const v = lane < nb ? blk[lane] : (T)0;
        T const d = __shfl_sync(0xffffffffu, v, 0);
        T const y = rsqrt_t<T>(d);
        if (lane == 0) {
            if (!(d > (T)0) && *s_info == 0) *s_info = k0 + 1;
            rinv[0] = y;
        }
        if (lane < nb) blk[lane] = v * y;
    }
    __syncthreads();
    for (int j = 0; j + 1 < nb; ++j) {
        T const* cj = blk + j * NMAX;
        for (int l = j + 1 + warp; l < nb; l += kWarps) {
            int const i = l + lane;
            T const v = i < nb ? fma(-cj[i], cj[l], blk[l * NMAX + i]) : (T)0;
            if (l == j + 1) {  // warp 0: the next pivot column
                T const d = __shfl_sync(0xffffffffu, v, 0);
                T const y = rsqrt_t<T>(d);
                if (lane == 0) {
                    if (!(d > (T)0) && *s_info == 0) *s_info = k0 + j + 2;
                    rinv[j + 1] = y;
                }
                if (i < nb) blk[l * NMAX + i] = v * y;
            } else if (i < nb) {
                blk[l * NMAX + i] = v;
            }
        }
        __syncthreads();
    }
}

// Cholesky of the nb x nb diagonal block held in shared memory (column j at blk + j * NMAX),
// right-looking in sub-panels of 8 columns. Warp 0 (lane = row of the block) factors a sub-panel
// in registers: pivot d from the owning lane by a shuffle, y = 1/sqrt(d), l_jj = d*y, l_ij = a_ij*y,
// then the sub-panel's later columns take fma(-l_ij, l_lj, .) with l_lj shuffled from lane l. All
// threads then apply the 8 columns to the rest of the block, element by element in column order.
// Every element sees the same fused multiply-adds in the same order as the column-at-a-time
// version above (RegisterMatrix::potrf's products), with 2 barriers per 8 columns; binary32 only.
// rinv[j] = 1/l_jj. Records the first bad pivot (k0 + j + 1) in *s_info.
template <typename T, int NMAX>
__device__ __forceinline__ void cta_chol_block(T* blk, int nb, int k0, T* rinv, int* s_info) {
    if constexpr (sizeof(T) == 8) {
        cta_chol_block_cols<T, NMAX>(blk, nb, k0, rinv, s_info);
        return;
    }
    int const tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int s0 = 0; s0 < nb; s0 += 8) {
        int const ns = min(8, nb - s0);
        if (warp == 0) {
            int const i = lane;  // row of the block
            T v[8];
#pragma unroll
            for (int c = 0; c < 8; ++c) v[c] = (c < ns && i >= s0 + c && i < nb) ? blk[(s0 + c) * NMAX + i] : (T)0;
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                if (c < ns) {  // warp-uniform
                    int const j = s0 + c;
                    T const d = __shfl_sync(0xffffffffu, v[c], j);
                    T const y = rsqrt_t<T>(d);
                    if (lane == 0) {
                        if (!(d > (T)0) && *s_info == 0) *s_info = k0 + j + 1;
                        rinv[j] = y;
                    }
                    if (i == j) v[c] = d * y;
                    else if (i > j) v[c] *= y;
#pragma unroll
                    for (int c2 = c + 1; c2 < 8; ++c2) {
                        T const llj = __shfl_sync(0xffffffffu, v[c], s0 + c2);
                        if (c2 < ns && i >= s0 + c2) v[c2] = fma(-v[c], llj, v[c2]);
                    }
                }
            }
#pragma unroll
            for (int c = 0; c < 8; ++c)
                if (c < ns && i >= s0 + c && i < nb) blk[(s0 + c) * NMAX + i] = v[c];
        }
        __syncthreads();
        // the block's columns l >= s0 + 8 take the sub-panel: a_il -= sum_c l_i,s0+c * l_l,s0+c
        int const l0 = s0 + 8;
        if (l0 < nb) {
            int const w = nb - l0;  // columns l0 .. nb-1; element (i, l), i >= l
            for (int e = tid; e < w * 32; e += kThreads) {
                int const l = l0 + e / 32, i = l + (e & 31);
                if (i < nb) {
                    T acc = blk[l * NMAX + i];
#pragma unroll
                    for (int c = 0; c < 8; ++c) acc = fma(-blk[(s0 + c) * NMAX + i], blk[(s0 + c) * NMAX + l], acc);
                    blk[l * NMAX + i] = acc;
                }
            }
        }
        __syncthreads();
    }
}

// The second half of one panel step, shared by every factorisation below: the panel (rows
// k0 .. n-1, nb columns) is in shared memory at buf (column c at buf + c * NMAX), already updated
// with all previous columns. Factors its nb x nb diagonal block, solves the rows below against
// it, and writes the panel to F. With blk64 (binary32 factor only), the diagonal block is factored
// in binary64: widened into blk64 (32 x 32 doubles), factored column at a time, and rounded back.
template <typename T, int NMAX>
__device__ __forceinline__ void cta_panel_finish(T* buf, int nb, int m, int k0, T* F, int ldf, T* rinv,
                                                 int* s_info, double* blk64 = nullptr) {
    int const tid = threadIdx.x;
    if (blk64 != nullptr) {
        double* rinv64 = blk64 + 32 * 32;
        for (int e = tid; e < 32 * 32; e += kThreads) {
            int const c = e >> 5, r = e & 31;
            blk64[e] = (r < nb && c < nb && r >= c) ? (double)buf[c * NMAX + r] : 0.0;
        }
        __syncthreads();
        cta_chol_block_cols<double, 32>(blk64, nb, k0, rinv64, s_info);
        for (int e = tid; e < 32 * 32; e += kThreads) {
            int const c = e >> 5, r = e & 31;
            if (r < nb && c < nb && r >= c) buf[c * NMAX + r] = (T)blk64[e];
        }
        if (tid < nb) rinv[tid] = (T)rinv64[tid];
        __syncthreads();
    } else {
        // Diagonal block (nb x nb), all threads, in shared memory.
        cta_chol_block<T, NMAX>(buf, nb, k0, rinv, s_info);
    }
    // Rows below the block: x_j = (p_j - sum_{q<j} x_q l_jq) / l_jj, one thread per row, the
    // row in registers and the block's entries broadcast from shared memory.
    for (int r = nb + tid; r < m; r += kThreads) {
        T x[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            if (j < nb) {
                T v = buf[j * NMAX + r];
#pragma unroll
                for (int q = 0; q < j; ++q) v = fma(-x[q], buf[q * NMAX + j], v);
                x[j] = v * rinv[j];
                buf[j * NMAX + r] = x[j];
            }
        }
    }
    __syncthreads();
    // Panel to the factor (lower part), four columns per pass with their shared-memory loads
    // issued before the stores.
    for (int cb = 0; cb < nb; cb += 4) {
        for (int r = cb + tid; r < m; r += kThreads) {
            T v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) v[u] = (cb + u < nb && r >= cb + u) ? buf[(cb + u) * NMAX + r] : (T)0;
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (cb + u < nb && r >= cb + u) F[(k0 + r) + (int64_t)(k0 + cb + u) * ldf] = v[u];
        }
    }
    __syncthreads();
}

// Left-looking blocked Cholesky of the n x n matrix: lower(A) -> F (precision T, ld ldf).
// Returns info (0 or first bad pivot + 1) identically in all threads. With rowsum (n doubles in
// shared memory, zeroed by the caller), also accumulates the row sums of |A| of the symmetric
// matrix from the lower triangle it reads (|A|_inf = max rowsum), so that A is read once: per
// panel, every warp leaves its rows' partial sums (and its columns' sums below the diagonal) in
// the staging buffer, and one thread per row adds them up.
template <typename T, int MAXR>
__device__ int cta_potrf(int n, const double* A, int lda, T* F, int ldf, T* buf, int* s_info,
                         double* rowsum = nullptr, double* blk64 = nullptr) {
    constexpr int NMAX = 32 * MAXR;
    __shared__ T rinv[kNB];
    int const tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) *s_info = 0;
    for (int k0 = 0; k0 < n; k0 += kNB) {
        int const nb = min(kNB, n - k0);
        int const m = n - k0;
        int const c0 = warp * 4;  // this warp's panel columns c0..c0+3 (relative to k0)
        T acc[MAXR][4];
        // All of the panel's loads are issued before any use, so that they overlap.
#pragma unroll
        for (int i = 0; i < MAXR; ++i) {
            int const r = lane + 32 * i;  // row relative to k0
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                int const c = c0 + j;
                acc[i][j] = (T)((r < m && c < nb && r >= c) ? A[(k0 + r) + (int64_t)(k0 + c) * lda] : 0.0);
            }
        }
        if (rowsum) {
            double* part = reinterpret_cast<double*>(buf);  // [kWarps][NMAX] rows, then [kNB] columns
            float csum[4] = {0.f, 0.f, 0.f, 0.f};  // |a| below the diagonal, per panel column
#pragma unroll
            for (int i = 0; i < MAXR; ++i) {
                int const r = lane + 32 * i;
                float rs = 0.f;  // binary32 sums: |A|_inf only scales the backward error
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    float const av = fabsf((float)acc[i][j]);  // (float)acc[i][j] == (float)a_rc for T float or double
                    rs += av;
                    if (r > c0 + j) csum[j] += av;
                }
                if (r < m) part[warp * NMAX + r] = rs;
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float v = csum[j];
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
                if (lane == 0) part[kWarps * NMAX + c0 + j] = v;
            }
            __syncthreads();
            for (int r = tid; r < m; r += kThreads) {
                double t = r < nb ? part[kWarps * NMAX + r] : 0.0;
#pragma unroll
                for (int w = 0; w < kWarps; ++w) t += part[w * NMAX + r];
                rowsum[k0 + r] += t;
            }
        }
        // The next panel's columns of A (lower part) start towards L2 while this panel is updated.
        if (k0 + kNB < n) {
            int const kn = k0 + kNB, cols = min(kNB, n - kn), lines = (n - kn + 15) / 16;
            for (int e = tid; e < cols * lines; e += kThreads) {
                int const c = e / lines, r = kn + (e - c * lines) * 16;
                asm volatile("prefetch.global.L2 [%0];" ::"l"(A + r + (int64_t)(kn + c) * lda));
            }
        }
        // Panel update with the previous columns.
        panel_update_dispatch<T, MAXR>(acc, F, ldf, buf, k0, m, c0);
        __syncthreads();
        // Panel to shared memory, column-major with stride NMAX.
#pragma unroll
        for (int i = 0; i < MAXR; ++i) {
            int const r = lane + 32 * i;
            if (r < m) {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (c0 + j < nb) buf[(c0 + j) * NMAX + r] = acc[i][j];
            }
        }
        __syncthreads();
        cta_panel_finish<T, NMAX>(buf, nb, m, k0, F, ldf, rinv, s_info, blk64);
    }
    return *s_info;
}

// ---------------------------------------------------------------------------------------------
// Tensor-core panel update for the binary32 factor (mixed path, modes 1 and 2).
//
// The update of panel k0 is the rank-k0 product P = F(k0:n, 0:k0) * F(k0:k0+32, 0:k0)^T
// subtracted from the panel of A: a (n-k0) x 32 x k0 gemm. It runs on the tensor cores as
// mma.sync m16n8k8 with TF32 operands and binary32 accumulation, in the 3xTF32 scheme: every
// binary32 operand x is split into x_hi = tf32(x) and x_lo = tf32(x - x_hi) (exact in binary32),
// and a*b is formed as a_lo*b_hi + a_hi*b_lo + a_hi*b_hi (the a_lo*b_lo term, about 2^-22 of
// a*b, is dropped); plain TF32 (about 2^-11) would stop the refinement from converging at
// cond(A) = 1e6. The accumulators start from the panel of A and take -F(i, k) (negation is
// exact), so D = A - P directly.
//
// Accumulator layout (mma's C fragment): warp w owns the row tiles rt = (w >> 1) + 4s (16 rows
// each) and the column tiles 2(w & 1) and 2(w & 1) + 1 (8 columns each) of the 32-column panel;
// lane (g = lane >> 2, t = lane & 3) holds rows 16rt + g (+8) and columns 2t, 2t + 1 of a tile.
// The previous columns are staged through shared memory with cp.async as in panel_update, 16 at
// a time and double-buffered, with a padded column stride (NMAX + 8 floats) so that the
// fragment reads are free of bank conflicts.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void tf32_split(float x, uint32_t& hi, uint32_t& lo) {
    uint32_t h, l;
    asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(h) : "f"(x));
    float const rest = x - __uint_as_float(h);
    asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(l) : "f"(rest));
    hi = h;
    lo = l;
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], uint32_t const (&a)[4], uint32_t b0, uint32_t b1) {
    asm("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

template <int MAXR>
struct TcShape {
    static constexpr int NMAX = 32 * MAXR;
    static constexpr int SP = NMAX + 8;                     // padded column stride of the staging buffer
    static constexpr int RT = MAXR >= 2 ? MAXR / 2 : 1;     // row tiles per warp (rows <= NMAX)
    static constexpr int kStageElems = kKC * SP;
};

template <int MAXR>
__device__ __forceinline__ void tc_stage(const float* F, int ldf, float* buf, int k0, int m, int ch) {
    constexpr int SP = TcShape<MAXR>::SP, KH = kKC / 2;
    int const kk = ch * KH;
    float* dst = buf + (ch & 1) * KH * SP;
    for (int q = 0; q < KH; ++q) {
        float const* src = F + k0 + (int64_t)(kk + q) * ldf;
        for (int r = threadIdx.x; r < m; r += kThreads) cp_async(dst + q * SP + r, src + r);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// R = row tiles this panel needs per warp (ceil(ceil(m / 16) / 4)), fixed at compile time.
template <int R, int MAXR>
__device__ __forceinline__ void tc_panel_update(float (&acc)[TcShape<MAXR>::RT][2][4], const float* F, int ldf,
                                                float* buf, int k0, int m) {
    constexpr int SP = TcShape<MAXR>::SP, KH = kKC / 2;
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int const g = lane >> 2, t = lane & 3, rg = warp >> 1, cp = warp & 1;
    int const rows16 = (m + 15) >> 4;
    int const nch = k0 / KH;  // k0 is a multiple of the panel width, so every chunk is full
    if (nch == 0) return;
    __syncthreads();  // the buffer's earlier contents are no longer read
    tc_stage<MAXR>(F, ldf, buf, k0, m, 0);
    for (int ch = 0; ch < nch; ++ch) {
        if (ch + 1 < nch) {
            tc_stage<MAXR>(F, ldf, buf, k0, m, ch + 1);
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        }
        __syncthreads();
        float const* base = buf + (ch & 1) * KH * SP;
#pragma unroll
        for (int ks = 0; ks < KH / 8; ++ks) {
            float const* col = base + (8 * ks + t) * SP;  // column 8ks + t; column 8ks + t + 4 at col + 4 SP
            uint32_t bh[2][2], bl[2][2];
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                int const cb = 16 * cp + 8 * j + g;
                tf32_split(col[cb], bh[j][0], bl[j][0]);
                tf32_split(col[4 * SP + cb], bh[j][1], bl[j][1]);
            }
            // Row tiles in pairs: the three products of the pair's four tiles are issued term by
            // term, so that the instructions updating one accumulator are four apart and the
            // ones in between are independent.
            int const live = min(R, (rows16 - rg + 3) >> 2);  // this warp's row tiles below the diagonal
#pragma unroll
            for (int s0 = 0; s0 < R; s0 += 2) {
                if (s0 < live) {  // warp-uniform
                    uint32_t ah[2][4], al[2][4];
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        int const r0 = 16 * (rg + 4 * (s0 + u)) + g;
                        tf32_split(-col[r0], ah[u][0], al[u][0]);
                        tf32_split(-col[r0 + 8], ah[u][1], al[u][1]);
                        tf32_split(-col[4 * SP + r0], ah[u][2], al[u][2]);
                        tf32_split(-col[4 * SP + r0 + 8], ah[u][3], al[u][3]);
                    }
                    bool const two = s0 + 1 < live && s0 + 1 < R;
#pragma unroll
                    for (int u = 0; u < 2; ++u)
                        if (u == 0 || two)
#pragma unroll
                            for (int j = 0; j < 2; ++j)
                                mma_tf32(acc[s0 + u < R ? s0 + u : s0][j], al[u], bh[j][0], bh[j][1]);
#pragma unroll
                    for (int u = 0; u < 2; ++u)
                        if (u == 0 || two)
#pragma unroll
                            for (int j = 0; j < 2; ++j)
                                mma_tf32(acc[s0 + u < R ? s0 + u : s0][j], ah[u], bl[j][0], bl[j][1]);
#pragma unroll
                    for (int u = 0; u < 2; ++u)
                        if (u == 0 || two)
#pragma unroll
                            for (int j = 0; j < 2; ++j)
                                mma_tf32(acc[s0 + u < R ? s0 + u : s0][j], ah[u], bh[j][0], bh[j][1]);
                }
            }
        }
        __syncthreads();  // every thread is done with this half before chunk ch + 2 is staged into it
    }
}

template <int MAXR>
__device__ __forceinline__ void tc_panel_update_dispatch(float (&acc)[TcShape<MAXR>::RT][2][4], const float* F,
                                                         int ldf, float* buf, int k0, int m) {
    int const rows16 = (m + 15) >> 4;
    switch ((rows16 + 3) >> 2) {
#define BLASTGPU_TC_CASE(R) \
    case R:                 \
        if constexpr (R <= TcShape<MAXR>::RT) tc_panel_update<R, MAXR>(acc, F, ldf, buf, k0, m); \
        break;
        BLASTGPU_TC_CASE(1) BLASTGPU_TC_CASE(2) BLASTGPU_TC_CASE(3) BLASTGPU_TC_CASE(4)
        BLASTGPU_TC_CASE(5) BLASTGPU_TC_CASE(6) BLASTGPU_TC_CASE(7) BLASTGPU_TC_CASE(8)
#undef BLASTGPU_TC_CASE
        default: break;
    }
}

// Binary32 left-looking Cholesky with the tensor-core panel update: lower(A) -> F, the same panel
// steps as cta_potrf<float> (and the same row sums of |A| when rowsum is given).
template <int MAXR>
__device__ int cta_potrf_tc(int n, const double* A, int lda, float* F, int ldf, float* buf, int* s_info,
                            double* rowsum, double* blk64) {
    constexpr int NMAX = 32 * MAXR, RT = TcShape<MAXR>::RT;
    __shared__ float rinv[kNB];
    int const tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int const g = lane >> 2, t = lane & 3, rg = warp >> 1, cp = warp & 1;
    if (tid == 0) *s_info = 0;
    for (int k0 = 0; k0 < n; k0 += kNB) {
        int const nb = min(kNB, n - k0);
        int const m = n - k0;
        float acc[RT][2][4];
        // The panel of A (lower part) into the accumulators, all loads issued before any use.
#pragma unroll
        for (int s = 0; s < RT; ++s)
#pragma unroll
            for (int j = 0; j < 2; ++j)
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    int const r = 16 * (rg + 4 * s) + g + 8 * (e >> 1);
                    int const c = 16 * cp + 8 * j + 2 * t + (e & 1);
                    acc[s][j][e] =
                        (r < m && c < nb && r >= c) ? (float)A[(k0 + r) + (int64_t)(k0 + c) * lda] : 0.f;
                }
        if (rowsum) {
            // part[cp][r]: row sums over this column pair's 16 columns; colp[rg][c]: column sums
            // strictly below the diagonal over this row group's rows.
            double* part = reinterpret_cast<double*>(buf);
            double* colp = part + 2 * NMAX;
#pragma unroll
            for (int s = 0; s < RT; ++s)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    float rs = fabsf(acc[s][0][2 * h]) + fabsf(acc[s][0][2 * h + 1]) + fabsf(acc[s][1][2 * h]) +
                               fabsf(acc[s][1][2 * h + 1]);
                    rs += __shfl_xor_sync(0xffffffffu, rs, 1);
                    rs += __shfl_xor_sync(0xffffffffu, rs, 2);
                    int const r = 16 * (rg + 4 * s) + g + 8 * h;
                    if (t == 0 && r < m) part[cp * NMAX + r] = rs;
                }
            float cs[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
            for (int s = 0; s < RT; ++s)
#pragma unroll
                for (int j = 0; j < 2; ++j)
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        int const r = 16 * (rg + 4 * s) + g + 8 * (e >> 1);
                        int const c = 16 * cp + 8 * j + 2 * t + (e & 1);
                        if (r > c) cs[j][e & 1] += fabsf(acc[s][j][e]);
                    }
#pragma unroll
            for (int j = 0; j < 2; ++j)
#pragma unroll
                for (int b = 0; b < 2; ++b) {
                    float v = cs[j][b];
                    v += __shfl_xor_sync(0xffffffffu, v, 4);
                    v += __shfl_xor_sync(0xffffffffu, v, 8);
                    v += __shfl_xor_sync(0xffffffffu, v, 16);
                    if (g == 0) colp[rg * kNB + 16 * cp + 8 * j + 2 * t + b] = v;
                }
            __syncthreads();
            for (int r = tid; r < m; r += kThreads) {
                double s2 = part[r] + part[NMAX + r];
                if (r < nb) s2 += colp[r] + colp[kNB + r] + colp[2 * kNB + r] + colp[3 * kNB + r];
                rowsum[k0 + r] += s2;
            }
        }
        // The next panel's columns of A (lower part) start towards L2 while this panel is updated.
        if (k0 + kNB < n) {
            int const kn = k0 + kNB, cols = min(kNB, n - kn), lines = (n - kn + 15) / 16;
            for (int e = tid; e < cols * lines; e += kThreads) {
                int const c = e / lines, r = kn + (e - c * lines) * 16;
                asm volatile("prefetch.global.L2 [%0];" ::"l"(A + r + (int64_t)(kn + c) * lda));
            }
        }
        tc_panel_update_dispatch<MAXR>(acc, F, ldf, buf, k0, m);
        __syncthreads();
        // Panel to shared memory, column-major with stride NMAX.
#pragma unroll
        for (int s = 0; s < RT; ++s)
#pragma unroll
            for (int j = 0; j < 2; ++j)
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    int const r = 16 * (rg + 4 * s) + g + 8 * (e >> 1);
                    int const c = 16 * cp + 8 * j + 2 * t + (e & 1);
                    if (r < m && c < nb) buf[c * NMAX + r] = acc[s][j][e];
                }
        __syncthreads();
        cta_panel_finish<float, NMAX>(buf, nb, m, k0, F, ldf, rinv, s_info, blk64);
    }
    return *s_info;
}

// In-place solve with the factor: v := F^{-T} F^{-1} v (v in shared memory, precision T).
// Blockwise with look-ahead, one barrier per 32-row block: once block b is solved, warp 0 applies
// it to the next block's 32 entries and solves that block's 32 x 32 triangle from registers
// (loaded straight from the factor, shuffles along the chain), while warps 1..7 apply block b to
// all entries beyond. Forward: row i of v takes each block's columns in order, j ascending;
// backward: entry i takes each solved block's rows r ascending, blocks from the bottom.
template <typename T>
__device__ __forceinline__ void potrs_fwd_block(const T* F, int ldf, int n, int j0, T* v, int lane) {
    int const nb = min(32, n - j0);
    T a[32];
#pragma unroll
    for (int k = 0; k < 32; ++k)
        a[k] = (lane < nb && k < lane) ? F[(j0 + lane) + (int64_t)(j0 + k) * ldf] : (T)0;
    T const rd = rcp_t<T>(lane < nb ? F[(j0 + lane) + (int64_t)(j0 + lane) * ldf] : (T)1);
    T x = lane < nb ? v[j0 + lane] : (T)0;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
        if (lane == j) x *= rd;
        T const xj = __shfl_sync(0xffffffffu, x, j);
        if (lane > j) x = fma(-a[j], xj, x);
    }
    if (lane < nb) v[j0 + lane] = x;
}

template <typename T>
__device__ __forceinline__ void potrs_bwd_block(const T* F, int ldf, int n, int j0, T* v, int lane) {
    int const nb = min(32, n - j0);
    T c[32];  // column lane of the block: c[k] = F(j0 + k, j0 + lane), k > lane
#pragma unroll
    for (int k = 0; k < 32; ++k)
        c[k] = (lane < nb && k > lane && k < nb) ? F[(j0 + k) + (int64_t)(j0 + lane) * ldf] : (T)0;
    T const rd = rcp_t<T>(lane < nb ? F[(j0 + lane) + (int64_t)(j0 + lane) * ldf] : (T)1);
    T x = lane < nb ? v[j0 + lane] : (T)0;
#pragma unroll
    for (int j = 31; j >= 0; --j) {
        if (lane == j) x *= rd;
        T const xj = __shfl_sync(0xffffffffu, x, j);
        if (lane < j) x = fma(-c[j], xj, x);
    }
    if (lane < nb) v[j0 + lane] = x;
}

template <typename T, int MAXR>
__device__ void cta_potrs(int n, const T* F, int ldf, T* v) {
    int const tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int const nblk = (n + 31) / 32;
    // forward: F * y = v
    if (warp == 0) potrs_fwd_block<T>(F, ldf, n, 0, v, lane);
    __syncthreads();
    for (int b = 0; b + 1 < nblk; ++b) {
        int const j0 = 32 * b, jn = j0 + 32, nbn = min(32, n - jn);  // block b is 32 wide
        if (warp == 0) {
            if (lane < nbn) {
                int const r = jn + lane;
                T acc = v[r];
#pragma unroll
                for (int j = 0; j < 32; ++j) acc = fma(-F[r + (int64_t)(j0 + j) * ldf], v[j0 + j], acc);
                v[r] = acc;
            }
            __syncwarp();
            potrs_fwd_block<T>(F, ldf, n, jn, v, lane);
        } else {
            for (int r = jn + 32 + (tid - 32); r < n; r += kThreads - 32) {
                T acc = v[r];
#pragma unroll
                for (int j = 0; j < 32; ++j) acc = fma(-F[r + (int64_t)(j0 + j) * ldf], v[j0 + j], acc);
                v[r] = acc;
            }
        }
        __syncthreads();
    }
    // backward: F^T * x = y, blocks from the bottom
    if (warp == 0) potrs_bwd_block<T>(F, ldf, n, 32 * (nblk - 1), v, lane);
    __syncthreads();
    for (int b = nblk - 1; b > 0; --b) {
        int const j0 = 32 * b, jp = j0 - 32, nb = min(32, n - j0);  // block b - 1 is 32 wide
        if (warp == 0) {
            int const i = jp + lane;
            T acc = v[i];
            const T* col = F + j0 + (int64_t)i * ldf;
#pragma unroll 8
            for (int r = 0; r < nb; ++r) acc = fma(-col[r], v[j0 + r], acc);
            v[i] = acc;
            __syncwarp();
            potrs_bwd_block<T>(F, ldf, n, jp, v, lane);
        } else {
            for (int i = tid - 32; i < jp; i += kThreads - 32) {
                T acc = v[i];
                const T* col = F + j0 + (int64_t)i * ldf;
#pragma unroll 8
                for (int r = 0; r < nb; ++r) acc = fma(-col[r], v[j0 + r], acc);
                v[i] = acc;
            }
        }
        __syncthreads();
    }
}

// Block-wide max reduction of non-negative values (NaN propagates as the result).
__device__ __forceinline__ double cta_max(double v, double* red) {
    int const tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        double const o = __shfl_xor_sync(0xffffffffu, v, off);
        v = (o > v || o != o) ? o : v;
    }
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double r = red[0];
    for (int w = 1; w < kWarps; ++w) r = (red[w] > r || red[w] != red[w]) ? red[w] : r;
    return r;
}

// y = A*x for symmetric A given by its lower triangle (binary64); x, y in shared memory; part:
// kWarps * NMAX doubles of shared scratch. One pass over the lower triangle: a warp takes a group
// of 16 columns (groups g and ng-1-g together, so that the warps' shares are even), lanes over
// rows, and every element a_ji (j >= i) feeds both the row sum of j (in the lane, then the warp's
// row partials in part) and, below the diagonal, the column sum of i (16 accumulators per lane,
// folded across the warp at the end of the group). Each element is read once and costs its two
// FMAs; the cross-lane sums take 16 additions per 16 columns.
template <int NMAX>
__device__ void cta_symv_lower(int n, const double* A, int lda, const double* x, double* y, double* part) {
    int const tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    double* mine = part + warp * NMAX;
    for (int i = lane; i < n; i += 32) mine[i] = 0.0;
    __syncwarp();
    int const ng = (n + 15) / 16;
    for (int t = warp; t < (ng + 1) / 2; t += kWarps) {
        for (int h = 0; h < 2; ++h) {
            int const g = h == 0 ? t : ng - 1 - t;
            if (h == 1 && g == t) break;
            int const i0 = 16 * g, gc = min(16, n - i0);
            double p[16], xc[16];
#pragma unroll
            for (int c = 0; c < 16; ++c) {
                p[c] = 0.0;
                xc[c] = c < gc ? x[i0 + c] : 0.0;
            }
            for (int jb = i0; jb < n; jb += 32) {
                int const j = jb + lane;
                double const xj = j < n ? x[j] : 0.0;
                double a[16];
#pragma unroll
                for (int c = 0; c < 16; ++c)
                    a[c] = (j < n && c < gc && j >= i0 + c) ? A[j + (int64_t)(i0 + c) * lda] : 0.0;
                double r = 0.0;
#pragma unroll
                for (int c = 0; c < 16; ++c) {
                    r = fma(a[c], xc[c], r);
                    p[c] = fma(a[c], j > i0 + c ? xj : 0.0, p[c]);
                }
                if (j < n) mine[j] += r;
            }
            // fold p[c] across the 32 lanes: after the halving steps lane l holds column (l & 15)'s
            // sum over one half-warp; one more exchange adds the other half
#pragma unroll
            for (int w = 8; w >= 1; w >>= 1) {
                bool const upper = (lane & w) != 0;
#pragma unroll
                for (int c = 0; c < w; ++c) {
                    double const give = upper ? p[c] : p[c + w];
                    double const keep = upper ? p[c + w] : p[c];
                    p[c] = keep + __shfl_xor_sync(0xffffffffu, give, w);
                }
            }
            double const colsum = p[0] + __shfl_xor_sync(0xffffffffu, p[0], 16);
            __syncwarp();
            int const ci = lane & 15;
            if (lane < 16 && ci < gc) mine[i0 + ci] += colsum;
            __syncwarp();
        }
    }
    __syncthreads();
    for (int i = tid; i < n; i += kThreads) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) s += part[w * NMAX + i];
        y[i] = s;
    }
    __syncthreads();
}

struct CtaArgs {
    int64_t batch;
    int32_t* info;
    int32_t* iters;
    double* berr;
    double tol;
    int max_iter;
};

// Plain binary64 path: factor into L, then X = A^{-1} B column by column.
template <int MAXR, class Batch>
__global__ void __launch_bounds__(kThreads, MAXR <= 8 ? 2 : 1) posv_cta_f64_kernel(Batch batch, CtaArgs args) {
    using S = Smem<double, MAXR>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* buf = reinterpret_cast<double*>(smem_raw);
    double* vec = buf + S::kBufElems;
    __shared__ int s_info;
    int64_t const b = blockIdx.x;
    if (b >= args.batch) return;
    CtaItem const it = batch.get(b);
    int const n = it.n;
    if (it.A != nullptr) {  // A == nullptr: solves with the given factor L only
        int const info = cta_potrf<double, MAXR>(n, it.A, it.lda, it.L, it.ldl, buf, &s_info);
        if (threadIdx.x == 0 && args.info) args.info[b] = info;
    }
    for (int c = 0; c < it.nrhs; ++c) {
        for (int i = threadIdx.x; i < n; i += kThreads) vec[i] = it.B[i + (int64_t)c * it.ldb];
        __syncthreads();
        cta_potrs<double, MAXR>(n, it.L, it.ldl, vec);
        for (int i = threadIdx.x; i < n; i += kThreads) it.X[i + (int64_t)c * it.ldx] = vec[i];
        __syncthreads();
    }
}

// Shared-memory layout of the mixed kernel: the panel / staging buffer (binary32, large enough
// for the tensor-core update's padded staging in modes 1 and 2), four vectors of NMAX doubles plus
// reductions, and, for binary64 diagonal blocks, a 32 x 32 block of doubles and its 32 reciprocals.
template <int MAXR, int MODE>
struct MixedSmem {
    static constexpr int NMAX = 32 * MAXR;
    static constexpr bool kTc = MODE == 1 || MODE == 2;
    static constexpr bool kDiag64 = MODE == 2 || MODE == 3;
    static constexpr int kBufElems = (kTc && TcShape<MAXR>::kStageElems > Smem<float, MAXR>::kBufElems)
                                         ? TcShape<MAXR>::kStageElems
                                         : Smem<float, MAXR>::kBufElems;
    static constexpr size_t kVecOffset = sizeof(float) * kBufElems;
    static constexpr size_t kBlkOffset = kVecOffset + sizeof(double) * (4 * NMAX + 64);
    static constexpr size_t kBytes = kBlkOffset + (kDiag64 ? sizeof(double) * (32 * 32 + 32) : 0);
};

// Mixed path: binary32 factor in the workspace, binary64 refinement. MODE selects the
// factorisation: 0 = binary32 CUDA-core panel update (cta_potrf<float>), 1 = tensor-core 3xTF32
// panel update (cta_potrf_tc), 2 = as 1 with binary64 diagonal blocks, 3 = as 0 with binary64
// diagonal blocks.
template <int MAXR, class Batch, int MODE>
__global__ void __launch_bounds__(kThreads, 2) posv_cta_mixed_kernel(Batch batch, CtaArgs args) {
    using S = MixedSmem<MAXR, MODE>;
    constexpr int NMAX = S::NMAX;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* buf = reinterpret_cast<float*>(smem_raw);
    double* x = reinterpret_cast<double*>(smem_raw + S::kVecOffset);
    double* r = x + NMAX;
    double* bb = r + NMAX;
    float* w = reinterpret_cast<float*>(bb + NMAX);  // NMAX floats (fits in the 4th vector)
    double* red = bb + 2 * NMAX;
    double* blk64 = S::kDiag64 ? reinterpret_cast<double*>(smem_raw + S::kBlkOffset) : nullptr;
    __shared__ int s_info;
    int64_t const b = blockIdx.x;
    if (b >= args.batch) return;
    CtaItem const it = batch.get(b);
    int const n = it.n, tid = threadIdx.x;
    if (n < 0) {  // scratch range outside the fixed array: reported, nothing written
        if (tid == 0) {
            if (args.info) args.info[b] = -1;
            if (args.iters) args.iters[b] = 0;
            if (args.berr) args.berr[b] = CUDART_NAN;
        }
        return;
    }
    float* F = reinterpret_cast<float*>(it.ws);
    for (int i = tid; i < n; i += kThreads) r[i] = 0.0;
    __syncthreads();
    // the factorisation also leaves the row sums of |A| in r
    int info;
    if constexpr (S::kTc) info = cta_potrf_tc<MAXR>(n, it.A, it.lda, F, n, buf, &s_info, r, blk64);
    else info = cta_potrf<float, MAXR>(n, it.A, it.lda, F, n, buf, &s_info, r, blk64);
    if (tid == 0 && args.info) args.info[b] = info;

    // |A|_inf = max row sum of |A| (accumulated by the factorisation from the lower triangle)
    double anorm;
    {
        double m = 0.0;
        for (int i = tid; i < n; i += kThreads) m = fmax(m, r[i]);
        anorm = cta_max(m, red);
    }

    int total_iters = 0;
    double worst = 0.0;
    for (int c = 0; c < it.nrhs; ++c) {
        double bm = 0.0;
        for (int i = tid; i < n; i += kThreads) {
            bb[i] = it.B[i + (int64_t)c * it.ldb];
            bm = fmax(bm, fabs(bb[i]));
        }
        double const bnorm = cta_max(bm, red);
        // x0 = F^{-T} F^{-1} b in binary32
        for (int i = tid; i < n; i += kThreads) w[i] = (float)bb[i];
        __syncthreads();
        if (info == 0) cta_potrs<float, MAXR>(n, F, n, w);
        for (int i = tid; i < n; i += kThreads) x[i] = info == 0 ? (double)w[i] : CUDART_NAN;
        __syncthreads();
        double be = CUDART_NAN;  // a failed binary32 factorisation leaves no solution to refine
        int it_count = 0;
        while (info == 0) {
            // r = b - A x (binary64)
            cta_symv_lower<NMAX>(n, it.A, it.lda, x, r, reinterpret_cast<double*>(buf));
            double rm = 0.0, xm = 0.0;
            for (int i = tid; i < n; i += kThreads) {
                r[i] = bb[i] - r[i];
                double const ar = fabs(r[i]), ax = fabs(x[i]);
                rm = (ar > rm || ar != ar) ? ar : rm;  // NaN-propagating maxima
                xm = (ax > xm || ax != ax) ? ax : xm;
            }
            rm = cta_max(rm, red);
            xm = cta_max(xm, red);
            double const den = anorm * xm + bnorm;
            be = den > 0.0 ? rm / den : (rm == 0.0 ? 0.0 : CUDART_INF);
            if (!(be > args.tol) || it_count >= args.max_iter) break;
            // d = F^{-T} F^{-1} (r / s) * s in binary32, with s = |r|_inf keeping r in range
            double const s = rm;
            for (int i = tid; i < n; i += kThreads) w[i] = (float)(r[i] / s);
            __syncthreads();
            cta_potrs<float, MAXR>(n, F, n, w);
            for (int i = tid; i < n; i += kThreads) x[i] += (double)w[i] * s;
            __syncthreads();
            ++it_count;
        }
        for (int i = tid; i < n; i += kThreads) it.X[i + (int64_t)c * it.ldx] = x[i];
        __syncthreads();
        total_iters = max(total_iters, it_count);
        worst = (be > worst || be != be) ? be : worst;
    }
    if (tid == 0) {
        if (args.iters) args.iters[b] = total_iters;
        if (args.berr) args.berr[b] = worst;
    }
}

// Adjoint of X = A^{-1} B for SPD A (no BLAST counterpart): given the factor L (or A, to
// recompute it) and dl/dX, writes dl/dB = A^{-1} dl/dX and the symmetric
// dl/dA = -(dl/dB X^T + X dl/dB^T)/2, all binary64.
struct BwdItem {
    int n, nrhs;
    const double* A; int lda;
    double* L; int ldl;
    const double* X; int ldx;
    const double* G; int ldg;   // dl/dX
    double* GB; int ldgb;       // dl/dB
    double* GA; int ldga;       // dl/dA
};

struct DescBwd {
    const blastgpu_posv_bwd_desc* desc;
    __device__ BwdItem get(int64_t b) const {
        blastgpu_posv_bwd_desc const& d = desc[b];
        return {d.A.rows, d.X.cols, d.A.data, d.A.ld, d.L.data, d.L.ld, d.X.data, d.X.ld,
                d.Xbar.data, d.Xbar.ld, d.Bbar.data, d.Bbar.ld, d.Abar.data, d.Abar.ld};
    }
};

template <int MAXR, class Batch>
// Two CTAs per SM up to n = 128 (MAXR <= 4 fits 128 registers per thread); larger bins keep the
// register budget of one CTA per SM.
__global__ void __launch_bounds__(kThreads, MAXR <= 4 ? 2 : 1)
    posv_bwd_kernel(Batch batch, int64_t count, int recompute, int32_t* info) {
    using S = Smem<double, MAXR>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* buf = reinterpret_cast<double*>(smem_raw);
    double* vec = buf + S::kBufElems;
    __shared__ int s_info;
    int64_t const b = blockIdx.x;
    if (b >= count) return;
    BwdItem const it = batch.get(b);
    int const n = it.n, tid = threadIdx.x;
    if (recompute) {
        int const r = cta_potrf<double, MAXR>(n, it.A, it.lda, it.L, it.ldl, buf, &s_info);
        if (tid == 0 && info) info[b] = r;
    } else if (tid == 0 && info) {
        info[b] = 0;
    }
    __syncthreads();
    for (int c = 0; c < it.nrhs; ++c) {
        for (int i = tid; i < n; i += kThreads) vec[i] = it.G[i + (int64_t)c * it.ldg];
        __syncthreads();
        cta_potrs<double, MAXR>(n, it.L, it.ldl, vec);
        for (int i = tid; i < n; i += kThreads) it.GB[i + (int64_t)c * it.ldgb] = vec[i];
        __syncthreads();
    }
    // GA = -sym(GB X^T): warp per column, lanes over rows (coalesced stores). With one
    // right-hand side, GB (still in vec) and X come from shared memory.
    int const lane = tid & 31, warp = tid >> 5;
    if (it.nrhs == 1) {
        double* xs = vec + S::NMAX;
        for (int i = tid; i < n; i += kThreads) xs[i] = it.X[i];
        __syncthreads();
        for (int j = warp; j < n; j += kWarps) {
            double const xj = xs[j], gj = vec[j];
            double* ga = it.GA + (int64_t)j * it.ldga;
            for (int i = lane; i < n; i += 32) ga[i] = -0.5 * fma(xs[i], gj, vec[i] * xj);
        }
        return;
    }
    for (int j = warp; j < n; j += kWarps)
        for (int i = lane; i < n; i += 32) {
            double acc = 0.0;
            for (int c = 0; c < it.nrhs; ++c) {
                acc = fma(it.GB[i + (int64_t)c * it.ldgb], it.X[j + (int64_t)c * it.ldx], acc);
                acc = fma(it.X[i + (int64_t)c * it.ldx], it.GB[j + (int64_t)c * it.ldgb], acc);
            }
            it.GA[i + (int64_t)j * it.ldga] = -0.5 * acc;
        }
}

template <int MAXR>
int launch_bwd(DescBwd const& batch, int64_t count, int recompute, int32_t* info, cudaStream_t s) {
    size_t const smem = Smem<double, MAXR>::kBytes;
    cudaError_t e = ensure_smem<posv_bwd_kernel<MAXR, DescBwd>>(smem);
    if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
    posv_bwd_kernel<MAXR, DescBwd><<<(unsigned)count, kThreads, smem, s>>>(batch, count, recompute, info);
    return check_launch();
}

template <int MAXR, class Batch, int MODE>
cudaError_t launch_mixed(Batch const& batch, CtaArgs const& args, cudaStream_t s) {
    size_t const smem = MixedSmem<MAXR, MODE>::kBytes;
    cudaError_t const e = ensure_smem<posv_cta_mixed_kernel<MAXR, Batch, MODE>>(smem);
    if (e == cudaSuccess)
        posv_cta_mixed_kernel<MAXR, Batch, MODE><<<(unsigned)args.batch, kThreads, smem, s>>>(batch, args);
    return e;
}

// "posv.mixed.n<bin>" selects the mixed factorisation per size bin (MODE of posv_cta_mixed_kernel;
// default 0, the fastest measured on GB300).
template <int MAXR, class Batch>
int launch_cta(bool mixed, Batch const& batch, CtaArgs const& args, cudaStream_t s) {
    size_t const smem = Smem<double, MAXR>::kBytes;
    cudaError_t e = cudaSuccess;
    if (mixed) {
        // only descriptor batches carry the mixed path's workspace offsets
        if constexpr (std::is_same_v<Batch, DescPosv>) {
            switch (tune_get_bin("posv.mixed", 32 * MAXR, 0)) {
                case 1: e = launch_mixed<MAXR, Batch, 1>(batch, args, s); break;
                case 2: e = launch_mixed<MAXR, Batch, 2>(batch, args, s); break;
                case 3: e = launch_mixed<MAXR, Batch, 3>(batch, args, s); break;
                default: e = launch_mixed<MAXR, Batch, 0>(batch, args, s); break;
            }
        } else {
            return BLASTGPU_ERR_NOT_IMPLEMENTED;
        }
    } else {
        e = ensure_smem<posv_cta_f64_kernel<MAXR, Batch>>(smem);
        if (e == cudaSuccess) posv_cta_f64_kernel<MAXR, Batch><<<(unsigned)args.batch, kThreads, smem, s>>>(batch, args);
    }
    if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
    return check_launch();
}

template <class Batch>
int dispatch_cta(bool mixed, int max_n, Batch const& batch, CtaArgs const& args, cudaStream_t s) {
    if (args.batch == 0) return BLASTGPU_SUCCESS;
    if (args.batch > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    if (max_n <= 64) return launch_cta<2>(mixed, batch, args, s);
    if (max_n <= 128) return launch_cta<4>(mixed, batch, args, s);
    if (max_n <= 256) return launch_cta<8>(mixed, batch, args, s);
    if (max_n <= 512) return launch_cta<16>(mixed, batch, args, s);
    return BLASTGPU_ERR_TOO_LARGE;
}

}  // namespace

int launch_posv_cta_strided(int n, int nrhs, const double* A, int lda, int64_t sa, double* L, int ldl,
                            int64_t sl, const double* B, int ldb, int64_t sb, double* X, int ldx, int64_t sx,
                            int32_t* info, int64_t batch, cudaStream_t s) {
    StridedPosv const p{n, nrhs, A, lda, sa, L, ldl, sl, B, ldb, sb, X, ldx, sx};
    CtaArgs const a{batch, info, nullptr, nullptr, 0.0, 0};
    return dispatch_cta(false, n, p, a, s);
}

namespace {

// Scratch for blastgpu_dposv_mixed_batched_noalloc: a fixed array in the module's device memory,
// reserved on every GPU that loads the library until the process exits. It holds the binary32
// factors of one call; every call reuses it, so calls whose kernels overlap on the GPU race.
constexpr size_t kNoAllocScratchBytes = BLASTGPU_NOALLOC_SCRATCH_BYTES;  // 32 MiB
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch on the current device, looked up once per device (the
// host-side symbol is only a stand-in and must not be passed to a kernel).
cudaError_t noalloc_scratch(void** out) {
    static std::mutex mu;
    static void* addr[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        addr[dev] = p;
    }
    *out = addr[dev];
    return cudaSuccess;
}

}  // namespace
}  // namespace blastgpu

using namespace blastgpu;

extern "C" {

int blastgpu_dposv_mixed_batched_noalloc(const blastgpu_posv_desc* desc, int64_t batch, int max_n,
                                         size_t scratch_bytes, double tol, int max_iter, int32_t* info,
                                         int32_t* iters, double* berr, blastgpu_stream_t stream) {
    if (batch < 0) return -2;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (!desc) return -1;
    if (max_n < 0) return -3;
    if (max_n > 512) return BLASTGPU_ERR_TOO_LARGE;
    if (scratch_bytes > kNoAllocScratchBytes) return BLASTGPU_ERR_TOO_LARGE;
    if (!(tol >= 0.0)) return -5;
    if (max_iter < 0) return -6;
    void* scratch = nullptr;
    cudaError_t const e = noalloc_scratch(&scratch);
    if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
    CtaArgs a{batch, info, iters, berr, tol, max_iter};
    return dispatch_cta(true, max_n, DescPosv{desc, static_cast<char*>(scratch), (int64_t)kNoAllocScratchBytes}, a,
                        as_cuda(stream));
}

size_t blastgpu_dposv_mixed_workspace_bytes(int n) {
    if (n <= 0) return 0;
    size_t const bytes = sizeof(float) * (size_t)n * (size_t)n;
    return (bytes + 255) & ~(size_t)255;
}

int blastgpu_dposv_batched(const blastgpu_posv_desc* desc, int64_t batch, int max_n, int32_t* info,
                           blastgpu_stream_t stream) {
    if (batch < 0) return -2;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (!desc) return -1;
    if (max_n < 0) return -3;
    if (max_n > 512) return BLASTGPU_ERR_TOO_LARGE;
    // "posv.warp.n<bin>" (default 1): batches with every n <= 128 on the warp-per-matrix kernel
    if (max_n <= 128 && tune_get_bin("posv.warp", max_n, 1) != 0)
        return launch_posv_warp(desc, batch, max_n, info, as_cuda(stream));
    CtaArgs a{batch, info, nullptr, nullptr, 0.0, 0};
    return dispatch_cta(false, max_n, DescPosv{desc, nullptr}, a, as_cuda(stream));
}

int blastgpu_dposv_mixed_batched(const blastgpu_posv_desc* desc, int64_t batch, int max_n,
                                 void* workspace, double tol, int max_iter, int32_t* info,
                                 int32_t* iters, double* berr, blastgpu_stream_t stream) {
    if (batch < 0) return -2;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (!desc) return -1;
    if (max_n < 0) return -3;
    if (max_n > 512) return BLASTGPU_ERR_TOO_LARGE;
    if (!workspace) return -4;
    if (!(tol >= 0.0)) return -5;
    if (max_iter < 0) return -6;
    CtaArgs a{batch, info, iters, berr, tol, max_iter};
    return dispatch_cta(true, max_n, DescPosv{desc, static_cast<char*>(workspace)}, a, as_cuda(stream));
}

int blastgpu_dposv_bwd_batched(const blastgpu_posv_bwd_desc* desc, int64_t batch, int max_n,
                               int recompute, int32_t* info, blastgpu_stream_t stream) {
    if (batch < 0) return -2;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (!desc) return -1;
    if (max_n < 0) return -3;
    if (recompute != 0 && recompute != 1) return -4;
    if (batch > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    DescBwd d{desc};
    cudaStream_t const s = as_cuda(stream);
    // "posv.warp_bwd.n<bin>" (default 1): batches with every n <= 128 one warp per matrix
    if (max_n <= 128 && tune_get_bin("posv.warp_bwd", max_n, 1) != 0)
        return launch_posv_bwd_warp(desc, batch, max_n, recompute, info, s);
    if (max_n <= 64) return launch_bwd<2>(d, batch, recompute, info, s);
    if (max_n <= 128) return launch_bwd<4>(d, batch, recompute, info, s);
    if (max_n <= 256) return launch_bwd<8>(d, batch, recompute, info, s);
    if (max_n <= 512) return launch_bwd<16>(d, batch, recompute, info, s);
    return BLASTGPU_ERR_TOO_LARGE;
}

}  // extern "C"

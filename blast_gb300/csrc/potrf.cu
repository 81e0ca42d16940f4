// Batched Cholesky factorisation and solve (potrf, potrs, posv), binary64, sm_103a.
//
// Reference: blast::potrf (dense/Potrf.hpp:20-106): left-looking, column strips of KN = 4,
// each strip covered top-down by register tiles of 12, 8 and 4 rows (TileSize<double> = 4).
// Per tile: load A, subtract L(i:,0:k)*L(k:k+4,0:k)^T with fused rank-1 updates (ger(-1,..)),
// then either factor the diagonal tile in registers (RegisterMatrix::potrf,
// register_matrix/RegisterMatrix.hpp:710-739) or solve against the diagonal block
// (RegisterMatrix::trsm(Right, Upper), :566-602), and store.
// The solves follow blast::trsm (dense/Trsm.hpp:17-66): L*Y = B, then trans(L)*X = Y.
//
// GPU mapping ("thread per matrix"): on GB300 the binary64 pipe issues one warp-wide FMA per
// ~64 cycles per SM sub-partition (measured 1.2 TFLOP/s for the whole chip), and a division or
// square root costs about ten FMA slots. Splitting one small factorisation over a warp leaves
// most lanes idle on the diagonal (sqrt, reciprocal, short columns). Running BLAST's own
// single-instance algorithm in every thread keeps all 32 lanes on useful FMAs, the diagonal
// operations included, and keeps BLAST's register tiles (12/8/4 x 4) as the per-thread
// accumulators. Each thread reads its own column segments, which stay in L1/L2 between the
// strips of the left-looking sweep.
//
// Numerics: the per-element order of fused multiply-adds is BLAST's; the division by the pivot
// (s / sqrt(s_cc), s / l_cc) becomes a multiplication by a reciprocal square root computed once
// per column (rsqrt_nr). Results differ from BLAST's by a few units in the last place.
#include "common.cuh"

namespace blastgpu {
namespace {

// Addressing policies: BLAST's dense column-major storage and its panel storage with panel
// height PS (element (i, j) at (i/PS)*spacing + i%PS + j*PS, panel/StaticPanelMatrix.hpp:178-184).
struct ColAddr {
    int64_t ld;
    __device__ __forceinline__ int64_t operator()(int i, int j) const { return i + (int64_t)j * ld; }
};

template <int PS>
struct PanelAddr {
    int64_t spacing;
    __device__ __forceinline__ int64_t operator()(int i, int j) const {
        return (int64_t)(i / PS) * spacing + i % PS + (int64_t)j * PS;
    }
};

// Sources of the matrix being factorised; fill() loads the KM x KN tile at (i, k).
// LoadSrc: the input matrix A itself (blast::potrf(A, L)).
template <class Addr>
struct LoadSrc {
    const double* A;
    Addr ia;
    template <int KM, int KN, bool DIAG>
    __device__ __forceinline__ void fill(double (&acc)[KM][KN], int n, int k, int i, int nc) const {
#pragma unroll
        for (int c = 0; c < KN; ++c)
#pragma unroll
            for (int r = 0; r < KM; ++r)
                acc[r][c] = (c < nc && i + r < n) ? A[ia(i + r, k + c)] : 0.0;
    }
};

// SyrkSrc: beta*C + alpha*A*A^T (A: n x K, or K x n read transposed), formed tile by tile in the
// order of blast::syrkLower (dense/Syrk.hpp:15-145): v = beta*c_ij rounded (RegisterMatrix::load(
// beta, ..)), then for l ascending v = fma(alpha*a_il, a_jl, v) (RegisterMatrix::ger(alpha, ..)).
// The factorisation then runs on exactly the values syrkLower would have stored. ALPHA1: alpha is
// 1, so alpha*a_il is a_il exactly and its multiplication is left out.
template <bool ALPHA1>
struct SyrkSrc {
    const double* A;
    int64_t lda;
    int K;
    bool trans;
    double alpha, beta;
    const double* C;
    int64_t ldc;
    __device__ __forceinline__ double a(int i, int l) const {
        return trans ? A[l + (int64_t)i * lda] : A[i + (int64_t)l * lda];
    }
    template <int KM, int KN, bool DIAG>
    __device__ __forceinline__ void fill(double (&acc)[KM][KN], int n, int k, int i, int nc) const {
#pragma unroll
        for (int c = 0; c < KN; ++c)
#pragma unroll
            for (int r = 0; r < KM; ++r)
                acc[r][c] = (c < nc && i + r < n && (!DIAG || r >= c)) ? beta * C[(i + r) + (int64_t)(k + c) * ldc]
                                                                      : 0.0;
        for (int l = 0; l < K; ++l) {
            double ax[KM], b[KN];
#pragma unroll
            for (int r = 0; r < KM; ++r) ax[r] = (i + r < n) ? (ALPHA1 ? a(i + r, l) : alpha * a(i + r, l)) : 0.0;
#pragma unroll
            for (int c = 0; c < KN; ++c) b[c] = (c < nc) ? a(k + c, l) : 0.0;
#pragma unroll
            for (int c = 0; c < KN; ++c)
#pragma unroll
                for (int r = 0; r < KM; ++r)
                    if (!DIAG || r >= c) acc[r][c] = fma(ax[r], b[c], acc[r][c]);
        }
    }
};

// One KM x KN register tile of the left-looking strip k (rows i .. i+KM-1 of the n rows passed
// as the first argument, the matrix's row count). DIAG: the strip's
// first tile, which holds the diagonal block; its strictly upper entries (r < c) are never stored,
// so their fused multiply-adds are left out at compile time.
// PF: the operands of column l + 1 are loaded before the fused multiply-adds of column l (one column
// of look-ahead), so that a load's latency overlaps the previous column's arithmetic; the order of
// operations on every element is the same either way.
template <int KM, int KN, bool DIAG, bool PF = false, class Src, class Addr>
__device__ __forceinline__ void potrf_tile(int n, int k, int i, int nc, Src const& src, double* L, Addr il,
                                           double (&y)[KN], int& info) {
    constexpr bool diag = DIAG;
    double acc[KM][KN];
    src.template fill<KM, KN, DIAG>(acc, n, k, i, nc);

    // acc -= L(i:i+KM, 0:k) * L(k:k+KN, 0:k)^T, one fused rank-1 update per column l
    // (BLAST's ger(-1, ...) loop, dense/Potrf.hpp:40-41).
    if constexpr (PF) {
        double a[KM], b[KN];
        if (k > 0) {
#pragma unroll
            for (int r = 0; r < KM; ++r) a[r] = (i + r < n) ? L[il(i + r, 0)] : 0.0;
#pragma unroll
            for (int c = 0; c < KN; ++c) b[c] = (c < nc) ? L[il(k + c, 0)] : 0.0;
        }
        for (int l = 0; l < k; ++l) {
            double an[KM], bn[KN];
            int const ln = l + 1 < k ? l + 1 : l;
#pragma unroll
            for (int r = 0; r < KM; ++r) an[r] = (i + r < n) ? L[il(i + r, ln)] : 0.0;
#pragma unroll
            for (int c = 0; c < KN; ++c) bn[c] = (c < nc) ? L[il(k + c, ln)] : 0.0;
#pragma unroll
            for (int c = 0; c < KN; ++c)
#pragma unroll
                for (int r = 0; r < KM; ++r)
                    if (!DIAG || r >= c) acc[r][c] = fma(-a[r], b[c], acc[r][c]);
#pragma unroll
            for (int r = 0; r < KM; ++r) a[r] = an[r];
#pragma unroll
            for (int c = 0; c < KN; ++c) b[c] = bn[c];
        }
    } else {
        for (int l = 0; l < k; ++l) {
            double a[KM], b[KN];
#pragma unroll
            for (int r = 0; r < KM; ++r) a[r] = (i + r < n) ? L[il(i + r, l)] : 0.0;
#pragma unroll
            for (int c = 0; c < KN; ++c) b[c] = (c < nc) ? L[il(k + c, l)] : 0.0;
#pragma unroll
            for (int c = 0; c < KN; ++c)
#pragma unroll
                for (int r = 0; r < KM; ++r)
                    if (!DIAG || r >= c) acc[r][c] = fma(-a[r], b[c], acc[r][c]);
        }
    }

    if (diag) {
        // In-register Cholesky of the strip (RegisterMatrix::potrf).
#pragma unroll
        for (int c = 0; c < KN; ++c) {
            if (c < nc) {
#pragma unroll
                for (int j = 0; j < c; ++j) {
                    double const lcj = acc[c][j];
#pragma unroll
                    for (int r = 0; r < KM; ++r)
                        if (r >= c) acc[r][c] = fma(-lcj, acc[r][j], acc[r][c]);
                }
                double const s = acc[c][c];
                if (!(s > 0.0) && info == 0) info = k + c + 1;
                y[c] = rsqrt_nr(s);
#pragma unroll
                for (int r = 0; r < KM; ++r)
                    if (r >= c) acc[r][c] *= y[c];
            }
        }
#pragma unroll
        for (int c = 0; c < KN; ++c)
#pragma unroll
            for (int r = 0; r < KM; ++r)
                if (c < nc && r >= c && i + r < n) L[il(i + r, k + c)] = acc[r][c];
    } else {
        // Right upper solve against the strip's diagonal block (RegisterMatrix::trsm).
#pragma unroll
        for (int c = 0; c < KN; ++c) {
            if (c < nc) {
#pragma unroll
                for (int j = 0; j < c; ++j) {
                    double const lcj = L[il(k + c, k + j)];
#pragma unroll
                    for (int r = 0; r < KM; ++r) acc[r][c] = fma(-lcj, acc[r][j], acc[r][c]);
                }
#pragma unroll
                for (int r = 0; r < KM; ++r) acc[r][c] *= y[c];
            }
        }
#pragma unroll
        for (int c = 0; c < KN; ++c)
#pragma unroll
            for (int r = 0; r < KM; ++r)
                if (c < nc && i + r < n) L[il(i + r, k + c)] = acc[r][c];
    }
}

// Left-looking Cholesky of one n x n matrix, strips of KN columns, row tiles of 3, 2 and 1 times
// TS rows (dense: KN = TS = 4, dense/Potrf.hpp:87-105; panel: KN = min((RC-4)/3, SS), TS = SS,
// panel/Potrf.hpp:84-105). Returns info (0 or first bad pivot + 1).
struct NoStripHook {
    __device__ __forceinline__ void before(int, int) const {}
    __device__ __forceinline__ void after(int, int) const {}
};

// hook.before(k, nc) runs before strip k reads its columns, hook.after(k, nc) once columns
// k .. k+nc-1 of L are final. The matrix is m x n with m >= n (BLAST's potrf accepts such
// trapezoids, dense/Potrf.hpp:78-105: the tiles of every strip run down to row m, so the rows
// below the top n x n block are solved against its factor). PF selects the tiles' load look-ahead.
template <int KN, int TS, class Src, class Addr, class Hook = NoStripHook, bool PF = false>
__device__ int potrf_thread_src_mn(int m, int n, Src const& A, double* L, Addr il, Hook const& hook = Hook{}) {
    int info = 0;
    for (int k = 0; k < n; k += KN) {
        int const nc = min(KN, n - k);
        hook.before(k, nc);
        double y[KN];
        int i = k;
        while (i < m) {
            int const rem = m - i;
            // BLAST's tile cover: 3*TS rows while more than 2*TS remain, then 2*TS while more
            // than TS remain, then TS.
            bool const first = i == k;
            if (rem > 2 * TS) {
                if (first) potrf_tile<3 * TS, KN, true, PF>(m, k, i, nc, A, L, il, y, info);
                else potrf_tile<3 * TS, KN, false, PF>(m, k, i, nc, A, L, il, y, info);
                i += 3 * TS;
            } else if (rem > TS) {
                if (first) potrf_tile<2 * TS, KN, true, PF>(m, k, i, nc, A, L, il, y, info);
                else potrf_tile<2 * TS, KN, false, PF>(m, k, i, nc, A, L, il, y, info);
                i += 2 * TS;
            } else {
                if (first) potrf_tile<TS, KN, true, PF>(m, k, i, nc, A, L, il, y, info);
                else potrf_tile<TS, KN, false, PF>(m, k, i, nc, A, L, il, y, info);
                i += TS;
            }
        }
        hook.after(k, nc);
    }
    return info;
}

template <int KN, int TS, class Src, class Addr, class Hook = NoStripHook>
__device__ __forceinline__ int potrf_thread_src(int n, Src const& A, double* L, Addr il, Hook const& hook = Hook{}) {
    return potrf_thread_src_mn<KN, TS>(n, n, A, L, il, hook);
}

template <int KN, int TS, class Addr>
__device__ __forceinline__ int potrf_thread(int n, const double* A, Addr ia, double* L, Addr il) {
    return potrf_thread_src<KN, TS>(n, LoadSrc<Addr>{A, ia}, L, il);
}

constexpr int kRhs = 8;  // right-hand sides per register block of the solves

// Forward solve L*Y = B (Y written to X; X may alias B), register blocks of 4 rows x RB.
// Per element: acc = b_ij; for l < i ascending acc = fma(-l_il, y_lj, acc); y_ij = acc * (1/l_ii)
// (dense/Trsm.hpp:39-52 with the division by l_ii as a multiplication by its reciprocal). The
// right-hand sides are independent, so RB changes no element's operations.
template <int RB = kRhs>
__device__ void trsm_lower_thread(int n, int nrhs, const double* L, int ldl, const double* B, int ldb,
                                  double* X, int ldx) {
    for (int j0 = 0; j0 < nrhs; j0 += RB) {
        int const nj = min(RB, nrhs - j0);
        for (int i0 = 0; i0 < n; i0 += 4) {
            int const ni = min(4, n - i0);
            double acc[4][RB];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < RB; ++c)
                    acc[r][c] = (r < ni && c < nj) ? B[(i0 + r) + (int64_t)(j0 + c) * ldb] : 0.0;
            for (int l = 0; l < i0; ++l) {
                double a[4], x[RB];
#pragma unroll
                for (int r = 0; r < 4; ++r) a[r] = (r < ni) ? L[(i0 + r) + (int64_t)l * ldl] : 0.0;
#pragma unroll
                for (int c = 0; c < RB; ++c) x[c] = (c < nj) ? X[l + (int64_t)(j0 + c) * ldx] : 0.0;
#pragma unroll
                for (int r = 0; r < 4; ++r)
#pragma unroll
                    for (int c = 0; c < RB; ++c) acc[r][c] = fma(-a[r], x[c], acc[r][c]);
            }
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                if (r < ni) {
#pragma unroll
                    for (int q = 0; q < r; ++q) {
                        double const lrq = L[(i0 + r) + (int64_t)(i0 + q) * ldl];
#pragma unroll
                        for (int c = 0; c < RB; ++c) acc[r][c] = fma(-lrq, acc[q][c], acc[r][c]);
                    }
                    double const d = rcp_nr(L[(i0 + r) + (int64_t)(i0 + r) * ldl]);
#pragma unroll
                    for (int c = 0; c < RB; ++c) acc[r][c] *= d;
                }
            }
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < RB; ++c)
                    if (r < ni && c < nj) X[(i0 + r) + (int64_t)(j0 + c) * ldx] = acc[r][c];
        }
    }
}

// Backward solve L^T*X = Y in place in X (trsm<Upper> on trans(L), dense/Trsm.hpp:53-65).
template <int RB = kRhs>
__device__ void trsm_lower_trans_thread(int n, int nrhs, const double* L, int ldl, double* X, int ldx) {
    int const last = ((n - 1) / 4) * 4;
    for (int j0 = 0; j0 < nrhs; j0 += RB) {
        int const nj = min(RB, nrhs - j0);
        for (int i0 = last; i0 >= 0; i0 -= 4) {
            int const ni = min(4, n - i0);
            double acc[4][RB];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < RB; ++c)
                    acc[r][c] = (r < ni && c < nj) ? X[(i0 + r) + (int64_t)(j0 + c) * ldx] : 0.0;
            for (int l = i0 + 4; l < n; ++l) {
                double a[4], x[RB];
#pragma unroll
                for (int r = 0; r < 4; ++r) a[r] = (r < ni) ? L[l + (int64_t)(i0 + r) * ldl] : 0.0;
#pragma unroll
                for (int c = 0; c < RB; ++c) x[c] = (c < nj) ? X[l + (int64_t)(j0 + c) * ldx] : 0.0;
#pragma unroll
                for (int r = 0; r < 4; ++r)
#pragma unroll
                    for (int c = 0; c < RB; ++c) acc[r][c] = fma(-a[r], x[c], acc[r][c]);
            }
#pragma unroll
            for (int r = 3; r >= 0; --r) {
                if (r < ni) {
#pragma unroll
                    for (int q = r + 1; q < 4; ++q) {
                        if (q < ni) {
                            double const lqr = L[(i0 + q) + (int64_t)(i0 + r) * ldl];
#pragma unroll
                            for (int c = 0; c < RB; ++c) acc[r][c] = fma(-lqr, acc[q][c], acc[r][c]);
                        }
                    }
                    double const d = rcp_nr(L[(i0 + r) + (int64_t)(i0 + r) * ldl]);
#pragma unroll
                    for (int c = 0; c < RB; ++c) acc[r][c] *= d;
                }
            }
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < RB; ++c)
                    if (r < ni && c < nj) X[(i0 + r) + (int64_t)(j0 + c) * ldx] = acc[r][c];
        }
    }
}

struct PosvArgs {
    int n, nrhs;
    const double* A; int lda; int64_t sa;
    double* L; int ldl; int64_t sl;
    const double* B; int ldb; int64_t sb;
    double* X; int ldx; int64_t sx;
    int32_t* info;
    int64_t batch;
    int mode;  // 0 potrf, 1 potrf + solves, 2 solves only
    int m = 0; // rows of A and L for potrf (mode 0) of an m x n trapezoid; 0 means m = n
};

template <int THREADS, int MINB, bool PF = false>
__global__ void __launch_bounds__(THREADS, MINB) posv_thread_kernel(PosvArgs p) {
    int64_t const b = (int64_t)blockIdx.x * THREADS + threadIdx.x;
    if (b >= p.batch) return;
    double* L = p.L + b * p.sl;
    int info = 0;
    if (p.mode != 2) {
        int const m = p.m > p.n ? p.m : p.n;
        info = potrf_thread_src_mn<4, 4, LoadSrc<ColAddr>, ColAddr, NoStripHook, PF>(
            m, p.n, LoadSrc<ColAddr>{p.A + b * p.sa, ColAddr{p.lda}}, L, ColAddr{p.ldl});
        if (p.info) p.info[b] = info;
    }
    if (p.mode != 0 && p.nrhs > 0) {
        double* X = p.X + b * p.sx;
        trsm_lower_thread(p.n, p.nrhs, L, p.ldl, p.B + b * p.sb, p.ldb, X, p.ldx);
        trsm_lower_trans_thread(p.n, p.nrhs, L, p.ldl, X, p.ldx);
    }
}

// ---------------------------------------------------------------------------------------------
// Quad mode: four lanes per matrix. One thread per matrix fills the chip only when the batch
// gives every SM sub-partition a few warps (608 sub-partitions: 19,456 matrices a warp each); a
// smaller batch leaves most of them idle while each of its warps runs the whole serial chain.
// Quads spread the same batch over four times as many lanes: at n = 48 with 8 right-hand sides,
// 2,000 matrices take 0.56 ms instead of 1.74 ms, 24,000 take 2.13 ms instead of 2.49 ms; at
// 50,000 the thread kernel is faster again (4.15 against 4.55 ms: a quad repeats the diagonal
// block's square roots and the solves' reciprocals for its 4 lanes, and its solve tiles are
// narrower).
//
// Lane g (0..3) of a quad holds rows k + g + 4 j of strip k (j = j0 .. j0 + KM - 1), so that every
// lane runs the same tile shape and the warp never diverges; the quad's 4 lanes read 4 adjacent
// rows. Each element sees the operations of the thread-per-matrix tiles in the same order: the
// fill, the rank-1 updates over l ascending, then the diagonal block's in-register potrf or the
// trsm against it, and the scaling by the reciprocal square root. DIAG: the strip's first tile
// (j0 = 0), whose row j = 0 on lane g is row k + g of the 4 x 4 diagonal block; the block's
// entries reach the other lanes by shuffles within the quad. The strip's later tiles read them
// from L, as the thread-per-matrix trsm tiles do, and keep y (the reciprocal square roots).
template <int KM, bool DIAG>
__device__ __forceinline__ void quad_tile(int n, int k, int nc, int j0, const double* A, int64_t lda, double* L,
                                          int64_t ldl, int g, unsigned qmask, int qlead, double (&y)[4], int& info) {
    int const row0 = k + g + 4 * j0;
    double acc[KM][4];
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int r = 0; r < KM; ++r) {
            int const row = row0 + 4 * r;
            acc[r][c] = (c < nc && row < n) ? A[row + (int64_t)(k + c) * lda] : 0.0;
        }
    // acc -= L(rows, 0:k) * L(k:k+4, 0:k)^T, the operands of column l + 1 loaded before the fused
    // multiply-adds of column l (the row-0 entries above the diagonal are computed and never used)
    if (k > 0) {
        double a[KM], b[4];
#pragma unroll
        for (int r = 0; r < KM; ++r) a[r] = (row0 + 4 * r < n) ? L[row0 + 4 * r] : 0.0;
#pragma unroll
        for (int c = 0; c < 4; ++c) b[c] = (c < nc) ? L[k + c] : 0.0;
        for (int l = 0; l < k; ++l) {
            int const ln = l + 1 < k ? l + 1 : l;
            double an[KM], bn[4];
#pragma unroll
            for (int r = 0; r < KM; ++r) an[r] = (row0 + 4 * r < n) ? L[row0 + 4 * r + (int64_t)ln * ldl] : 0.0;
#pragma unroll
            for (int c = 0; c < 4; ++c) bn[c] = (c < nc) ? L[(k + c) + (int64_t)ln * ldl] : 0.0;
#pragma unroll
            for (int c = 0; c < 4; ++c)
#pragma unroll
                for (int r = 0; r < KM; ++r) acc[r][c] = fma(-a[r], b[c], acc[r][c]);
#pragma unroll
            for (int r = 0; r < KM; ++r) a[r] = an[r];
#pragma unroll
            for (int c = 0; c < 4; ++c) b[c] = bn[c];
        }
    }
    if constexpr (DIAG) {
        // RegisterMatrix::potrf on the block; row j = 0 takes column c's operations if g >= c
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            if (c < nc) {
#pragma unroll
                for (int j = 0; j < c; ++j) {
                    double const lcj = __shfl_sync(qmask, acc[0][j], qlead + c);
#pragma unroll
                    for (int r = 0; r < KM; ++r)
                        if (r > 0 || g >= c) acc[r][c] = fma(-lcj, acc[r][j], acc[r][c]);
                }
                double const sc = __shfl_sync(qmask, acc[0][c], qlead + c);
                if (!(sc > 0.0) && info == 0) info = k + c + 1;
                y[c] = rsqrt_nr(sc);
#pragma unroll
                for (int r = 0; r < KM; ++r)
                    if (r > 0 || g >= c) acc[r][c] *= y[c];
            }
        }
    } else {
        // RegisterMatrix::trsm against the block
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            if (c < nc) {
#pragma unroll
                for (int j = 0; j < c; ++j) {
                    double const lcj = L[(k + c) + (int64_t)(k + j) * ldl];
#pragma unroll
                    for (int r = 0; r < KM; ++r) acc[r][c] = fma(-lcj, acc[r][j], acc[r][c]);
                }
#pragma unroll
                for (int r = 0; r < KM; ++r) acc[r][c] *= y[c];
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int r = 0; r < KM; ++r) {
            int const row = row0 + 4 * r;
            if (c < nc && row < n && (!DIAG || r > 0 || g >= c)) L[row + (int64_t)(k + c) * ldl] = acc[r][c];
        }
}

// One tile of KM = rows rounded up to an even count (at most kQuadRows).
constexpr int kQuadRows = 12;

template <bool DIAG>
__device__ __forceinline__ void quad_tile_rows(int rows, int n, int k, int nc, int j0, const double* A,
                                               int64_t lda, double* L, int64_t ldl, int g, unsigned qmask,
                                               int qlead, double (&y)[4], int& info) {
    switch ((rows + 1) / 2) {
        case 1: quad_tile<2, DIAG>(n, k, nc, j0, A, lda, L, ldl, g, qmask, qlead, y, info); break;
        case 2: quad_tile<4, DIAG>(n, k, nc, j0, A, lda, L, ldl, g, qmask, qlead, y, info); break;
        case 3: quad_tile<6, DIAG>(n, k, nc, j0, A, lda, L, ldl, g, qmask, qlead, y, info); break;
        case 4: quad_tile<8, DIAG>(n, k, nc, j0, A, lda, L, ldl, g, qmask, qlead, y, info); break;
        case 5: quad_tile<10, DIAG>(n, k, nc, j0, A, lda, L, ldl, g, qmask, qlead, y, info); break;
        default: quad_tile<12, DIAG>(n, k, nc, j0, A, lda, L, ldl, g, qmask, qlead, y, info); break;
    }
}

// Left-looking Cholesky of one n x n matrix by a quad (strips of 4 columns, as potrf_thread). Out
// of line: inlined into the kernel beside the solves, it spilled 460 bytes a thread.
__device__ __noinline__ int potrf_quad(int n, const double* A, int64_t lda, double* L, int64_t ldl, int g,
                                       unsigned qmask, int qlead) {
    int info = 0;
    for (int k = 0; k < n; k += 4) {
        int const nc = min(4, n - k);
        int const rows = (n - k + 3) / 4;  // rows of the strip per lane
        double y[4];
        quad_tile_rows<true>(min(rows, kQuadRows), n, k, nc, 0, A, lda, L, ldl, g, qmask, qlead, y, info);
        if (rows > kQuadRows) {
            __syncwarp(qmask);  // the diagonal block, stored by its rows' lanes, is read below
            for (int j0 = kQuadRows; j0 < rows; j0 += kQuadRows)
                quad_tile_rows<false>(min(rows - j0, kQuadRows), n, k, nc, j0, A, lda, L, ldl, g, qmask, qlead, y,
                                      info);
        }
        __syncwarp(qmask);  // the strip's columns of L, stored by all four lanes, are read next
    }
    return info;
}

// The quad's solves: lane g takes right-hand sides g*q .. g*q + q - 1 (q = ceil(nrhs / 4)).
__device__ __forceinline__ void potrs_quad(int n, int nrhs, const double* L, int ldl, const double* B, int ldb,
                                           double* X, int ldx, int g) {
    int const q = (nrhs + 3) / 4, j0 = g * q, nj = min(q, nrhs - j0);
    if (nj <= 0) return;
    const double* Bg = B + (int64_t)j0 * ldb;
    double* Xg = X + (int64_t)j0 * ldx;
    if (q <= 1) {
        trsm_lower_thread<1>(n, nj, L, ldl, Bg, ldb, Xg, ldx);
        trsm_lower_trans_thread<1>(n, nj, L, ldl, Xg, ldx);
    } else if (q <= 2) {
        trsm_lower_thread<2>(n, nj, L, ldl, Bg, ldb, Xg, ldx);
        trsm_lower_trans_thread<2>(n, nj, L, ldl, Xg, ldx);
    } else if (q <= 4) {
        trsm_lower_thread<4>(n, nj, L, ldl, Bg, ldb, Xg, ldx);
        trsm_lower_trans_thread<4>(n, nj, L, ldl, Xg, ldx);
    } else {
        trsm_lower_thread<8>(n, nj, L, ldl, Bg, ldb, Xg, ldx);
        trsm_lower_trans_thread<8>(n, nj, L, ldl, Xg, ldx);
    }
}

// Square matrices only (p.m == 0 or p.m == p.n); 8 matrices per 32-thread CTA.
__global__ void __launch_bounds__(32, 12) posv_quad_kernel(PosvArgs p) {
    int const lane = threadIdx.x;
    int64_t const b = (int64_t)blockIdx.x * 8 + (lane >> 2);
    if (b >= p.batch) return;  // the whole quad: b depends on lane / 4 only
    int const g = lane & 3, qlead = lane & ~3;
    unsigned const qmask = 0xFu << qlead;
    double* L = p.L + b * p.sl;
    if (p.mode != 2) {
        int const info = potrf_quad(p.n, p.A + b * p.sa, p.lda, L, p.ldl, g, qmask, qlead);
        if (p.info && g == 0) p.info[b] = info;
    }
    if (p.mode != 0 && p.nrhs > 0)
        potrs_quad(p.n, p.nrhs, L, p.ldl, p.B + b * p.sb, p.ldb, p.X + b * p.sx, p.ldx, g);
}

// Cholesky solve whose inputs and outputs may live in host memory the GPU addresses directly
// (pinned, or any allocation on hardware-coherent systems). A and B are read once each, in place,
// by the thread that owns the instance; the factorisation and the solves run on working copies in
// the device workspaces p.L / p.X (ld = n), which they re-read. The warp copies its 32 instances'
// final L columns out to the caller's Lh after every strip of 4 columns (lanes over rows, so the
// host sees whole-line writes instead of one 8-byte store per thread, spread over the
// factorisation), and X at the end. On GB300 these reads and writes cross NVLink-C2C while the
// binary64 pipe computes.
struct MirrorOut {
    double* Lh; int ldlh; int64_t slh;
    double* Xh; int ldxh; int64_t sxh;
};

// Copies columns j0 .. j0+nc-1 (nc <= 4) of `cnt` consecutive instances from S to D, rows from j
// (lower) or from 0, one warp, lanes over rows. For n <= 64 the loads of 4 instances (up to 32 per
// lane) are issued together before their stores, so that a copy from host memory pays the link's
// latency once per 4 instances.
__device__ __forceinline__ void warp_stage_cols(int n, int j0, int nc, bool lower, int cnt, const double* S, int lds,
                                                int64_t ss, double* D, int ldd, int64_t sd, int lane) {
    if (n <= 64) {
        for (int m0 = 0; m0 < cnt; m0 += 4) {
            double v[4][4][2];
#pragma unroll
            for (int mm = 0; mm < 4; ++mm)
#pragma unroll
                for (int c = 0; c < 4; ++c)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        int const m = m0 + mm, j = j0 + c, i = (lower ? j : 0) + lane + 32 * h;
                        v[mm][c][h] = (m < cnt && c < nc && i < n) ? S[m * ss + i + (int64_t)j * lds] : 0.0;
                    }
#pragma unroll
            for (int mm = 0; mm < 4; ++mm)
#pragma unroll
                for (int c = 0; c < 4; ++c)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        int const m = m0 + mm, j = j0 + c, i = (lower ? j : 0) + lane + 32 * h;
                        if (m < cnt && c < nc && i < n) D[m * sd + i + (int64_t)j * ldd] = v[mm][c][h];
                    }
        }
    } else {
        for (int m = 0; m < cnt; ++m)
            for (int j = j0; j < j0 + nc; ++j)
                for (int i = (lower ? j : 0) + lane; i < n; i += 32)
                    D[m * sd + i + (int64_t)j * ldd] = S[m * ss + i + (int64_t)j * lds];
    }
}

// Copies rows j .. n-1 (lower) or 0 .. n-1 of columns j0 .. j0+nc-1 (any nc) of `cnt` consecutive
// instances, one warp, through warp_stage_cols' batched loads: a copy to host memory then waits on
// the source's latency once per batch instead of once per element.
__device__ __forceinline__ void warp_copy_cols(int n, int j0, int nc, bool lower, int cnt, const double* W, int ldw,
                                               int64_t sw, double* H, int ldh, int64_t sh, int lane) {
    for (int j = j0; j < j0 + nc; j += 4)
        warp_stage_cols(n, j, min(4, j0 + nc - j), lower, cnt, W, ldw, sw, H, ldh, sh, lane);
}

// Strip hooks of the mirror kernel (a full warp of 32 instances): before strip k the warp stages
// the strip's columns of A from host memory into the device working copy (where the tiles then
// read them, the factorisation running in place), after it the finished columns of L go back.
struct MirrorHook {
    int n, lane;
    const double* Ah; int ldah; int64_t sah;
    double* W; int ldw; int64_t sw;
    double* Lh; int ldlh; int64_t slh;
    __device__ __forceinline__ void before(int k, int nc) const {
        __syncwarp();
        warp_stage_cols(n, k, nc, true, 32, Ah, ldah, sah, W, ldw, sw, lane);
        __syncwarp();
    }
    __device__ __forceinline__ void after(int k, int nc) const {
        __syncwarp();
        warp_copy_cols(n, k, nc, true, 32, W, ldw, sw, Lh, ldlh, slh, lane);
    }
};

__global__ void __launch_bounds__(32, 12) posv_mirror_kernel(PosvArgs p, MirrorOut o) {
    int64_t const b0 = (int64_t)blockIdx.x * 32;
    int const lane = threadIdx.x;
    int64_t const b = b0 + lane;
    int const n = p.n;
    bool const full = b0 + 32 <= p.batch;  // warp-uniform
    int const cnt = full ? 32 : (int)(p.batch - b0);
    if (full) {  // A arrives and L leaves strip by strip, in whole-warp copies
        double* L = p.L + b * p.sl;
        MirrorHook const hook{n,     lane,  p.A + b0 * p.sa,  p.lda,  p.sa,  p.L + b0 * p.sl,
                              p.ldl, p.sl,  o.Lh + b0 * o.slh, o.ldlh, o.slh};
        int const info = potrf_thread_src<4, 4>(n, LoadSrc<ColAddr>{L, ColAddr{p.ldl}}, L, ColAddr{p.ldl}, hook);
        if (p.info) p.info[b] = info;
        if (p.nrhs > 0) {  // B staged into the working copy of X, then solved in place
            __syncwarp();
            for (int j0 = 0; j0 < p.nrhs; j0 += 4)
                warp_stage_cols(n, j0, min(4, p.nrhs - j0), false, 32, p.B + b0 * p.sb, p.ldb, p.sb, p.X + b0 * p.sx,
                                p.ldx, p.sx, lane);
            __syncwarp();
            double* X = p.X + b * p.sx;
            trsm_lower_thread(n, p.nrhs, L, p.ldl, X, p.ldx, X, p.ldx);
            trsm_lower_trans_thread(n, p.nrhs, L, p.ldl, X, p.ldx);
        }
    } else if (b < p.batch) {
        double* L = p.L + b * p.sl;
        int const info = potrf_thread<4, 4>(n, p.A + b * p.sa, ColAddr{p.lda}, L, ColAddr{p.ldl});
        if (p.info) p.info[b] = info;
        if (p.nrhs > 0) {
            double* X = p.X + b * p.sx;
            trsm_lower_thread(n, p.nrhs, L, p.ldl, p.B + b * p.sb, p.ldb, X, p.ldx);
            trsm_lower_trans_thread(n, p.nrhs, L, p.ldl, X, p.ldx);
        }
    }
    __syncwarp();
    if (!full)
        warp_copy_cols(n, 0, n, true, cnt, p.L + b0 * p.sl, p.ldl, p.sl, o.Lh + b0 * o.slh, o.ldlh, o.slh, lane);
    if (p.nrhs > 0)
        warp_copy_cols(n, 0, p.nrhs, false, cnt, p.X + b0 * p.sx, p.ldx, p.sx, o.Xh + b0 * o.sxh, o.ldxh, o.sxh, lane);
}

// Ragged potrf over descriptors whose matrices all have the layout `layout` (column-major, or
// panel with panel height PS); one thread per matrix.
template <int KN, int TS, class Addr>
__global__ void __launch_bounds__(32, 12) potrf_desc_kernel(const blastgpu_potrf_desc* desc, int64_t count,
                                                          int layout, int ps, int32_t* info) {
    int64_t const b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= count) return;
    blastgpu_potrf_desc const d = desc[b];
    int const m = d.A.rows, n = d.A.cols;  // m >= n: BLAST's trapezoidal potrf
    bool const ok = d.A.layout == layout && d.L.layout == layout && n <= m && d.L.rows == m &&
                    d.L.cols == n && (layout == BLASTGPU_COL_MAJOR || (d.A.ps == ps && d.L.ps == ps));
    if (!ok) {
        if (info) info[b] = -1;
        return;
    }
    Addr const ia{d.A.ld}, il{d.L.ld};
    int const r = potrf_thread_src_mn<KN, TS>(m, n, LoadSrc<Addr>{d.A.data, ia}, d.L.data, il);
    if (info) info[b] = r;
}

// D = chol(beta*C + alpha*op(A)*op(A)^T), lower, one thread per instance: syrkLower's values are
// formed inside the factorisation's register tiles and never stored.
struct SyrkPotrfArgs {
    int n, k, trans;
    double alpha, beta;
    const double* A; int lda; int64_t sa;
    const double* C; int ldc; int64_t sc;
    double* D; int ldd; int64_t sd;
    int32_t* info;
    int64_t batch;
};

template <bool ALPHA1>
__global__ void __launch_bounds__(32, 12) syrk_potrf_thread_kernel(SyrkPotrfArgs p) {
    int64_t const b = (int64_t)blockIdx.x * 32 + threadIdx.x;
    if (b >= p.batch) return;
    SyrkSrc<ALPHA1> const src{p.A + b * p.sa, p.lda, p.k, p.trans != 0, p.alpha, p.beta, p.C + b * p.sc, p.ldc};
    int const info = potrf_thread_src<4, 4>(p.n, src, p.D + b * p.sd, ColAddr{p.ldd});
    if (p.info) p.info[b] = info;
}

// Quads ("posv.quad.n<bin>" = T) when the batch holds fewer than T / 100 full warps per SM
// sub-partition. Defaults from measurements on GB300 (n = 16: quads win at 8,000 matrices and lose
// at 16,000; n = 32, 48 and 64: they win up to 24,000 and lose at 50,000; n = 96 and 128: 3.3-3.7x
// at 2,000 and 8,000, 1.6x at 16,000); 0 turns them off.
bool posv_quad_wanted(PosvArgs const& p) {
    if (p.m != 0 && p.m != p.n) return false;
    int const def = p.n <= 8 ? 0 : p.n <= 16 ? 50 : 150;
    int const t = tune_get_bin("posv.quad", p.n, def);
    if (t <= 0) return false;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return false;
    return p.batch * 100 < (int64_t)t * 32 * 4 * sms;
}

int launch_posv(PosvArgs const& p, cudaStream_t stream) {
    if (p.batch == 0 || p.n == 0) {
        if (p.info && p.batch > 0 && p.mode != 2) {
            cudaError_t const e = cudaMemsetAsync(p.info, 0, sizeof(int32_t) * p.batch, stream);
            if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
        }
        return BLASTGPU_SUCCESS;
    }
    // Square matrices from "posv.cta_min_n" (default 65) on go to the CTA-per-matrix kernels: one
    // thread per matrix would need more registers than a thread has, and a batch of them leaves
    // most of the chip idle.
    if ((p.m == 0 || p.m == p.n) && p.n >= tune_get("posv.cta_min_n", 65) && p.n <= 512)
        return launch_posv_cta_strided(p.n, p.nrhs, p.mode == 2 ? nullptr : p.A, p.lda, p.sa, p.L, p.ldl, p.sl,
                                       p.B, p.ldb, p.sb, p.X, p.ldx, p.sx, p.mode == 2 ? nullptr : p.info,
                                       p.batch, stream);
    // "posv.variant": CTA size and the occupancy the register allocation is bounded for (4: as 3,
    // with one column of load look-ahead in the factorisation's tile updates).
    // Measured on GB300 at n = 48 (50,000 instances): 32 threads x 12 CTAs/SM is fastest
    // (4.29 ms vs 4.56 ms for 64 x 6 and 5.30 ms for 64 x 1); it lets the block scheduler even
    // out the per-SM load one warp at a time.
    if (posv_quad_wanted(p)) {
        int64_t const qblocks = (p.batch + 7) / 8;
        if (qblocks > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
        posv_quad_kernel<<<(unsigned)qblocks, 32, 0, stream>>>(p);
        return check_launch();
    }
    int const variant = tune_get_bin("posv.variant", p.n, 3);
    int const threads = variant == 2 ? 128 : (variant == 3 || variant == 4) ? 32 : 64;
    int64_t const blocks = (p.batch + threads - 1) / threads;
    if (blocks > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    switch (variant) {
        case 0: posv_thread_kernel<64, 1><<<(unsigned)blocks, 64, 0, stream>>>(p); break;
        case 2: posv_thread_kernel<128, 3><<<(unsigned)blocks, 128, 0, stream>>>(p); break;
        case 3: posv_thread_kernel<32, 12><<<(unsigned)blocks, 32, 0, stream>>>(p); break;
        case 4: posv_thread_kernel<32, 12, true><<<(unsigned)blocks, 32, 0, stream>>>(p); break;
        default: posv_thread_kernel<64, 6><<<(unsigned)blocks, 64, 0, stream>>>(p); break;
    }
    return check_launch();
}

}  // namespace
}  // namespace blastgpu

using namespace blastgpu;

extern "C" {

int blastgpu_dpotrf_strided(int n, const double* A, int lda, int64_t stride_a, double* L, int ldl,
                            int64_t stride_l, int32_t* info, int64_t batch, blastgpu_stream_t stream) {
    if (n < 0) return -1;
    if (n > 0 && !A) return -2;
    if (lda < (n > 0 ? n : 1)) return -3;
    if (n > 0 && !L) return -5;
    if (ldl < (n > 0 ? n : 1)) return -6;
    if (batch < 0) return -9;
    PosvArgs p{n, 0, A, lda, stride_a, L, ldl, stride_l, nullptr, 1, 0, nullptr, 1, 0, info, batch, 0};
    return launch_posv(p, as_cuda(stream));
}

int blastgpu_dpotrf_mn_strided(int m, int n, const double* A, int lda, int64_t stride_a, double* L, int ldl,
                               int64_t stride_l, int32_t* info, int64_t batch, blastgpu_stream_t stream) {
    if (m < 0) return -1;
    if (n < 0 || n > m) return -2;
    if (m > 0 && n > 0 && !A) return -3;
    if (lda < (m > 0 ? m : 1)) return -4;
    if (m > 0 && n > 0 && !L) return -6;
    if (ldl < (m > 0 ? m : 1)) return -7;
    if (batch < 0) return -10;
    PosvArgs p{n, 0, A, lda, stride_a, L, ldl, stride_l, nullptr, 1, 0, nullptr, 1, 0, info, batch, 0, m};
    return launch_posv(p, as_cuda(stream));
}

int blastgpu_dpotrf_batched(const blastgpu_potrf_desc* desc, int64_t batch, int layout, int ps,
                            int32_t* info, blastgpu_stream_t stream) {
    if (batch < 0) return -2;
    if (layout != BLASTGPU_COL_MAJOR && layout != BLASTGPU_PANEL) return -3;
    if (layout == BLASTGPU_PANEL && ps != 2 && ps != 4) return -4;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (!desc) return -1;
    int64_t const blocks = (batch + 31) / 32;
    if (blocks > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    cudaStream_t const s = as_cuda(stream);
    if (layout == BLASTGPU_COL_MAJOR)
        potrf_desc_kernel<4, 4, ColAddr><<<(unsigned)blocks, 32, 0, s>>>(desc, batch, layout, ps, info);
    else if (ps == 4)  // AVX2 panels: SS = 4, 16 registers -> strips of min((16-4)/3, 4) = 4
        potrf_desc_kernel<4, 4, PanelAddr<4>><<<(unsigned)blocks, 32, 0, s>>>(desc, batch, layout, ps, info);
    else               // NEON panels: SS = 2, 32 registers -> strips of min((32-4)/3, 2) = 2
        potrf_desc_kernel<2, 2, PanelAddr<2>><<<(unsigned)blocks, 32, 0, s>>>(desc, batch, layout, ps, info);
    return check_launch();
}

int blastgpu_dposv_strided(int n, int nrhs, const double* A, int lda, int64_t stride_a, double* L,
                           int ldl, int64_t stride_l, const double* B, int ldb, int64_t stride_b,
                           double* X, int ldx, int64_t stride_x, int32_t* info, int64_t batch,
                           blastgpu_stream_t stream) {
    if (n < 0) return -1;
    if (nrhs < 0) return -2;
    if (n > 0 && !A) return -3;
    if (lda < (n > 0 ? n : 1)) return -4;
    if (n > 0 && !L) return -6;
    if (ldl < (n > 0 ? n : 1)) return -7;
    if (n > 0 && nrhs > 0 && !B) return -9;
    if (ldb < (n > 0 ? n : 1)) return -10;
    if (n > 0 && nrhs > 0 && !X) return -12;
    if (ldx < (n > 0 ? n : 1)) return -13;
    if (batch < 0) return -16;
    PosvArgs p{n, nrhs, A, lda, stride_a, L, ldl, stride_l, B, ldb, stride_b, X, ldx, stride_x, info, batch, 1};
    return launch_posv(p, as_cuda(stream));
}

int blastgpu_dpotrs_strided(int n, int nrhs, const double* L, int ldl, int64_t stride_l,
                            const double* B, int ldb, int64_t stride_b, double* X, int ldx,
                            int64_t stride_x, int64_t batch, blastgpu_stream_t stream) {
    if (n < 0) return -1;
    if (nrhs < 0) return -2;
    if (n > 0 && !L) return -3;
    if (ldl < (n > 0 ? n : 1)) return -4;
    if (n > 0 && nrhs > 0 && !B) return -6;
    if (ldb < (n > 0 ? n : 1)) return -7;
    if (n > 0 && nrhs > 0 && !X) return -9;
    if (ldx < (n > 0 ? n : 1)) return -10;
    if (batch < 0) return -12;
    if (nrhs == 0) return BLASTGPU_SUCCESS;
    PosvArgs p{n, nrhs, nullptr, 1, 0, const_cast<double*>(L), ldl, stride_l, B, ldb, stride_b, X, ldx,
               stride_x, nullptr, batch, 2};
    return launch_posv(p, as_cuda(stream));
}

int blastgpu_dposv_mirror_strided(int n, int nrhs, const double* A, int lda, int64_t stride_a,
                                  const double* B, int ldb, int64_t stride_b, double* L, int ldl,
                                  int64_t stride_l, double* X, int ldx, int64_t stride_x, double* L_work,
                                  double* X_work, int32_t* info, int64_t batch, blastgpu_stream_t stream) {
    if (n < 0) return -1;
    if (nrhs < 0) return -2;
    if (n > 0 && !A) return -3;
    if (lda < (n > 0 ? n : 1)) return -4;
    if (n > 0 && nrhs > 0 && !B) return -6;
    if (ldb < (n > 0 ? n : 1)) return -7;
    if (n > 0 && !L) return -9;
    if (ldl < (n > 0 ? n : 1)) return -10;
    if (n > 0 && nrhs > 0 && !X) return -12;
    if (ldx < (n > 0 ? n : 1)) return -13;
    if (n > 0 && !L_work) return -15;
    if (n > 0 && nrhs > 0 && !X_work) return -16;
    if (batch < 0) return -18;
    cudaStream_t const s = as_cuda(stream);
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (n == 0) {
        if (info) {
            cudaError_t const e = cudaMemsetAsync(info, 0, sizeof(int32_t) * batch, s);
            if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
        }
        return BLASTGPU_SUCCESS;
    }
    int64_t const blocks = (batch + 31) / 32;
    if (blocks > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    PosvArgs const p{n, nrhs, A, lda, stride_a, L_work, n, (int64_t)n * n, B, ldb, stride_b, X_work, n,
                     (int64_t)n * nrhs, info, batch, 1};
    MirrorOut const o{L, ldl, stride_l, X, ldx, stride_x};
    posv_mirror_kernel<<<(unsigned)blocks, 32, 0, s>>>(p, o);
    return check_launch();
}

int blastgpu_dsyrk_potrf_strided(int n, int k, int trans_a, double alpha, const double* A, int lda,
                                 int64_t stride_a, double beta, const double* C, int ldc, int64_t stride_c,
                                 double* D, int ldd, int64_t stride_d, int32_t* info, int64_t batch,
                                 blastgpu_stream_t stream) {
    if (n < 0) return -1;
    if (k < 0) return -2;
    if (trans_a != 0 && trans_a != 1) return -3;
    int const arows = trans_a ? k : n;
    if (n > 0 && k > 0 && !A) return -5;
    if (lda < (arows > 0 ? arows : 1)) return -6;
    if (n > 0 && !C) return -9;
    if (ldc < (n > 0 ? n : 1)) return -10;
    if (n > 0 && !D) return -12;
    if (ldd < (n > 0 ? n : 1)) return -13;
    if (batch < 0) return -16;
    cudaStream_t const s = as_cuda(stream);
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (n == 0) {
        if (info) {
            cudaError_t const e = cudaMemsetAsync(info, 0, sizeof(int32_t) * batch, s);
            if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
        }
        return BLASTGPU_SUCCESS;
    }
    // Two implementations with the same bits: syrkLower's warp-per-instance kernel followed by the
    // thread-per-matrix potrf, or the fused thread-per-matrix kernel, which never stores the sum
    // but runs the syrk part at thread-per-matrix granularity (1,563 warps for 50,000 instances,
    // unevenly spread over the 608 sub-partitions). Measured on GB300 at n = 60, k = 30, alpha = 1:
    // 8.85 ms for the pair vs 9.42 ms fused at 50,000 instances, and the pair is further ahead at
    // smaller batches, so the pair is the default; "syrk_potrf.fused_min_batch" selects the fused
    // kernel from that batch size on.
    // Sizes that the potrf entry point sends to the CTA kernels always take the pair, so that the
    // result stays equal to syrkLower followed by potrf bit for bit.
    if (batch < tune_get("syrk_potrf.fused_min_batch", 0x7fffffff) || n >= tune_get("posv.cta_min_n", 65)) {
        int st = launch_syrk_lower(n, k, trans_a, alpha, A, lda, stride_a, beta, C, ldc, stride_c, D, ldd,
                                   stride_d, batch, s);
        if (st != BLASTGPU_SUCCESS) return st;
        PosvArgs const q{n, 0, D, ldd, stride_d, D, ldd, stride_d, nullptr, 1, 0, nullptr, 1, 0, info, batch, 0};
        return launch_posv(q, s);
    }
    int64_t const blocks = (batch + 31) / 32;
    if (blocks > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    SyrkPotrfArgs const p{n, k, trans_a, alpha, beta, A, lda, stride_a, C, ldc, stride_c, D, ldd, stride_d, info,
                          batch};
    if (alpha == 1.0)
        syrk_potrf_thread_kernel<true><<<(unsigned)blocks, 32, 0, s>>>(p);
    else
        syrk_potrf_thread_kernel<false><<<(unsigned)blocks, 32, 0, s>>>(p);
    return check_launch();
}

}  // extern "C"

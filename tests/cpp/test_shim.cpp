// Exercises include/blastgpu/blast.hpp (BLAST's names over the C ABI) from plain C++ host code:
// gemm with a trans() view, potrf, trsm<Lower/Upper>, getrf, size and variant errors.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <stdexcept>
#include <vector>

#include <cuda_runtime.h>

#include "blastgpu/blast.hpp"

#define CHECK(c) do { if (!(c)) { std::printf("FAILED %s:%d %s\n", __FILE__, __LINE__, #c); std::exit(1); } } while (0)

static double* upload(std::vector<double> const& h) {
    double* d = nullptr;
    CHECK(cudaMalloc(&d, h.size() * sizeof(double)) == cudaSuccess);
    CHECK(cudaMemcpy(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess);
    return d;
}

static std::vector<double> download(double const* d, size_t n) {
    std::vector<double> h(n);
    CHECK(cudaMemcpy(h.data(), d, n * sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess);
    return h;
}

int main() {
    std::mt19937 gen(42);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    int const n = 24, batch = 5;
    size_t const nn = (size_t)n * n;
    std::vector<double> A(nn * batch), B(nn * batch), C(nn * batch);
    for (auto* v : {&A, &B, &C}) for (auto& x : *v) x = U(gen);
    double *dA = upload(A), *dB = upload(B), *dC = upload(C), *dD = upload(C);
    using blastgpu::Batch;
    auto bt = [&](double* p) { return Batch{blastgpu::matrix(p, n, n), (std::int64_t)nn, batch}; };

    // D = A * trans(B) + C  (BLAST's benchmark form, bench/blast/math/dense/StaticGemm.cpp)
    blastgpu::gemm(1.0, bt(dA), blastgpu::trans(bt(dB)), 1.0, bt(dC), bt(dD));
    CHECK(cudaDeviceSynchronize() == cudaSuccess);
    auto D = download(dD, nn * batch);
    for (int b = 0; b < batch; ++b)
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                double acc = 0.0;
                for (int k = 0; k < n; ++k) acc = std::fma(A[b * nn + i + k * n], B[b * nn + j + k * n], acc);
                double const ref = std::fma(1.0, C[b * nn + i + j * n], acc * 1.0);
                CHECK(D[b * nn + i + j * n] == ref);  // same order of operations: bit-identical
            }

    // potrf on SPD matrices S = A A^T + n I, then trsm<Lower> and trsm<Upper> on trans(L)
    std::vector<double> S(nn * batch, 0.0);
    for (int b = 0; b < batch; ++b)
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                double s = i == j ? n : 0.0;
                for (int k = 0; k < n; ++k) s += A[b * nn + i + k * n] * A[b * nn + j + k * n];
                S[b * nn + i + j * n] = s;
            }
    double *dS = upload(S), *dL = upload(std::vector<double>(nn * batch, 0.0));
    blastgpu::potrf(bt(dS), bt(dL));
    std::vector<double> rhs(n * batch);
    for (auto& x : rhs) x = U(gen);
    double* dX = upload(rhs);
    Batch xb{blastgpu::matrix(dX, n, 1), n, batch};
    blastgpu::trsm<blastgpu::UpLo::Lower, false>(bt(dL), xb, xb);
    blastgpu::trsm<blastgpu::UpLo::Upper, false>(blastgpu::trans(bt(dL)), xb, xb);
    CHECK(cudaDeviceSynchronize() == cudaSuccess);
    auto X = download(dX, n * batch);
    for (int b = 0; b < batch; ++b) {
        double rmax = 0.0;
        for (int i = 0; i < n; ++i) {
            double r = rhs[b * n + i];
            for (int j = 0; j < n; ++j) r -= S[b * nn + i + j * n] * X[b * n + j];
            rmax = std::fmax(rmax, std::fabs(r));
        }
        CHECK(rmax < 1e-12 * n * n);
    }

    // getrf on a singular matrix: BLAST's exception through check_singular
    std::vector<double> Z(nn, 0.0);
    double* dZ = upload(Z);
    std::int32_t *dpiv = nullptr, *dinfo = nullptr;
    CHECK(cudaMalloc(&dpiv, n * sizeof(std::int32_t)) == cudaSuccess);
    CHECK(cudaMalloc(&dinfo, sizeof(std::int32_t)) == cudaSuccess);
    blastgpu::getrf(blastgpu::batch(blastgpu::matrix(dZ, n, n)), dpiv, n, dinfo);
    std::int32_t info = -1;
    CHECK(cudaMemcpy(&info, dinfo, sizeof(info), cudaMemcpyDeviceToHost) == cudaSuccess);
    bool threw = false;
    try { blastgpu::check_singular(&info, 1); } catch (std::invalid_argument const&) { threw = true; }
    CHECK(threw && info == 1);

    // ger, trsvLeftLower and iamax on one instance: B = A + 0.5*x*y^T, solve tril(B + n I) x = b
    {
        std::vector<double> x(n), y(n), b(n);
        for (int i = 0; i < n; ++i) { x[i] = U(gen); y[i] = U(gen); b[i] = U(gen); }
        double *dx = upload(x), *dy = upload(y), *db = upload(b), *dB2 = upload(A);
        blastgpu::ger(0.5, blastgpu::batch(blastgpu::vector(dx, n)), blastgpu::batch(blastgpu::vector(dy, n)),
                      blastgpu::batch(blastgpu::matrix(dA, n, n)), blastgpu::batch(blastgpu::matrix(dB2, n, n)));
        auto G = download(dB2, nn);
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) CHECK(G[i + j * n] == std::fma(0.5 * x[i], y[j], A[i + j * n]));
        for (int i = 0; i < n; ++i) G[i + i * n] += n;
        double* dG = upload(G);
        blastgpu::trsvLeftLower(blastgpu::batch(blastgpu::matrix(dG, n, n)), blastgpu::batch(blastgpu::vector(db, n)),
                                blastgpu::batch(blastgpu::vector(dx, n)));
        auto xs = download(dx, n);
        for (int i = 0; i < n; ++i) {
            double r = b[i];
            for (int j = 0; j <= i; ++j) r -= G[i + j * n] * xs[j];
            CHECK(std::fabs(r) < 1e-12 * n);
        }
        std::int32_t* didx = nullptr;
        CHECK(cudaMalloc(&didx, sizeof(std::int32_t)) == cudaSuccess);
        blastgpu::iamax(blastgpu::batch(blastgpu::vector(db, n)), didx);
        std::int32_t idx = -1;
        CHECK(cudaMemcpy(&idx, didx, sizeof(idx), cudaMemcpyDeviceToHost) == cudaSuccess);
        int want = 0;
        for (int i = 1; i < n; ++i) if (std::fabs(b[i]) > std::fabs(b[want])) want = i;
        CHECK(idx == want);
    }

    // BLAST's matrix types on the device: StaticMatrix / DynamicMatrix (column-major) and
    // StaticPanelMatrix / DynamicPanelMatrix (panels of 4 rows), all through the descriptor calls
    {
        blastgpu::DescriptorArena arena;
        int const m = 13;
        std::vector<double> G(m * m), Sm(m * m);
        for (auto& v : G) v = U(gen);
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < m; ++j) {
                double s = i == j ? m : 0.0;
                for (int k = 0; k < m; ++k) s += G[i + k * m] * G[j + k * m];
                Sm[i + j * m] = s;
            }
        blastgpu::StaticMatrix<13, 13> sA;
        blastgpu::DynamicMatrix dL(m, m);
        blastgpu::StaticPanelMatrix<13, 13, 4> pA;
        blastgpu::DynamicPanelMatrix pL(m, m, 4);
        CHECK(sA.rows() == 13 && pA.spacing() == 52 && pL.spacing() == 52 && dL.spacing() == 13);
        blastgpu::copy_to_device(sA, Sm.data());
        blastgpu::copy_to_device(pA, Sm.data());
        // dense and panel potrf give the same factor to rounding (both follow BLAST's algorithm)
        blastgpu::potrf(blastgpu::Matrix(sA), blastgpu::Matrix(dL), nullptr, arena);
        blastgpu::potrf(blastgpu::Matrix(pA), blastgpu::Matrix(pL), nullptr, arena);
        CHECK(cudaDeviceSynchronize() == cudaSuccess);
        std::vector<double> L1(m * m), L2(m * m);
        blastgpu::copy_to_host(dL, L1.data());
        blastgpu::copy_to_host(pL, L2.data());
        for (int j = 0; j < m; ++j)
            for (int i = j; i < m; ++i) {
                double r = Sm[i + j * m];
                for (int k = 0; k <= j; ++k) r -= L1[i + k * m] * L1[j + k * m];
                CHECK(std::fabs(r) < 1e-11 * m);
                CHECK(std::fabs(L1[i + j * m] - L2[i + j * m]) < 1e-13 * m);
            }
        // panel gemm: D = L * trans(L) with L in panel storage, trans(L) the row-major view of dL
        // (whose upper triangle is zero from its zero-filled construction)
        blastgpu::DynamicMatrix dD(m, m), dZ(m, m);
        blastgpu::DynamicPanelMatrix pLt(m, m, 4);
        std::vector<double> Lsym(m * m, 0.0);
        for (int j = 0; j < m; ++j)
            for (int i = j; i < m; ++i) Lsym[i + j * m] = L2[i + j * m];
        blastgpu::copy_to_device(pLt, Lsym.data());
        blastgpu::gemm(1.0, blastgpu::Matrix(pLt), blastgpu::trans(blastgpu::Matrix(dL)), 0.0, blastgpu::Matrix(dZ),
                       blastgpu::Matrix(dD), arena);
        CHECK(cudaDeviceSynchronize() == cudaSuccess);
        std::vector<double> Dh(m * m);
        blastgpu::copy_to_host(dD, Dh.data());
        for (int i = 0; i < m * m; ++i) CHECK(std::fabs(Dh[i] - Sm[i]) < 1e-11 * m);

        // row() and column() views: swap row 2 of a panel matrix with column 5 of a dense one
        blastgpu::DynamicMatrix dV(m, m);
        std::vector<double> V(m * m), P(m * m);
        for (auto& v : V) v = U(gen);
        for (auto& v : P) v = U(gen);
        blastgpu::DynamicPanelMatrix pP(m, m, 4);
        blastgpu::copy_to_device(dV, V.data());
        blastgpu::copy_to_device(pP, P.data());
        blastgpu::Matrix const r2 = blastgpu::row(blastgpu::Matrix(pP), 2), c5 = blastgpu::column(blastgpu::Matrix(dV), 5);
        CHECK(r2.rows == 1 && r2.cols == m && c5.rows == m && c5.cols == 1);
        std::vector<blastgpu_swap_desc> sds{blastgpu_swap_desc{blastgpu::to_mat(r2), blastgpu::to_mat(c5)}};
        CHECK(blastgpu_dswap_batched(arena.upload(sds, nullptr), 1, nullptr, nullptr) == BLASTGPU_SUCCESS);
        CHECK(cudaDeviceSynchronize() == cudaSuccess);
        std::vector<double> V2(m * m), P2(m * m);
        blastgpu::copy_to_host(dV, V2.data());
        blastgpu::copy_to_host(pP, P2.data());
        for (int j = 0; j < m; ++j) CHECK(P2[2 + j * m] == V[j + 5 * m] && V2[j + 5 * m] == P[2 + j * m]);
        blastgpu::Vector const rv = blastgpu::as_vector(blastgpu::row(blastgpu::Matrix(dV), 1));
        CHECK(rv.size == m && rv.inc == m);

        // a ragged batch of different sizes: gemm, potrf, trsm<Lower>/<Upper>, syrkLower per instance
        std::vector<blastgpu::DynamicMatrix> store;
        std::vector<blastgpu::Matrix> RA, RB, RC, RD, RS, RL, RX;
        int const sizes[3] = {3, 17, 40};
        std::vector<std::vector<double>> hA(3), hB(3), hS(3);
        for (int t = 0; t < 3; ++t) {
            int const q = sizes[t];
            hA[t].resize(q * q);
            hB[t].resize(q * 2);
            for (auto& v : hA[t]) v = U(gen);
            for (auto& v : hB[t]) v = U(gen);
            hS[t].assign(q * q, 0.0);
            for (int i = 0; i < q; ++i)
                for (int j = 0; j < q; ++j) {
                    double s = i == j ? q : 0.0;
                    for (int k = 0; k < q; ++k) s += hA[t][i + k * q] * hA[t][j + k * q];
                    hS[t][i + j * q] = s;
                }
        }
        store.reserve(18);
        for (int t = 0; t < 3; ++t)
            for (int w = 0; w < 6; ++w) store.emplace_back(sizes[t], w == 1 || w == 5 ? 2 : sizes[t]);
        for (int t = 0; t < 3; ++t) {
            blastgpu::Matrix a = store[6 * t], d = store[6 * t + 2], s2 = store[6 * t + 3], l = store[6 * t + 4],
                             x = store[6 * t + 5];
            blastgpu::copy_to_device(a, hA[t].data());
            blastgpu::copy_to_device(s2, hS[t].data());
            blastgpu::copy_to_device(x, hB[t].data());
            RA.push_back(a);
            RB.push_back(blastgpu::trans(a));
            RC.push_back(s2);
            RD.push_back(d);
            RS.push_back(s2);
            RL.push_back(l);
            RX.push_back(x);
        }
        blastgpu::gemm(1.0, RA, RB, 0.0, RC, RD, arena);        // D = A * A^T
        blastgpu::potrf(RS, RL, nullptr, arena);                // L = chol(S)
        blastgpu::trsm<blastgpu::UpLo::Lower, false>(RL, RX, RX, arena);
        std::vector<blastgpu::Matrix> RLt;
        for (auto const& l : RL) RLt.push_back(blastgpu::trans(l));
        blastgpu::trsm<blastgpu::UpLo::Upper, false>(RLt, RX, RX, arena);  // X = S^{-1} B
        blastgpu::syrkLower(1.0, RA, 1.0, RD, RD, arena);      // D_lower += A A^T
        CHECK(cudaDeviceSynchronize() == cudaSuccess);
        for (int t = 0; t < 3; ++t) {
            int const q = sizes[t];
            std::vector<double> Dg(q * q), Xg(q * 2);
            blastgpu::copy_to_host(RD[t], Dg.data());
            blastgpu::copy_to_host(RX[t], Xg.data());
            for (int j = 0; j < q; ++j)
                for (int i = 0; i < q; ++i) {
                    double const aat = hS[t][i + j * q] - (i == j ? q : 0.0);
                    CHECK(std::fabs(Dg[i + j * q] - (i >= j ? 2.0 : 1.0) * aat) < 1e-12 * q);
                }
            for (int c = 0; c < 2; ++c)
                for (int i = 0; i < q; ++i) {
                    double r = hB[t][i + c * q];
                    for (int j = 0; j < q; ++j) r -= hS[t][i + j * q] * Xg[j + c * q];
                    CHECK(std::fabs(r) < 1e-11 * q);
                }
        }
        bool threw2 = false;
        try { blastgpu::trans(blastgpu::Matrix(pA)); } catch (std::logic_error const&) { threw2 = true; }
        CHECK(threw2);
    }

    // size mismatch and unimplemented variants throw BLAST's exception types
    threw = false;
    try { blastgpu::gemm(bt(dA), blastgpu::batch(blastgpu::matrix(dB, n - 1, n)), bt(dC), bt(dD)); }
    catch (std::invalid_argument const&) { threw = true; }
    CHECK(threw);
    threw = false;
    try { blastgpu::trmm(1.0, bt(dA), blastgpu::UpLo::Lower, false, bt(dB), bt(dC)); }
    catch (std::logic_error const&) { threw = true; }
    CHECK(threw);
    std::printf("shim ok\n");
    return 0;
}

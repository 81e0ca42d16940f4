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

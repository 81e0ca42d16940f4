// Library-level entry points of blastgpu: version, status strings, error and launch accounting.
#include <atomic>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace blastgpu {

namespace {
thread_local int g_last_cuda_error = 0;
std::atomic<int64_t> g_launches{0};
}  // namespace

void set_cuda_error(cudaError_t e) { g_last_cuda_error = static_cast<int>(e); }
void count_launch(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

namespace {
std::mutex g_tune_mu;
std::map<std::string, int>& tune_table() {
    static std::map<std::string, int> t;
    return t;
}
}  // namespace

int tune_get(const char* key, int fallback) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto const& t = tune_table();
    auto it = t.find(key);
    return it == t.end() ? fallback : it->second;
}

int tune_get_bin(const char* prefix, int n, int fallback) {
    std::string const base(prefix);
    std::string const key = base + ".n" + std::to_string(size_bin(n));
    return tune_get(key.c_str(), tune_get(base.c_str(), fallback));
}

int sm_count() {
    static std::mutex mu;
    static std::vector<int> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    std::lock_guard<std::mutex> lock(mu);
    if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
    if (cache[dev] == 0) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
        cache[dev] = n;
    }
    return cache[dev];
}

// Self-test kernels for the Newton-Raphson reciprocal helpers (compared against IEEE 1/sqrt(x)
// and 1/x by the test-suite).
__global__ void selftest_kernel(int which, const double* x, double* y, int n) {
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = which == 0 ? rsqrt_nr(x[i]) : rcp_nr(x[i]);
}

// Binary64 FMA throughput probe: CHAINS independent FMA chains per thread, the loop unrolled
// UNROLL times; every CTA stores its per-thread sums into one small static array, so nothing
// needs allocating. Several shapes are timed and the best is reported, so that the figure is the
// pipe's throughput rather than one code shape's.
template <int CHAINS, int UNROLL>
__global__ void fp64_probe_kernel(int iters, double a, double b, double* sink) {
    double x[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) x[c] = threadIdx.x + c;
#pragma unroll UNROLL
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) x[c] = fma(x[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += x[c];
    sink[threadIdx.x] = s;
}

// The same measurement with one output per thread (no shared sink).
__global__ void fp64_probe_plain_kernel(double* out, int iters, double a, double b) {
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

// Binary64 tensor-core throughput probe: CHAINS independent accumulators per warp, each step one
// mma.sync.m8n8k4 (8*8*4 fused multiply-adds = 512 flops per warp instruction) per accumulator.
template <int CHAINS>
__global__ void dmma_probe_kernel(int iters, double* sink) {
    double const a = 1.0 + 1e-9 * threadIdx.x, b = 1e-6;
    double c[CHAINS][2];
#pragma unroll
    for (int q = 0; q < CHAINS; ++q) c[q][0] = c[q][1] = (double)q;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int q = 0; q < CHAINS; ++q)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
                         : "+d"(c[q][0]), "+d"(c[q][1])
                         : "d"(a), "d"(b));
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < CHAINS; ++q) s += c[q][0] + c[q][1];
    sink[threadIdx.x] = s;
}

// Binary32-accumulating tensor-core throughput probe (mma.sync): KIND 0 = m16n8k8 TF32,
// KIND 1 = m16n8k16 BF16; CHAINS independent accumulators per warp.
template <int KIND, int CHAINS>
__global__ void mma_probe_kernel(int iters, double* sink) {
    float c[CHAINS][4];
#pragma unroll
    for (int q = 0; q < CHAINS; ++q)
#pragma unroll
        for (int e = 0; e < 4; ++e) c[q][e] = 0.f;
    uint32_t const a0 = 0x3c003c00u + threadIdx.x, a1 = a0 + 1u, a2 = a0 + 2u, a3 = a0 + 3u, b0 = 0x3c003c00u;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int q = 0; q < CHAINS; ++q) {
            if constexpr (KIND == 0)
                asm volatile(
                    "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
                    "{%0, %1, %2, %3};\n"
                    : "+f"(c[q][0]), "+f"(c[q][1]), "+f"(c[q][2]), "+f"(c[q][3])
                    : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b0));
            else
                asm volatile(
                    "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
                    "{%0, %1, %2, %3};\n"
                    : "+f"(c[q][0]), "+f"(c[q][1]), "+f"(c[q][2]), "+f"(c[q][3])
                    : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b0));
        }
    }
    float s = 0.f;
#pragma unroll
    for (int q = 0; q < CHAINS; ++q)
#pragma unroll
        for (int e = 0; e < 4; ++e) s += c[q][e];
    sink[threadIdx.x] = s;
}

constexpr int kProbeMaxThreads = 160 * 8 * 256;
__device__ double g_probe_out[kProbeMaxThreads];
__device__ double g_probe_sink[256];

}  // namespace blastgpu

using namespace blastgpu;

extern "C" {

int blastgpu_version(void) { return 100; }

const char* blastgpu_status_string(int status) {
    switch (status) {
        case BLASTGPU_SUCCESS: return "success";
        case BLASTGPU_ERR_NOT_IMPLEMENTED: return "variant not implemented (BLAST throws std::logic_error)";
        case BLASTGPU_ERR_CUDA: return "CUDA error";
        case BLASTGPU_ERR_NO_DEVICE: return "no usable CUDA device";
        case BLASTGPU_ERR_TOO_LARGE: return "size beyond the supported maximum";
        default: break;
    }
    if (status < 0 && status > -100) return "invalid argument";
    return "unknown status";
}

int blastgpu_last_cuda_error(void) { return g_last_cuda_error; }

int blastgpu_tune_set(const char* key, int value) {
    if (!key || !*key || std::strlen(key) > 64) return -1;
    std::lock_guard<std::mutex> lock(g_tune_mu);
    tune_table()[key] = value;
    return BLASTGPU_SUCCESS;
}

int blastgpu_tune_get(const char* key, int* value) {
    if (!key || !*key) return -1;
    if (!value) return -2;
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto const& t = tune_table();
    auto it = t.find(key);
    if (it == t.end()) return -1;
    *value = it->second;
    return BLASTGPU_SUCCESS;
}

int64_t blastgpu_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

// Diagnostic export: y = rsqrt_nr(x) (which = 0) or rcp_nr(x) (which = 1), device arrays.
int blastgpu_selftest_recip(int which, const double* x, double* y, int n, blastgpu_stream_t stream) {
    if (which != 0 && which != 1) return -1;
    if (n < 0) return -4;
    if (n == 0) return BLASTGPU_SUCCESS;
    if (!x) return -2;
    if (!y) return -3;
    selftest_kernel<<<(n + 255) / 256, 256, 0, as_cuda(stream)>>>(which, x, y, n);
    return check_launch();
}

// Diagnostic export: measures the binary64 FMA throughput of the current device (TFLOP/s,
// two flops per FMA) with CUDA events on `stream`; synchronises the stream.
int blastgpu_probe_fp64_tflops(double* tflops, blastgpu_stream_t stream) {
    if (!tflops) return -1;
    cudaStream_t const s = as_cuda(stream);
    double* sink = nullptr;
    cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&sink), g_probe_sink);
    if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
    int const threads = 256, blocks = sm_count() * 8;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    double* out = nullptr;
    e = cudaGetSymbolAddress(reinterpret_cast<void**>(&out), g_probe_out);
    if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
    int const nshapes = blocks * threads <= kProbeMaxThreads ? 5 : 4;
    for (int shape = 0; shape < nshapes && e == cudaSuccess; ++shape) {
        int const chains = (shape < 2 || shape == 4) ? 8 : 16;
        int const iters = 8192 / chains * 4;
        for (int rep = 0; rep < 3; ++rep) {
            cudaEventRecord(e0, s);
            switch (shape) {
                case 0: fp64_probe_kernel<8, 1><<<blocks, threads, 0, s>>>(iters, 0.999, 1e-3, sink); break;
                case 1: fp64_probe_kernel<8, 4><<<blocks, threads, 0, s>>>(iters, 0.999, 1e-3, sink); break;
                case 2: fp64_probe_kernel<16, 1><<<blocks, threads, 0, s>>>(iters, 0.999, 1e-3, sink); break;
                case 3: fp64_probe_kernel<16, 2><<<blocks, threads, 0, s>>>(iters, 0.999, 1e-3, sink); break;
                default: fp64_probe_plain_kernel<<<blocks, threads, 0, s>>>(out, iters, 0.999, 1e-3); break;
            }
            cudaEventRecord(e1, s);
            e = cudaEventSynchronize(e1);
            if (e != cudaSuccess) break;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            double const tf = 2.0 * chains * (double)iters * blocks * threads / (ms * 1e-3) / 1e12;
            if (rep > 0 && tf > best) best = tf;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
    e = cudaGetLastError();
    if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
    *tflops = best;
    return BLASTGPU_SUCCESS;
}

// Diagnostic export: binary64 tensor-core (DMMA, mma.sync.m8n8k4.f64) throughput of the current
// device in TFLOP/s, measured like blastgpu_probe_fp64_tflops; synchronises the stream.
int blastgpu_probe_fp64_dmma_tflops(double* tflops, blastgpu_stream_t stream) {
    if (!tflops) return -1;
    cudaStream_t const s = as_cuda(stream);
    double* sink = nullptr;
    cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&sink), g_probe_sink);
    if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
    int const threads = 256, blocks = sm_count() * 4, iters = 2048;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    for (int shape = 0; shape < 2 && e == cudaSuccess; ++shape) {
        int const chains = shape == 0 ? 4 : 8;
        for (int rep = 0; rep < 3; ++rep) {
            cudaEventRecord(e0, s);
            if (shape == 0) dmma_probe_kernel<4><<<blocks, threads, 0, s>>>(iters, sink);
            else dmma_probe_kernel<8><<<blocks, threads, 0, s>>>(iters, sink);
            cudaEventRecord(e1, s);
            e = cudaEventSynchronize(e1);
            if (e != cudaSuccess) break;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            double const warps = (double)blocks * threads / 32;
            double const tf = 512.0 * chains * (double)iters * warps / (ms * 1e-3) / 1e12;
            if (rep > 0 && tf > best) best = tf;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
    e = cudaGetLastError();
    if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
    *tflops = best;
    return BLASTGPU_SUCCESS;
}

// Diagnostic export: throughput (TFLOP/s) of the warp-level tensor-core instruction the mixed
// path's tensor-core update uses (kind 0: mma.sync m16n8k8 TF32) or its BF16 counterpart
// (kind 1: m16n8k16), binary32 accumulation; synchronises the stream.
int blastgpu_probe_mma_tflops(int kind, double* tflops, blastgpu_stream_t stream) {
    if (kind != 0 && kind != 1) return -1;
    if (!tflops) return -2;
    cudaStream_t const s = as_cuda(stream);
    double* sink = nullptr;
    cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&sink), g_probe_sink);
    if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
    int const threads = 256, blocks = sm_count() * 2, iters = 4096, chains = 8;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
        cudaEventRecord(e0, s);
        if (kind == 0) mma_probe_kernel<0, 8><<<blocks, threads, 0, s>>>(iters, sink);
        else mma_probe_kernel<1, 8><<<blocks, threads, 0, s>>>(iters, sink);
        cudaEventRecord(e1, s);
        e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        double const k = kind == 0 ? 8.0 : 16.0;
        double const warps = (double)blocks * threads / 32;
        double const tf = 2.0 * 16 * 8 * k * chains * (double)iters * warps / (ms * 1e-3) / 1e12;
        if (rep > 0 && tf > best) best = tf;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
    e = cudaGetLastError();
    if (e != cudaSuccess) { set_cuda_error(e); return BLASTGPU_ERR_CUDA; }
    *tflops = best;
    return BLASTGPU_SUCCESS;
}

}  // extern "C"

// FP32 CUDA-core throughput microbenchmark for the benchmark script (built into its own library,
// libgbfwn_bench.so, not into the product library): the denominator of the traversal kernels'
// FP32-op fraction.  Every thread runs 8 independent FMA chains (no dependency between them, so the
// FMA pipes, not latency, set the pace) on a persistent grid of 8 blocks per SM; the result is
// written only under a condition the data never meets, so the work cannot be removed.
#include <cuda_runtime.h>

#include <algorithm>

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) fmaKernel(int iters, float seed, float* sink) {
    float a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = seed + float(threadIdx.x + k);
    const float m = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int r = 0; r < 16; ++r) {
#pragma unroll
            for (int k = 0; k < kChains; ++k) a[k] = fmaf(a[k], m, c);
        }
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += a[k];
    if (s == -1.2345f) sink[threadIdx.x] = s;
}

}  // namespace

// Measured FP32 FMA throughput of `device` in TFLOP/s (2 FLOP per FMA), best of `reps` launches of
// about 10 ms each.  Returns a cudaError_t value (0 = success).
extern "C" __attribute__((visibility("default"))) int bench_fp32_peak(int device, int reps, double* tflops) {
    if (!tflops || reps <= 0) return int(cudaErrorInvalidValue);
    int prev = -1;
    cudaGetDevice(&prev);
    cudaError_t e = cudaSetDevice(device);
    int sms = 0;
    if (!e) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    float* sink = nullptr;
    if (!e) e = cudaMalloc((void**)&sink, 256 * sizeof(float));
    cudaEvent_t a = nullptr, b = nullptr;
    if (!e) e = cudaEventCreate(&a);
    if (!e) e = cudaEventCreate(&b);
    const int blocks = sms * 8, threads = 256, iters = 8192;
    double best = 0;
    for (int r = 0; !e && r <= reps; ++r) {  // launch 0 warms up
        cudaEventRecord(a, 0);
        fmaKernel<<<blocks, threads>>>(iters, 1.0f, sink);
        cudaEventRecord(b, 0);
        e = cudaEventSynchronize(b);
        float ms = 0;
        if (!e) e = cudaEventElapsedTime(&ms, a, b);
        if (!e && r > 0 && ms > 0) {
            const double flop = 2.0 * double(blocks) * threads * iters * 16 * kChains;
            best = std::max(best, flop / (double(ms) * 1e-3) / 1e12);
        }
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (sink) cudaFree(sink);
    if (prev >= 0) cudaSetDevice(prev);
    if (!e) *tflops = best;
    return int(e);
}

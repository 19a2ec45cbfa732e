// Diagnostics of the FP64 arithmetic:
//  * a throughput probe of the FP64 pipe, the denominator of the FP64
//    pushes' roofline.  GB300 executes FP64 at a small fraction of its FP32
//    rate, and the plain FP64 push is bound there, not by memory; the probe
//    measures the rate the pipe sustains on the part the library runs on,
//    with the clocks as they are (nothing is locked or changed);
//  * the FP64 push's power function (kpt_pow.h) evaluated on the device, so
//    tests can compare it bit for bit with the host's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "kpt_internal.h"
#include "kpt_pow.h"

namespace kpt {
namespace {

constexpr int kChains = 8;  // independent FMA chains per thread (hides the pipe latency)

// Every thread runs kChains dependent chains a <- a * m + c for `iters`
// iterations: 2 * kChains * iters flop per thread, no memory traffic inside
// the loop.  m and c come from the arguments so the compiler cannot fold the
// chains; the sum is stored so it cannot drop them.
__global__ void __launch_bounds__(256) fp64_fma_kernel(int iters, double m, double c,
                                                       double* __restrict__ sink) {
    double a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) {
        a[k] = 1.0 + 1e-3 * static_cast<double>(threadIdx.x + k);
    }
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) {
            a[k] = __fma_rn(a[k], m, c);
        }
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += a[k];
    if (s == 12345.678) {  // never true for these inputs; keeps the chains live
        sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
    }
}

__global__ void __launch_bounds__(256) pow_kernel(uint64_t n, const double* __restrict__ x,
                                                  const double* __restrict__ y,
                                                  double* __restrict__ out) {
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        out[i] = kpt_pow(x[i], y[i]);
    }
}

}  // namespace

cudaError_t launch_pow(uint64_t n, const double* x, const double* y, double* out, int sm_count,
                       cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const uint64_t want = (n + 255) / 256;
    const uint64_t cap = static_cast<uint64_t>(sm_count) * 16;
    pow_kernel<<<static_cast<int>(want < cap ? want : cap), 256, 0, stream>>>(n, x, y, out);
    return cudaGetLastError();
}

cudaError_t fp64_fma_rate(int sm_count, cudaStream_t stream, double* tflops) {
    const int threads = 256;
    const int blocks = sm_count * 8;
    const int iters = 4096;
    double* sink = nullptr;
    cudaError_t err = cudaMalloc(&sink, sizeof(double) * threads * blocks);
    if (err != cudaSuccess) return err;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    double best_ms = 0.0;
    // one warm-up launch, then the best of five
    for (int rep = 0; rep < 6 && err == cudaSuccess; ++rep) {
        err = cudaEventRecord(e0, stream);
        if (err != cudaSuccess) break;
        fp64_fma_kernel<<<blocks, threads, 0, stream>>>(iters, 0.9999999, 1e-7, sink);
        err = cudaGetLastError();
        if (err != cudaSuccess) break;
        err = cudaEventRecord(e1, stream);
        if (err != cudaSuccess) break;
        err = cudaEventSynchronize(e1);
        if (err != cudaSuccess) break;
        float ms = 0.0f;
        err = cudaEventElapsedTime(&ms, e0, e1);
        if (err == cudaSuccess && rep > 0) {
            best_ms = best_ms == 0.0 ? ms : std::min(best_ms, static_cast<double>(ms));
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(sink);
    if (err != cudaSuccess) return err;
    const double flop = 2.0 * kChains * static_cast<double>(iters) * threads * blocks;
    *tflops = best_ms > 0.0 ? flop / (best_ms * 1e-3) / 1e12 : 0.0;
    return cudaSuccess;
}

}  // namespace kpt

// FP32 FMA throughput probe (sm_103a): the measured ceiling that the radiality
// kernel's roofline is read against, next to the nominal 128 FMA lanes per SM
// at the maximum clock. Every thread runs 16 independent FMA chains (as packed
// f32x2 pairs) for a fixed number of iterations over a grid of 8 CTAs of 256
// threads per SM; throughput = 2 flops per FMA over the CUDA-event time of the
// launch. No counterpart in the reference (measurement only).
#include <cuda_runtime.h>

#include "srrf_internal.h"

namespace rfba {
namespace {

constexpr int kProbeThreads = 256;
constexpr int kProbeChains = 8;  // f32x2 pairs: 16 FMAs per iteration

__global__ void __launch_bounds__(kProbeThreads) fma_probe_kernel(float* out, int iters, float a, float b) {
    float2 x[kProbeChains];
#pragma unroll
    for (int i = 0; i < kProbeChains; ++i) x[i] = make_float2(threadIdx.x * 1e-3f + i, 0.5f * i);
    const float2 A = make_float2(a, a), B = make_float2(b, b);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < kProbeChains; ++i) x[i] = __ffma2_rn(x[i], A, B);
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < kProbeChains; ++i) s += x[i].x + x[i].y;
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

}  // namespace

int probe_fp32_fma(int device, double* tflops) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return (int)e;
    int sms = 0;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) return (int)e;
    const int blocks = sms * 8, iters = 1 << 15;
    float* out = nullptr;
    if ((e = cudaMalloc(&out, sizeof(float) * (size_t)blocks * kProbeThreads)) != cudaSuccess) return (int)e;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 0.f;
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {  // the first launch warms up
        cudaEventRecord(e0);
        fma_probe_kernel<<<blocks, kProbeThreads>>>(out, iters, 0.9999f, 1e-4f);
        cudaEventRecord(e1);
        e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaGetLastError();
        float ms = 0.f;
        if (e == cudaSuccess && rep > 0 && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms > 0.f) {
            const double fmas = (double)blocks * kProbeThreads * iters * 2.0 * kProbeChains;
            const float tf = (float)(2.0 * fmas / (ms * 1e-3) / 1e12);
            if (tf > best) best = tf;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    *tflops = best;
    return (int)e;
}

}  // namespace rfba

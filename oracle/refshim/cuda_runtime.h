// Host-side stand-in for the CUDA runtime, used only to compile the reference's
// GradientCalc/kernel.cu as plain C++ so that its arithmetic can run on CPU cores
// and pin the oracle. Test infrastructure: nothing in the product links this.
//
// A "launch" runs every (block, thread) index of the 1-D grid on the host; blocks
// are distributed over OpenMP threads. Each emulated GPU thread sees its own
// blockIdx/threadIdx through thread_local variables. Device allocations are
// zero-filled host allocations padded by one full copy of the requested size, so
// that the reference's reads just past an array end (the tap at q = dim - 1.5 and
// the odd-length TRAC binning read) see zeros instead of undefined memory.
#pragma once
#include <cstdlib>
#include <cstring>
#include <cstdio>
#include <cmath>
#include <functional>

#define __global__
#define __device__
#define __host__

struct ref_uint3 { unsigned x, y, z; };
extern thread_local ref_uint3 blockIdx;
extern thread_local ref_uint3 threadIdx;
extern thread_local ref_uint3 blockDim;
extern thread_local ref_uint3 gridDim;

typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind { cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1,
                      cudaMemcpyDeviceToHost = 2, cudaMemcpyDeviceToDevice = 3 };

static inline cudaError_t cudaMalloc(void** p, size_t n) {
    *p = std::calloc(2 * n + 256, 1);
    return cudaSuccess;
}
static inline cudaError_t cudaFree(void* p) { std::free(p); return cudaSuccess; }
static inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) {
    std::memcpy(d, s, n);
    return cudaSuccess;
}
static inline cudaError_t cudaMemset(void* d, int v, size_t n) {
    std::memset(d, v, n);
    return cudaSuccess;
}

void ref_launch_1d(int grid, int block, const std::function<void()>& body);

// The build recipe rewrites each `kernel << <g, b >> > (args)` of the reference
// into `REF_LAUNCH(g, b, kernel, args)`.
#define REF_LAUNCH(g, b, k, ...) ref_launch_1d((g), (b), [&]() { k(__VA_ARGS__); })

// Host grid loop for the reference kernels compiled as C++ (see cuda_runtime.h).
#include "cuda_runtime.h"

thread_local ref_uint3 blockIdx;
thread_local ref_uint3 threadIdx;
thread_local ref_uint3 blockDim;
thread_local ref_uint3 gridDim;

void ref_launch_1d(int grid, int block, const std::function<void()>& body) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int b = 0; b < grid; ++b) {
        gridDim = {(unsigned)grid, 1, 1};
        blockDim = {(unsigned)block, 1, 1};
        blockIdx = {(unsigned)b, 0, 0};
        for (int t = 0; t < block; ++t) {
            threadIdx = {(unsigned)t, 0, 0};
            body();
        }
    }
}

// SRRF-guided spot seeding (sm_103a).
//
// The reference seeds 3B's spots from the SRRF map by rejection sampling on
// the host (multispot5_place_methods.cc:291-341, multispot5.cc:2164-2231):
// the magnified subvoxels of the block's input voxels are candidates, a
// candidate is kept with probability value / max, and a kept one gives the spot
// (subvoxel + U(-0.5, 0.5) per axis) / mag. Here the same distribution is drawn
// by inverse CDF, one thread per spot:
//   1. weights: the map value of every candidate subvoxel (NaN and negative
//      values count as 0, as they do after multispot5_place_methods.cc:260-269);
//   2. inclusive prefix sum of the weights in FP64 (block scan + carries);
//   3. per spot, four uniforms from Philox4x32-10 (Salmon, Moraes, Dror, Shaw,
//      "Parallel random numbers: as easy as 1, 2, 3", SC 2011; counter = spot
//      index, key = seed): a 53-bit uniform picks the subvoxel by binary search
//      of the CDF, three 32-bit uniforms place the spot inside it.
// An all-zero map makes every candidate equally likely, as the reference's
// `y <= value` test with max = 0 does.
#include <cuda_runtime.h>
#include <cstdint>

#include "philox.h"
#include "srrf_internal.h"

namespace rfba {
namespace {

constexpr int kScanThreads = 512;

// weight of candidate i: voxel v = i / mag^3, sub-offset (j1, j2, j3) in the
// reference's order (x slowest of the three, multispot5_place_methods.cc:297-303)
__global__ void seed_weights_kernel(const float* __restrict__ map, const int* __restrict__ vox, long long ncand,
                                    int mag, long long Wm, long long Hm, long long Dm, double* __restrict__ w,
                                    unsigned long long* err) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncand) return;
    const int m3 = mag * mag * mag;
    const long long v = i / m3;
    const int r = (int)(i - v * m3);
    const int j1 = r / (mag * mag), j2 = (r / mag) % mag, j3 = r % mag;
    const long long x = (long long)vox[3 * v] * mag + j1, y = (long long)vox[3 * v + 1] * mag + j2,
                    z = (long long)vox[3 * v + 2] * mag + j3;
    double val = 0.0;
    if (x >= 0 && x < Wm && y >= 0 && y < Hm && z >= 0 && z < Dm) {
        const float f = map[(z * Hm + y) * Wm + x];
        val = (f > 0.f) ? (double)f : 0.0;  // NaN compares false
    } else if (err) {
        atomicCAS(err, 0ull, (0x53ull << 56) | (unsigned long long)i);
    }
    w[i] = val;
}

// inclusive scan of w within each block of kScanThreads elements; block totals to sums
__global__ void scan_block_kernel(double* __restrict__ w, long long n, double* __restrict__ sums) {
    __shared__ double s[kScanThreads];
    const long long i = (long long)blockIdx.x * kScanThreads + threadIdx.x;
    s[threadIdx.x] = i < n ? w[i] : 0.0;
    __syncthreads();
    for (int off = 1; off < kScanThreads; off <<= 1) {
        const double add = threadIdx.x >= off ? s[threadIdx.x - off] : 0.0;
        __syncthreads();
        s[threadIdx.x] += add;
        __syncthreads();
    }
    if (i < n) w[i] = s[threadIdx.x];
    if (threadIdx.x == kScanThreads - 1) sums[blockIdx.x] = s[threadIdx.x];
}

__global__ void add_carry_kernel(double* __restrict__ w, long long n, const double* __restrict__ carry) {
    const long long i = (long long)blockIdx.x * kScanThreads + threadIdx.x;
    if (blockIdx.x > 0 && i < n) w[i] += carry[blockIdx.x - 1];
}

__global__ void seed_draw_kernel(const double* __restrict__ cdf, long long ncand, const int* __restrict__ vox,
                                 int mag, int nspots, uint32_t k0, uint32_t k1, float* __restrict__ xyz) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nspots) return;
    uint32_t c[4] = {(uint32_t)s, 0u, 0x5EEDu, 0u};
    Philox::gen(c, k0, k1);
    const double total = cdf[ncand - 1];
    const double u = u53(c[0], c[1]);
    long long pick;
    if (total > 0.0) {
        const double target = u * total;
        long long lo = 0, hi = ncand - 1;  // first index with cdf > target
        while (lo < hi) {
            const long long mid = (lo + hi) >> 1;
            if (cdf[mid] > target)
                hi = mid;
            else
                lo = mid + 1;
        }
        pick = lo;
    } else {
        pick = (long long)(u * (double)ncand);
        if (pick >= ncand) pick = ncand - 1;
    }
    const int m3 = mag * mag * mag;
    const long long v = pick / m3;
    const int r = (int)(pick - v * m3);
    const int j1 = r / (mag * mag), j2 = (r / mag) % mag, j3 = r % mag;
    // (subvoxel + U - 0.5) / mag in float, as the reference forms it
    uint32_t d[4] = {(uint32_t)s, 1u, 0x5EEDu, 0u};
    Philox::gen(d, k0, k1);
    const float fx = (float)((double)(vox[3 * v] * mag + j1) + u32(d[0]) - 0.5);
    const float fy = (float)((double)(vox[3 * v + 1] * mag + j2) + u32(d[1]) - 0.5);
    const float fz = (float)((double)(vox[3 * v + 2] * mag + j3) + u32(d[2]) - 0.5);
    xyz[3 * s] = fx / (float)mag;
    xyz[3 * s + 1] = fy / (float)mag;
    xyz[3 * s + 2] = fz / (float)mag;
}

}  // namespace

// Scratch: w (ncand doubles), sums (ceil(ncand / 512) doubles), carry (ceil(ncand / 512^2) + 1
// doubles). Up to 512^3 candidates.
int launch_seed_spots(const float* map, const int map_dims[3], int mag, const int* vox, long long nvox, int nspots,
                      unsigned long long seed, float* xyz, double* w, double* sums, double* carry,
                      unsigned long long* err, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const long long ncand = nvox * mag * mag * mag;
    if (ncand <= 0 || nspots <= 0) return 0;
    const long long n1 = (ncand + kScanThreads - 1) / kScanThreads;
    const long long n2 = (n1 + kScanThreads - 1) / kScanThreads;
    if (n2 > kScanThreads) return (int)cudaErrorInvalidValue;
    seed_weights_kernel<<<(unsigned)((ncand + 255) / 256), 256, 0, st>>>(map, vox, ncand, mag, map_dims[0], map_dims[1],
                                                                         map_dims[2], w, err);
    scan_block_kernel<<<(unsigned)n1, kScanThreads, 0, st>>>(w, ncand, sums);
    if (n1 > 1) {
        scan_block_kernel<<<(unsigned)n2, kScanThreads, 0, st>>>(sums, n1, carry);
        if (n2 > 1) {
            scan_block_kernel<<<1, kScanThreads, 0, st>>>(carry, n2, carry + n2);
            add_carry_kernel<<<(unsigned)n2, kScanThreads, 0, st>>>(sums, n1, carry);
        }
        add_carry_kernel<<<(unsigned)n1, kScanThreads, 0, st>>>(w, ncand, sums);
    }
    seed_draw_kernel<<<(nspots + 255) / 256, 256, 0, st>>>(w, ncand, vox, mag, nspots, (uint32_t)seed,
                                                           (uint32_t)(seed >> 32), xyz);
    return (int)cudaGetLastError();
}

}  // namespace rfba

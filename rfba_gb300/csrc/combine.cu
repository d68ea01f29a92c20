// CombineBlock on the GPU (Matlab Scripts/CombineBlock.m:24-173): localisation
// histogram on the zoomed grid, the noise mask from box sums of the occupied
// voxels, convn(..., psf, 'same') with the uint16 PSF of genpsf.m, and the
// scaling to uint16. Everything is integer arithmetic up to the final scaling
// (counts x uint16 PSF, summed in 64-bit integers), so the result does not
// depend on the order of the additions.
//
// Grid layout [z][y][x], x fastest (X' = X * zoom, ...). The reference's array
// is imgout(y, x, z) of size (Y' + 1, X' + 1, Z' + 1) cropped to (Y', X', Z'):
// a spot lands at round(p * zoom) (round half away from zero), spots rounding
// to X' (or beyond) fall in the cropped margin.
#include <cuda_runtime.h>
#include <cstdint>

#include "srrf_internal.h"

namespace rfba {
namespace {

__device__ __forceinline__ long long matlab_round(double v) {
    return (long long)(v < 0.0 ? -floor(-v + 0.5) : floor(v + 0.5));
}

__global__ void hist_kernel(const double* __restrict__ spots, long long n, int zoom, int Xp, int Yp, int Zp,
                            unsigned int* __restrict__ hist, unsigned long long* __restrict__ dropped) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long ix = matlab_round(spots[5 * i + 2] * zoom);
    const long long iy = matlab_round(spots[5 * i + 3] * zoom);
    const long long iz = matlab_round(spots[5 * i + 4] * zoom);
    if (ix < 0 || iy < 0 || iz < 0 || ix >= Xp || iy >= Yp || iz >= Zp) {
        atomicAdd(dropped, 1ull);
        return;
    }
    atomicAdd(hist + ((size_t)iz * Yp + iy) * Xp + ix, 1u);
}

// L[z][y][x] = sum over |dy| <= r of (hist > 0) for y in [r, Y' - r - 1], else 0
// (CombineBlock.m:89-101): one thread per (z, x) column, running sum along y.
__global__ void box_y_kernel(const unsigned int* __restrict__ hist, int Xp, int Yp, int Zp, int r,
                             unsigned char* __restrict__ L) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long long)Xp * Zp) return;
    const int x = (int)(c % Xp), z = (int)(c / Xp);
    const size_t base = (size_t)z * Yp * Xp + x;
    int s = 0;
    for (int y = 0; y < Yp; ++y) {
        if (y <= 2 * r) s += hist[base + (size_t)y * Xp] > 0;
        L[base + (size_t)y * Xp] = 0;
    }
    if (Yp < 2 * r + 1) return;
    L[base + (size_t)r * Xp] = (unsigned char)s;
    for (int y = r + 1; y <= Yp - r - 1; ++y) {
        s += (hist[base + (size_t)(y + r) * Xp] > 0) - (hist[base + (size_t)(y - r - 1) * Xp] > 0);
        L[base + (size_t)y * Xp] = (unsigned char)s;
    }
}

// S[z][y][x] = sum over |dx| <= r of L for x in [r, X' - r - 1], else 0
// (CombineBlock.m:103-114). One warp per (z, y) row, 8 rows per CTA: the row is
// staged in shared memory with coalesced loads, then each lane runs the sum
// along its own stretch of x.
constexpr int kBoxRows = 8;
__global__ void __launch_bounds__(32 * kBoxRows) box_x_warp_kernel(const unsigned char* __restrict__ L, int Xp,
                                                                    int Yp, int Zp, int r,
                                                                    unsigned short* __restrict__ S) {
    extern __shared__ unsigned char srow[];  // [kBoxRows][Xp]
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long row = (long long)blockIdx.x * kBoxRows + w;
    if (row >= (long long)Yp * Zp) return;  // whole warps only; no CTA barrier below
    unsigned char* sr = srow + (size_t)w * Xp;
    const unsigned char* l = L + (size_t)row * Xp;
    for (int x = lane; x < Xp; x += 32) sr[x] = l[x];
    __syncwarp();
    unsigned short* o = S + (size_t)row * Xp;
    const int chunk = (Xp + 31) / 32;
    const int x0 = lane * chunk, x1 = min(Xp, x0 + chunk);
    unsigned int sum = 0;
    bool have = false;
    for (int x = x0; x < x1; ++x) {
        if (Xp < 2 * r + 1 || x < r || x > Xp - r - 1) {
            o[x] = 0;
            continue;
        }
        if (!have) {
            for (int k = x - r; k <= x + r; ++k) sum += sr[k];
            have = true;
        } else {
            sum += sr[x + r] - sr[x - r - 1];
        }
        o[x] = (unsigned short)sum;
    }
}

// The same with one thread per row, for rows too long to stage.
__global__ void box_x_kernel(const unsigned char* __restrict__ L, int Xp, int Yp, int Zp, int r,
                             unsigned short* __restrict__ S) {
    const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= (long long)Yp * Zp) return;
    const unsigned char* l = L + (size_t)row * Xp;
    unsigned short* o = S + (size_t)row * Xp;
    if (Xp < 2 * r + 1) {
        for (int x = 0; x < Xp; ++x) o[x] = 0;
        return;
    }
    unsigned int s = 0;
    for (int x = 0; x <= 2 * r; ++x) s += l[x];
    for (int x = 0; x < r; ++x) o[x] = 0;
    o[r] = (unsigned short)s;
    for (int x = r + 1; x <= Xp - r - 1; ++x) {
        s += l[x + r] - l[x - r - 1];
        o[x] = (unsigned short)s;
    }
    for (int x = Xp - r; x < Xp; ++x) o[x] = 0;
}

// V = sum over |dz| <= rz of S for z in [rz, Z' - rz - 1]; mask = V > thr there, 1
// elsewhere (CombineBlock.m:117-137); hist *= mask in place. One thread per (y, x).
__global__ void box_z_mask_kernel(const unsigned short* __restrict__ S, int Xp, int Yp, int Zp, int r, int rz,
                                  int thr, unsigned int* __restrict__ hist) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long long)Xp * Yp) return;
    const int x = (int)(c % Xp), y = (int)(c / Xp);
    const size_t plane = (size_t)Xp * Yp;
    const bool inxy = x >= r && x <= Xp - r - 1 && y >= r && y <= Yp - r - 1;
    if (!inxy || Zp < 2 * rz + 1) return;  // mask 1: nothing to do
    unsigned int s = 0;
    for (int z = 0; z <= 2 * rz; ++z) s += S[z * plane + c];
    for (int z = rz; z <= Zp - rz - 1; ++z) {
        if (z > rz) s += S[(size_t)(z + rz) * plane + c] - S[(size_t)(z - rz - 1) * plane + c];
        if (!(s > (unsigned int)thr)) hist[(size_t)z * plane + c] = 0;
    }
}

__global__ void compact_kernel(const unsigned int* __restrict__ hist, long long n, unsigned long long* __restrict__ idx,
                               unsigned int* __restrict__ val, unsigned long long* __restrict__ count,
                               unsigned long long cap) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned int h = hist[i];
    if (!h) return;
    const unsigned long long k = atomicAdd(count, 1ull);
    if (k < cap) {
        idx[k] = (unsigned long long)i;
        val[k] = h;
    }
}

// convn(A, psf, 'same'): A(a) adds A(a) * psf(k) at a + k - floor(K / 2) per axis.
// One CTA per nonzero voxel (grid-stride), the PSF in shared memory.
__global__ void scatter_conv_kernel(const unsigned long long* __restrict__ idx, const unsigned int* __restrict__ val,
                                    const unsigned long long* __restrict__ count, unsigned long long cap,
                                    const uint16_t* __restrict__ psf, int Kx, int Ky, int Kz, int Xp, int Yp, int Zp,
                                    unsigned long long* __restrict__ out) {
    extern __shared__ uint16_t spsf[];
    const unsigned long long nnz = *count < cap ? *count : cap;
    const int nk = Kx * Ky * Kz;
    for (int i = threadIdx.x; i < nk; i += blockDim.x) spsf[i] = psf[i];
    __syncthreads();
    const int hx = Kx / 2, hy = Ky / 2, hz = Kz / 2;
    for (unsigned long long e = blockIdx.x; e < nnz; e += gridDim.x) {
        const unsigned long long a = idx[e];
        const unsigned long long c = val[e];
        const int ax = (int)(a % Xp), ay = (int)((a / Xp) % Yp), az = (int)(a / ((unsigned long long)Xp * Yp));
        for (int k = threadIdx.x; k < nk; k += blockDim.x) {
            const int kx = k % Kx, ky = (k / Kx) % Ky, kz = k / (Kx * Ky);
            const int ox = ax + kx - hx, oy = ay + ky - hy, oz = az + kz - hz;
            const unsigned int w = spsf[k];
            if (w && ox >= 0 && ox < Xp && oy >= 0 && oy < Yp && oz >= 0 && oz < Zp)
                atomicAdd(out + ((size_t)oz * Yp + oy) * Xp + ox, c * w);
        }
    }
}

__global__ void max_kernel(const unsigned long long* __restrict__ v, long long n, unsigned long long* __restrict__ mx) {
    unsigned long long m = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        m = v[i] > m ? v[i] : m;
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_down_sync(0xffffffffu, m, o);
        m = t > m ? t : m;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(mx, m);
}

// result / max * 65535 in double, then MATLAB's uint16(): round half away, saturate
__global__ void scale_kernel(const unsigned long long* __restrict__ v, long long n,
                             const unsigned long long* __restrict__ mx, uint16_t* __restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long vi = v[i];
    if (vi == 0) {  // (0 / m) * 65535 rounds to 0: no FP64 division for the empty grid voxels
        out[i] = 0;
        return;
    }
    const double m = (double)*mx;
    double r = m > 0.0 ? ((double)vi / m) * 65535.0 : 0.0;
    r = r >= 65535.0 ? 65535.0 : floor(r + 0.5);
    out[i] = (uint16_t)r;
}

unsigned grid_for(long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

int launch_combine(const double* spots, long long n, int zoom, int Xp, int Yp, int Zp, int r, int rz, int thr,
                   const uint16_t* psf, int Kx, int Ky, int Kz, unsigned int* hist, unsigned char* L,
                   unsigned short* S, unsigned long long* idx, unsigned int* val, unsigned long long cap,
                   unsigned long long* counters /* [0] dropped, [1] nnz, [2] max */, unsigned long long* out,
                   uint16_t* out16, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const long long nvox = (long long)Xp * Yp * Zp;
    cudaMemsetAsync(hist, 0, (size_t)nvox * 4, st);
    cudaMemsetAsync(out, 0, (size_t)nvox * 8, st);
    cudaMemsetAsync(counters, 0, 3 * sizeof(unsigned long long), st);
    if (n > 0) hist_kernel<<<grid_for(n, 256), 256, 0, st>>>(spots, n, zoom, Xp, Yp, Zp, hist, counters);
    box_y_kernel<<<grid_for((long long)Xp * Zp, 256), 256, 0, st>>>(hist, Xp, Yp, Zp, r, L);
    if ((size_t)kBoxRows * Xp <= 48 * 1024)
        box_x_warp_kernel<<<grid_for((long long)Yp * Zp, kBoxRows), 32 * kBoxRows, (size_t)kBoxRows * Xp, st>>>(
            L, Xp, Yp, Zp, r, S);
    else
        box_x_kernel<<<grid_for((long long)Yp * Zp, 256), 256, 0, st>>>(L, Xp, Yp, Zp, r, S);
    box_z_mask_kernel<<<grid_for((long long)Xp * Yp, 256), 256, 0, st>>>(S, Xp, Yp, Zp, r, rz, thr, hist);
    compact_kernel<<<grid_for(nvox, 256), 256, 0, st>>>(hist, nvox, idx, val, counters + 1, cap);
    const size_t psf_bytes = (size_t)Kx * Ky * Kz * 2;
    cudaError_t e = cudaFuncSetAttribute(scatter_conv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)psf_bytes);
    if (e != cudaSuccess) return (int)e;
    // nonzero count is on the device: launch a fixed persistent grid that strides over it
    scatter_conv_kernel<<<4 * 152, 256, psf_bytes, st>>>(idx, val, counters + 1, cap, psf, Kx, Ky, Kz, Xp, Yp, Zp,
                                                         out);
    max_kernel<<<4 * 152, 256, 0, st>>>(out, nvox, counters + 2);
    scale_kernel<<<grid_for(nvox, 256), 256, 0, st>>>(out, nvox, counters + 2, out16);
    return (int)cudaGetLastError();
}

}  // namespace rfba

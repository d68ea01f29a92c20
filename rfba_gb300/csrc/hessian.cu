// 3B's sampled-background Hessian of a spot's log probability (sm_103a, FP64).
//
// sampled_background_spot_hessian_ffbs (RFBA Main/multispot5.cc:824-985):
// for every background sample i (the Gibbs draws with the spot taken off) and
// frame f, the parts the frame adds when the spot is on,
//   hess_if = sum_p e H_p - g_p g_p^T,   deriv_if = sum_p e g_p,
//   e = data - (sample + spot intensity),
// over all pixels p, with the spot's value, gradient g_p and Hessian H_p from
// spot_shape_hess_position (storm.h:87-146); then the spot's on / off chain is
// filtered on the sample (SpotWithBackground over all pixels,
// spot_with_background.hh:98-150; forward_algorithm_delta) and bs_iterations
// state sequences are drawn backwards (backward_sampling), each adding
// hess + deriv deriv^T and deriv over the frames where the spot is on. The
// host divides by (bs_iterations * samples * variance), subtracts the outer
// product of the mean derivative and adds the log-normal priors' second
// derivatives.
//
// FreeEnergyHessian::hessian (multispot5.cc:693-775), the "pure MCMC"
// Hessian, uses the first three kernels on draws that hold every spot
// (e = data - sample) and finishes on the host from the drawn states.
//
// Kernels:
//   hess_table_kernel   one thread per pixel: value, gradient (5) and the 15
//                       upper entries of the spot's Hessian at the pixel
//   hess_parts_kernel   one thread per (frame, sample) and pixel chunk: the 22
//                       sums (on / off sums of squares, 15 + 5 parts) over
//                       the chunk, written per chunk and summed in chunk order
//   hess_gg_kernel      one CTA: sum_p g_p g_p^T (the same for every frame)
//   hess_ffbs_kernel    one CTA per sample: chunk sums, emission terms,
//                       forward filter (ffbs.cuh), per-frame thresholds, the
//                       backward walks (one per thread at a time, uniforms from
//                       Philox4x32-10 with counter (frame, walk, sample)) and
//                       the sample's 20 sums in thread order.
//
// The reference's Hessian entry [4][3] is never written (storm.h:143 assigns
// it to itself) and holds whatever the stack held; here the matrix is
// symmetric, [4][3] = [3][4].
#include <cuda_runtime.h>
#include <cstdint>

#include "ffbs.cuh"
#include "philox.h"
#include "srrf_internal.h"

namespace rfba {
namespace {

constexpr int kPartThreads = 128;
constexpr int kFfbsThreads = 256;
constexpr int kTab = 21;    // value, gradient 5, Hessian upper 15
constexpr int kParts = 22;  // sum e^2 (on), sum (d - s)^2 (off), Hessian 15, gradient 5

// upper-triangle index of (a, b), a <= b
__host__ __device__ constexpr int up(int a, int b) { return a * 5 - a * (a - 1) / 2 + (b - a); }

__global__ void hess_table_kernel(const int* __restrict__ pixels, int P, const double* __restrict__ phi, double zf,
                                  double* __restrict__ tab) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const double p0 = phi[0], p1 = phi[1];
    const double dx = pixels[3 * p] - phi[2], dy = pixels[3 * p + 1] - phi[3], dz = pixels[3 * p + 2] - phi[4];
    const double dzs = dz / zf;
    const double s = -(dx * dx + dy * dy + dzs * dzs) / (2 * p1 * p1);
    const double r2pi = sqrt(2 * 3.14159265358979323846);
    const double es = exp(s);
    double* t = tab + (size_t)p * kTab;
    t[0] = es * p0 / (p1 * r2pi);
    const double c = es / (p1 * r2pi);
    t[1] = c * 1.0;
    t[2] = c * (-p0 * (1 + 2 * s) / p1);
    t[3] = c * (dx * (p0 / (p1 * p1)));
    t[4] = c * (dy * (p0 / (p1 * p1)));
    t[5] = c * (dz * (p0 / (p1 * p1)));
    const double p13 = pow(p1, 3.0), p14 = pow(p1, 4.0), p15 = pow(p1, 5.0);
    double* h = t + 6;
    h[up(0, 0)] = 0;
    h[up(0, 1)] = -es * (1 + 2 * s) / (p1 * p1 * r2pi);
    h[up(0, 2)] = es * dx / (p13 * r2pi);
    h[up(0, 3)] = es * dy / (p13 * r2pi);
    h[up(0, 4)] = es * dz / (p13 * r2pi);
    h[up(1, 1)] = 2 * p0 * es * (1 + 5 * s + 2 * s * s) / (p13 * r2pi);
    h[up(1, 2)] = -p0 * es * (3 + 2 * s) * dx / (p14 * r2pi);
    h[up(1, 3)] = -p0 * es * (3 + 2 * s) * dy / (p14 * r2pi);
    h[up(1, 4)] = -p0 * es * (3 + 2 * s) * dz / (p14 * r2pi);
    h[up(2, 2)] = p0 * es * (dx * dx - p1 * p1) / (r2pi * p15);
    h[up(3, 3)] = p0 * es * (dy * dy - p1 * p1) / (r2pi * p15);
    h[up(4, 4)] = p0 * es * (dz * dz - p1 * p1) / (r2pi * p15);
    h[up(2, 3)] = p0 * es * dx * dy / (r2pi * p15);
    h[up(2, 4)] = p0 * es * dx * dz / (r2pi * p15);
    h[up(3, 4)] = p0 * es * dy * dz / (r2pi * p15);
}

// part[c][q][22], q = f * S + i: the chunk's sums for frame f of sample i
// spot_scale 1: the samples lack the spot (e = d - (s + v)); 0: they hold it
// already (e = d - s, FreeEnergyHessian).
__global__ void __launch_bounds__(kPartThreads) hess_parts_kernel(const double* __restrict__ bg,
                                                                   const double* __restrict__ pix,
                                                                   const double* __restrict__ tab, int S, int F, int P,
                                                                   int chunk, double spot_scale,
                                                                   double* __restrict__ part) {
    const long long q = (long long)blockIdx.x * kPartThreads + threadIdx.x;
    const long long nq = (long long)S * F;
    if (q >= nq) return;
    const int f = (int)(q / S), i = (int)(q % S);
    const int p0 = blockIdx.y * chunk, p1 = min(P, p0 + chunk);
    const double* d = pix + (size_t)f * P;
    const double* b = bg + ((size_t)i * F + f) * P;
    double on = 0.0, off = 0.0, acc[20];
#pragma unroll
    for (int n = 0; n < 20; ++n) acc[n] = 0.0;
    for (int p = p0; p < p1; ++p) {
        const double* t = tab + (size_t)p * kTab;
        const double dv = __ldg(d + p), sv = __ldg(b + p);
        const double e = dv - (sv + spot_scale * __ldg(t));
        on += e * e;
        const double o = dv - sv;
        off += o * o;
#pragma unroll
        for (int n = 0; n < 15; ++n) acc[n] = fma(e, __ldg(t + 6 + n), acc[n]);
#pragma unroll
        for (int n = 0; n < 5; ++n) acc[15 + n] = fma(e, __ldg(t + 1 + n), acc[15 + n]);
    }
    double* out = part + ((size_t)blockIdx.y * nq + q) * kParts;
    out[0] = on;
    out[1] = off;
#pragma unroll
    for (int n = 0; n < 20; ++n) out[2 + n] = acc[n];
}

// sum_p g_p g_p^T (15 upper entries) by one CTA, in thread order
__global__ void __launch_bounds__(kFfbsThreads) hess_gg_kernel(const double* __restrict__ tab, int P,
                                                                double* __restrict__ gg) {
    __shared__ double red[kFfbsThreads / 32][15];
    double acc[15];
#pragma unroll
    for (int n = 0; n < 15; ++n) acc[n] = 0.0;
    for (int p = threadIdx.x; p < P; p += kFfbsThreads) {
        const double* g = tab + (size_t)p * kTab + 1;
        int n = 0;
#pragma unroll
        for (int a = 0; a < 5; ++a)
#pragma unroll
            for (int b2 = a; b2 < 5; ++b2) acc[n++] += g[a] * g[b2];
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int n = 0; n < 15; ++n) {
        double v = acc[n];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[w][n] = v;
    }
    __syncthreads();
    if (threadIdx.x < 15) {
        double v = 0.0;
        for (int k = 0; k < kFfbsThreads / 32; ++k) v += red[k][threadIdx.x];
        gg[threadIdx.x] = v;
    }
}

struct FfbsArgs {
    const double* part;  // [NC][S * F][22]
    const double* gg;    // [15]
    double* frame;       // [S][F][20] scratch: the frames' Hessian and gradient parts
    double* out;         // [S][20]: sum over walks of hess + deriv deriv^T (15), deriv (5)
    int S, F, P, nc, bs;
    double variance;
    double A[9], pi[3];
    unsigned long long seed;
};

__global__ void __launch_bounds__(kFfbsThreads) hess_ffbs_kernel(const FfbsArgs a) {
    extern __shared__ double hsm[];
    const int F = a.F, S = a.S, i = blockIdx.x;
    float2* xs = reinterpret_cast<float2*>(hsm);             // [F][3]
    float2* emf = xs + (size_t)3 * F;                        // [F][2]
    float2* thr = emf + (size_t)2 * F;                       // [F][4]: cumulative thresholds of states 0, 1
    int* es = reinterpret_cast<int*>(thr + (size_t)4 * F);   // [F][3]
    int* emk = es + (size_t)3 * F;                           // [F][2]
    __shared__ double red[kFfbsThreads / 32][20];
    double* fr = a.frame + (size_t)i * F * 20;
    const size_t nq = (size_t)S * F;
    const double log_norm = a.P * log(2 * 3.14159265358979323846 * a.variance) / 2;
    // chunk sums in chunk order; the frame's emission terms and parts
    for (int f = threadIdx.x; f < F; f += kFfbsThreads) {
        const size_t q = (size_t)f * S + i;
        double v[kParts];
#pragma unroll
        for (int n = 0; n < kParts; ++n) v[n] = 0.0;
        for (int c = 0; c < a.nc; ++c) {
            const double* pc = a.part + ((size_t)c * nq + q) * kParts;
#pragma unroll
            for (int n = 0; n < kParts; ++n) v[n] += pc[n];
        }
        const double lon = -v[0] / (2 * a.variance) - log_norm;
        const double loff = -v[1] / (2 * a.variance) - log_norm;
        ffbs::emission_terms(lon, loff, emf + 2 * f, emk + 2 * f);
#pragma unroll
        for (int n = 0; n < 15; ++n) fr[(size_t)f * 20 + n] = v[2 + n] - a.gg[n];
#pragma unroll
        for (int n = 0; n < 5; ++n) fr[(size_t)f * 20 + 15 + n] = v[17 + n];
    }
    __syncthreads();
    if (threadIdx.x < 32) ffbs::forward_filter(threadIdx.x, F, a.A, a.pi, emf, emk, xs, es);
    __syncthreads();
    // thresholds of every frame for each state of the next frame (3: none)
    float Af[9];
    unsigned nzA;
    ffbs::transition_floats(a.A, Af, &nzA);
    for (int e = threadIdx.x; e < 4 * F; e += kFfbsThreads) thr[e] = ffbs::frame_thresholds(e >> 2, e & 3, xs, es, Af, nzA);
    __syncthreads();
    // backward walks
    double accH[15], accD[5];
#pragma unroll
    for (int n = 0; n < 15; ++n) accH[n] = 0.0;
#pragma unroll
    for (int n = 0; n < 5; ++n) accD[n] = 0.0;
    for (int w = threadIdx.x; w < a.bs; w += kFfbsThreads) {
        double H[15], D[5];
#pragma unroll
        for (int n = 0; n < 15; ++n) H[n] = 0.0;
#pragma unroll
        for (int n = 0; n < 5; ++n) D[n] = 0.0;
        int next = 3;
        for (int t = F - 1; t >= 0; --t) {
            uint32_t cc[4] = {(uint32_t)t, (uint32_t)w, (uint32_t)i, 0x48455353u};
            Philox::gen(cc, (uint32_t)a.seed, (uint32_t)(a.seed >> 32));
            const unsigned long long U = ffbs::uniform53(cc[0], cc[1]);
            const int st = ffbs::draw_state(U, thr[4 * t + next]);
            next = st;
            if (st == 0) {
                const double* p = fr + (size_t)t * 20;
#pragma unroll
                for (int n = 0; n < 15; ++n) H[n] += p[n];
#pragma unroll
                for (int n = 0; n < 5; ++n) D[n] += p[15 + n];
            }
        }
        int n = 0;
#pragma unroll
        for (int r = 0; r < 5; ++r)
#pragma unroll
            for (int c = r; c < 5; ++c, ++n) accH[n] += H[n] + D[r] * D[c];
#pragma unroll
        for (int r = 0; r < 5; ++r) accD[r] += D[r];
    }
    const int wp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int n = 0; n < 20; ++n) {
        double v = n < 15 ? accH[n] : accD[n - 15];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[wp][n] = v;
    }
    __syncthreads();
    if (threadIdx.x < 20) {
        double v = 0.0;
        for (int k = 0; k < kFfbsThreads / 32; ++k) v += red[k][threadIdx.x];
        a.out[(size_t)i * 20 + threadIdx.x] = v;
    }
}

size_t ffbs_smem(int F) { return (size_t)F * (24 + 16 + 32 + 12 + 8); }

}  // namespace

int hessian_chunks(long long S, long long F, int P, int sm_count) {
    const long long want = (long long)sm_count * 16 * 32;  // threads enough to cover the SMs a few times
    long long nc = (want + S * F - 1) / (S * F);
    if (nc < 1) nc = 1;
    if (nc > 64) nc = 64;
    if (nc > P) nc = P;
    return (int)nc;
}

size_t hessian_ffbs_smem(int F) { return ffbs_smem(F); }

int launch_hessian_parts(const HessParams& h, bool samples_hold_spot, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    hess_table_kernel<<<(h.P + 127) / 128, 128, 0, st>>>(h.pixels, h.P, h.phi, h.zf, h.tab);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return (int)e;
    const int chunk = (h.P + h.nc - 1) / h.nc;
    const long long nq = (long long)h.S * h.F;
    hess_parts_kernel<<<dim3((unsigned)((nq + kPartThreads - 1) / kPartThreads), (unsigned)h.nc), kPartThreads, 0, st>>>(
        h.bg, h.pix, h.tab, h.S, h.F, h.P, chunk, samples_hold_spot ? 0.0 : 1.0, h.part);
    if ((e = cudaGetLastError()) != cudaSuccess) return (int)e;
    hess_gg_kernel<<<1, kFfbsThreads, 0, st>>>(h.tab, h.P, h.gg);
    return (int)cudaGetLastError();
}

int launch_spot_hessian(const HessParams& h, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = (cudaError_t)launch_hessian_parts(h, false, stream);
    if (e != cudaSuccess) return (int)e;
    FfbsArgs a;
    a.part = h.part;
    a.gg = h.gg;
    a.frame = h.frame;
    a.out = h.out;
    a.S = h.S;
    a.F = h.F;
    a.P = h.P;
    a.nc = h.nc;
    a.bs = h.bs;
    a.variance = h.variance;
    for (int n = 0; n < 9; ++n) a.A[n] = h.A[n];
    for (int n = 0; n < 3; ++n) a.pi[n] = h.pi[n];
    a.seed = h.seed;
    const size_t smem = ffbs_smem(h.F);
    if ((e = cudaFuncSetAttribute(hess_ffbs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
        cudaSuccess)
        return (int)e;
    hess_ffbs_kernel<<<h.S, kFfbsThreads, smem, st>>>(a);
    return (int)cudaGetLastError();
}

}  // namespace rfba

// 3B spot gradient with sampled backgrounds (sm_103a, FP64).
//
// The derivative of the negative log probability of one spot with respect to
// its parameters (brightness, blur, x, y, z), given S samples of the other
// spots' intensities, which 3B's conjugate-gradient spot optimiser evaluates
// over and over: SpotNegProbabilityDiffWithSampledBackground::operator()
// (RFBA Main/multispot5.cc:616-664). Four kernels:
//   1. spot_pixels_kernel: the spot's intensity and its parameter derivative
//      at every mask voxel (spot_shape_diff_position, storm.h:51-84);
//   2. spot_sums_kernel: the spot's sums over the mask (sum v^2, sum der v);
//   3. emission_kernel, one CTA per (sample, frame): the frame's log
//      probability with the spot on and off and the derivative of the "on" one
//      (SpotWithBackground, spot_with_background.hh:98-133), reduced over the
//      mask voxels in FP64 — the sums of squares reach 1e7-1e8 while the
//      forward algorithm weighs states by exp of their differences, so FP32
//      sums would be wrong by whole units of log probability;
//   4. forward_kernel, one warp per state of each sample: the 3-state forward algorithm
//      with derivatives over the frames (forward_algorithm.h:157-259,
//      compute_hessian = 0), giving each sample's log probability and gradient.
// The host averages the samples' gradients and adds the log-normal priors'
// derivatives (storm.h:431-434).
#include <cuda_runtime.h>

#include "srrf_internal.h"

namespace rfba {
namespace {

constexpr int kM = 5;
constexpr int kEmitThreads = 256;

// forward_algorithm.h:34-40
__device__ __forceinline__ double ln0(double x) { return x == 0.0 ? -1e100 : log(x); }

__global__ void spot_pixels_kernel(const int* __restrict__ pixels, int P, const double* __restrict__ phi_in,
                                   double zf, double* __restrict__ val, double* __restrict__ der) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const double phi0 = phi_in[0], phi1 = phi_in[1], phi2 = phi_in[2], phi3 = phi_in[3], phi4 = phi_in[4];
    const double x0 = pixels[3 * p], x1 = pixels[3 * p + 1], x2 = pixels[3 * p + 2];
    const double d0 = x0 - phi2, d1 = x1 - phi3, d2 = (x2 - phi4) / zf;
    const double s = -(d0 * d0 + d1 * d1 + d2 * d2) / (2 * phi1 * phi1);
    const double r_2_pi = sqrt(2 * 3.14159265358979323846);
    const double es = exp(s);
    val[p] = es * phi0 / (phi1 * r_2_pi);
    const double k = es / (phi1 * r_2_pi);
    const double q = phi0 / (phi1 * phi1);
    double* d = der + (size_t)p * kM;
    d[0] = k;
    d[1] = k * (-phi0 * (1 + 2 * s) / phi1);
    d[2] = k * ((x0 - phi2) * q);
    d[3] = k * ((x1 - phi3) * q);
    d[4] = k * ((x2 - phi4) * q);
}

// The spot's own sums over the mask, sum v^2 and sum der_n v (one CTA, fixed
// order): with d = I - G, sum (d - v)^2 = sum d^2 - 2 sum d v + sum v^2 and
// sum der_n (d - v) = sum der_n d - sum der_n v, so the per-(sample, frame)
// pass needs 8 FP64 operations per voxel instead of 10.
constexpr int kSumThreads = 512;
__global__ void __launch_bounds__(kSumThreads) spot_sums_kernel(const double* __restrict__ val,
                                                                 const double* __restrict__ der, int P,
                                                                 double* __restrict__ sums) {
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int p = threadIdx.x; p < P; p += kSumThreads) {
        const double v = val[p];
        acc[0] += v * v;
#pragma unroll
        for (int n = 0; n < kM; ++n) acc[1 + n] += der[(size_t)p * kM + n] * v;
    }
#pragma unroll
    for (int i = 0; i < 6; ++i)
        for (int o = 16; o > 0; o >>= 1) acc[i] += __shfl_down_sync(0xffffffffu, acc[i], o);
    __shared__ double part[kSumThreads / 32][6];
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int i = 0; i < 6; ++i) part[threadIdx.x >> 5][i] = acc[i];
    __syncthreads();
    if (threadIdx.x == 0) {
        double t[6] = {0, 0, 0, 0, 0, 0};
        for (int w = 0; w < kSumThreads / 32; ++w)
#pragma unroll
            for (int i = 0; i < 6; ++i) t[i] += part[w][i];
#pragma unroll
        for (int i = 0; i < 6; ++i) sums[i] = t[i];
    }
}

// out[(s*F + f)*8 + {0: log prob on, 1: log prob off, 2..6: d(log prob on)/d phi}]
__global__ void __launch_bounds__(kEmitThreads) emission_kernel(const double* __restrict__ bg,
                                                                 const double* __restrict__ pix,
                                                                 const double* __restrict__ val,
                                                                 const double* __restrict__ der,
                                                                 const double* __restrict__ spot_sums, int F, int P,
                                                                 double twovar, double var, double c0,
                                                                 double* __restrict__ out) {
    const int sf = blockIdx.x;  // sample * F + frame
    const int f = sf % F;
    const double* G = bg + (size_t)sf * P;
    const double* I = pix + (size_t)f * P;
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};  // sum d v, sum d^2, sum der_n d (d = I - G)
    for (int p = threadIdx.x; p < P; p += kEmitThreads) {
        const double dI = I[p] - G[p];
        acc[1] += dI * dI;
        acc[0] += dI * val[p];
        const double* d = der + (size_t)p * kM;
#pragma unroll
        for (int n = 0; n < kM; ++n) acc[2 + n] += d[n] * dI;
    }
#pragma unroll
    for (int i = 0; i < 7; ++i)
        for (int o = 16; o > 0; o >>= 1) acc[i] += __shfl_down_sync(0xffffffffu, acc[i], o);
    __shared__ double part[kEmitThreads / 32][7];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < 7; ++i) part[warp][i] = acc[i];
    __syncthreads();
    if (threadIdx.x == 0) {
        double t[7] = {0, 0, 0, 0, 0, 0, 0};
        for (int w = 0; w < kEmitThreads / 32; ++w)
#pragma unroll
            for (int i = 0; i < 7; ++i) t[i] += part[w][i];
        double* o = out + (size_t)sf * 8;
        const double on = t[1] - 2.0 * t[0] + spot_sums[0];  // sum (d - v)^2
        o[0] = -on / twovar - c0;
        o[1] = -t[1] / twovar - c0;
#pragma unroll
        for (int n = 0; n < kM; ++n) o[2 + n] = (t[2 + n] - spot_sums[1 + n]) / var;
        o[7] = 0.0;
    }
}

// One CTA per sample, one warp per state j: each step every warp holds the
// previous delta_i and its derivative for all i, forms its own state's new
// values (forward_algorithm.h:196-224) and the three warps exchange them
// through shared memory. exp is skipped where its argument is exactly 0 (the
// largest term of each sum: exp(0) = 1) or carries ln(0) = -1e100 (the
// transitions the model forbids: exp = 0), which changes no result. lnA
// row-major 3 x 3 and lnpi with ln(0) = -1e100 as the reference's ln.
__device__ __forceinline__ double exp_term(double a) {
    return a == 0.0 ? 1.0 : (a < -1e99 ? 0.0 : exp(a));
}

__global__ void __launch_bounds__(96) forward_kernel(const double* __restrict__ em, int S, int F,
                                                      const double* __restrict__ lnA9,
                                                      const double* __restrict__ lnpi3, double* __restrict__ res) {
    // one warp per state j; the new delta_j and its derivative go through
    // shared memory (double-buffered, one barrier per frame)
    __shared__ double sh[2][3][8];
    const int s = blockIdx.x;
    const int j = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    double lnAj[3];
    for (int i = 0; i < 3; ++i) lnAj[i] = lnA9[i * 3 + j];
    const double* e = em + (size_t)s * F * 8;
    double delta[3], dd[3][kM];
    for (int i = 0; i < 3; ++i) {
        delta[i] = lnpi3[i] + (i == 0 ? e[0] : e[1]);
        for (int n = 0; n < kM; ++n) dd[i][n] = i == 0 ? e[2 + n] : 0.0;
    }
    for (int t = 1; t < F; ++t) {
        const double* et = e + (size_t)t * 8;
        double Z = -__longlong_as_double(0x7ff0000000000000ll);
        for (int i = 0; i < 3; ++i) Z = fmax(Z, delta[i] + lnAj[i]);
        double w[3], sum = 0.0;
        for (int i = 0; i < 3; ++i) {
            w[i] = exp_term(delta[i] + lnAj[i] - Z);
            sum += w[i];
        }
        const double nd = (j == 0 ? et[0] : et[1]) + Z + ln0(sum);
        double top[kM] = {0, 0, 0, 0, 0};
        for (int i = 0; i < 3; ++i)
            for (int n = 0; n < kM; ++n) top[n] += dd[i][n] * w[i];
        double* o = sh[t & 1][j];
        if (lane == 0) {
            // one reciprocal instead of five divisions (FP64 division is a long
            // sequence here); the products differ from the quotients by an ulp
            const double rs = 1.0 / sum;
            o[0] = nd;
            for (int n = 0; n < kM; ++n) o[1 + n] = (j == 0 ? et[2 + n] : 0.0) + top[n] * rs;
        }
        __syncthreads();
        for (int i = 0; i < 3; ++i) {
            const double* q = sh[t & 1][i];
            delta[i] = q[0];
            for (int n = 0; n < kM; ++n) dd[i][n] = q[1 + n];
        }
    }
    if (threadIdx.x != 0) return;
    double Z = -__longlong_as_double(0x7ff0000000000000ll);
    for (int i = 0; i < 3; ++i) Z = fmax(Z, delta[i]);
    double sum = 0.0;
    for (int i = 0; i < 3; ++i) sum += exp(delta[i] - Z);
    const double logp = Z + ln0(sum);
    double g[kM] = {0, 0, 0, 0, 0};
    for (int i = 0; i < 3; ++i) {
        const double w = exp(delta[i] - logp);
        for (int n = 0; n < kM; ++n) g[n] += w * dd[i][n];
    }
    double* r = res + (size_t)s * 6;
    for (int n = 0; n < kM; ++n) r[n] = g[n];
    r[5] = logp;
}

}  // namespace

int launch_threeb(const double* bg, const double* pix, const int* pixels, int S, int F, int P, const double* phi_dev,
                  double zf, double variance, double c0, const double* lnA_dev, const double* lnpi_dev,
                  double* val, double* der, double* em, double* res, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    spot_pixels_kernel<<<(P + 255) / 256, 256, 0, st>>>(pixels, P, phi_dev, zf, val, der);
    double* sums = res + (size_t)S * 6;  // 6 doubles after the per-sample results
    spot_sums_kernel<<<1, kSumThreads, 0, st>>>(val, der, P, sums);
    emission_kernel<<<(unsigned)((long long)S * F), kEmitThreads, 0, st>>>(bg, pix, val, der, sums, F, P,
                                                                           2 * variance, variance, c0, em);
    forward_kernel<<<S, 96, 0, st>>>(em, S, F, lnA_dev, lnpi_dev, res);
    return (int)cudaGetLastError();
}

}  // namespace rfba

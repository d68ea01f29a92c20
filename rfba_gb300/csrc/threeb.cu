// 3B spot gradient with sampled backgrounds (sm_103a, FP64).
//
// The derivative of the negative log probability of one spot with respect to
// its parameters (brightness, blur, x, y, z), given S samples of the other
// spots' intensities, which 3B's conjugate-gradient spot optimiser evaluates
// over and over: SpotNegProbabilityDiffWithSampledBackground::operator()
// (RFBA Main/multispot5.cc:616-664). Three kernels:
//   1. spot_pixels_kernel: the spot's intensity and its parameter derivative
//      at every mask voxel (spot_shape_diff_position, storm.h:51-84);
//   2. emission_kernel, one CTA per (sample, frame): the frame's log
//      probability with the spot on and off and the derivative of the "on" one
//      (SpotWithBackground, spot_with_background.hh:98-133), reduced over the
//      mask voxels in FP64 — the sums of squares reach 1e7-1e8 while the
//      forward algorithm weighs states by exp of their differences, so FP32
//      sums would be wrong by whole units of log probability;
//   3. forward_kernel, one warp per sample (a lane per state): the 3-state forward algorithm
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

// out[(s*F + f)*8 + {0: log prob on, 1: log prob off, 2..6: d(log prob on)/d phi}]
__global__ void __launch_bounds__(kEmitThreads) emission_kernel(const double* __restrict__ bg,
                                                                 const double* __restrict__ pix,
                                                                 const double* __restrict__ val,
                                                                 const double* __restrict__ der, int F, int P,
                                                                 double twovar, double var, double c0,
                                                                 double* __restrict__ out) {
    const int sf = blockIdx.x;  // sample * F + frame
    const int f = sf % F;
    const double* G = bg + (size_t)sf * P;
    const double* I = pix + (size_t)f * P;
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};  // on, off, diff[5]
    for (int p = threadIdx.x; p < P; p += kEmitThreads) {
        const double dI = I[p] - G[p];
        const double e = I[p] - (G[p] + val[p]);
        acc[1] += dI * dI;
        acc[0] += e * e;
        const double* d = der + (size_t)p * kM;
#pragma unroll
        for (int n = 0; n < kM; ++n) acc[2 + n] += d[n] * e;
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
        o[0] = -t[0] / twovar - c0;
        o[1] = -t[1] / twovar - c0;
#pragma unroll
        for (int n = 0; n < kM; ++n) o[2 + n] = t[2 + n] / var;
        o[7] = 0.0;
    }
}

// One warp per sample, lanes 0..2 the three states j: each step every lane
// holds the previous delta_i and its derivative for all i, forms its own
// state's new values (forward_algorithm.h:196-224) and the three lanes
// exchange them by shuffles. exp is skipped where its argument is exactly 0
// (the largest term of each sum: exp(0) = 1) or carries ln(0) = -1e100 (the
// transitions the model forbids: exp = 0), which changes no result. lnA
// row-major 3 x 3 and lnpi with ln(0) = -1e100 as the reference's ln.
__device__ __forceinline__ double exp_term(double a) {
    return a == 0.0 ? 1.0 : (a < -1e99 ? 0.0 : exp(a));
}

__global__ void __launch_bounds__(32) forward_kernel(const double* __restrict__ em, int S, int F,
                                                      const double* __restrict__ lnA9,
                                                      const double* __restrict__ lnpi3, double* __restrict__ res) {
    const int s = blockIdx.x;
    const int lane = threadIdx.x;
    if (s >= S) return;
    const int j = lane < 3 ? lane : 0;
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
        double ndd[kM];
        for (int n = 0; n < kM; ++n) ndd[n] = (j == 0 ? et[2 + n] : 0.0) + top[n] / sum;
        for (int i = 0; i < 3; ++i) {
            delta[i] = __shfl_sync(0xffffffffu, nd, i);
            for (int n = 0; n < kM; ++n) dd[i][n] = __shfl_sync(0xffffffffu, ndd[n], i);
        }
    }
    if (lane != 0) return;
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
    emission_kernel<<<(unsigned)((long long)S * F), kEmitThreads, 0, st>>>(bg, pix, val, der, F, P,
                                                                           2 * variance, variance, c0, em);
    forward_kernel<<<S, 32, 0, st>>>(em, S, F, lnA_dev, lnpi_dev, res);
    return (int)cudaGetLastError();
}

}  // namespace rfba

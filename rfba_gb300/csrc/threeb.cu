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
//   4. forward_kernel, one warp per sample: the 3-state forward algorithm
//      with derivatives over the frames (forward_algorithm.h:157-259,
//      compute_hessian = 0), giving each sample's log probability and gradient.
//      The reference runs it in log space (a log-sum-exp per state and frame);
//      here it runs on probabilities, each state's value kept as a mantissa and
//      its own power-of-two exponent: the same sums with no exp or log inside
//      the sequential chain, and no underflow however far apart the states'
//      probabilities drift (an absorbing state can hold all the mass while the
//      frames start to favour a state it cannot reach).
// The host averages the samples' gradients and adds the log-normal priors'
// derivatives (storm.h:431-434).
//
// The spot optimiser evaluates the gradient thousands of times on the same
// samples and needs no log probability, so for it the samples' residuals
// (data minus background) are staged once as double-float numbers
// (residual_df_kernel) and emission_df_kernel forms the gradient's sums
// (sum d v, sum der_n d) on the FP32 pipe in double-float arithmetic, about
// 2^-46 relative per operation, four samples of a frame per CTA so the spot's
// table is read once per four, over the spot's support only (the pixels where
// its Gaussian factor is at least 2^-60, listed in pixel order by
// support_compact_kernel); forward_df_kernel runs the recursion in
// double-float too. The FP64 pipe, 1/64 of the FP32 one here, would otherwise
// bound every evaluation. The log-probability path keeps the FP64 sums over
// every pixel.
#include <cuda_runtime.h>

#include "dfloat.cuh"
#include "srrf_internal.h"

namespace rfba {
namespace {

constexpr int kM = 5;
constexpr int kEmitThreads = 256;
// The double-float path sums only over the spot's support: the pixels where
// its Gaussian factor exp(s) is at least 2^-60 (terms below that are far under
// the 2^-46 resolution of the double-float sums they would join).
constexpr double kSupportS = -41.58883083359672;  // ln(2^-60)

using namespace dfloat;

constexpr int kPixThreads = 256;
__global__ void __launch_bounds__(kPixThreads) spot_pixels_kernel(const int* __restrict__ pixels, int P,
                                                                   const double* __restrict__ phi_in, double zf,
                                                                   double* __restrict__ val, double* __restrict__ der,
                                                                   float2* __restrict__ vdf,
                                                                   double* __restrict__ partial,
                                                                   unsigned char* __restrict__ support) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    double acc[6] = {0, 0, 0, 0, 0, 0};  // this pixel's v^2 and der_n v
    if (p < P) {
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
        if (support) support[p] = s >= kSupportS;
        if (vdf) {  // value and derivative as double-floats: [P][6]
            float2* o = vdf + (size_t)p * 6;
            o[0] = df_from(val[p]);
#pragma unroll
            for (int n = 0; n < kM; ++n) o[1 + n] = df_from(d[n]);
        }
        const double v = val[p];
        acc[0] = v * v;
#pragma unroll
        for (int n = 0; n < kM; ++n) acc[1 + n] = d[n] * v;
    }
    // the block's share of the spot's sums, in a fixed order
#pragma unroll
    for (int i = 0; i < 6; ++i)
        for (int o = 16; o > 0; o >>= 1) acc[i] += __shfl_down_sync(0xffffffffu, acc[i], o);
    __shared__ double part[kPixThreads / 32][6];
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int i = 0; i < 6; ++i) part[threadIdx.x >> 5][i] = acc[i];
    __syncthreads();
    if (threadIdx.x < 6) {
        double t = 0;
        for (int w = 0; w < kPixThreads / 32; ++w) t += part[w][threadIdx.x];
        partial[(size_t)blockIdx.x * 6 + threadIdx.x] = t;
    }
}

// The samples' residuals, data minus background, as double-floats [S][F][P].
__global__ void residual_df_kernel(const double* __restrict__ bg, const double* __restrict__ pix, int F, int P,
                                   long long n, float2* __restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long fp = i % ((long long)F * P);
    out[i] = df_from(pix[fp] - bg[i]);
}

// The spot's own sums over the mask, sum v^2 and sum der_n v, from the
// blocks' partial sums in block order (one thread per sum): with d = I - G,
// sum (d - v)^2 = sum d^2 - 2 sum d v + sum v^2 and sum der_n (d - v) =
// sum der_n d - sum der_n v, so the per-(sample, frame) pass needs 8 FP64
// operations per voxel instead of 10.
__global__ void spot_sums_kernel(const double* __restrict__ partial, int nblocks, double* __restrict__ sums) {
    if (threadIdx.x >= 6) return;
    double t = 0;
    for (int b = 0; b < nblocks; ++b) t += partial[(size_t)b * 6 + threadIdx.x];
    sums[threadIdx.x] = t;
}

// The support's pixel indices in pixel order (one CTA): each thread counts a
// contiguous run of flags, a block-wide exclusive scan places the runs, and
// the indices are written in order; count[0] = the support's size.
constexpr int kScanThreads = 1024;
__global__ void __launch_bounds__(kScanThreads) support_compact_kernel(const unsigned char* __restrict__ flag, int P,
                                                                        int* __restrict__ idx,
                                                                        int* __restrict__ count) {
    const int per = (P + kScanThreads - 1) / kScanThreads;
    const int p0 = min(P, threadIdx.x * per), p1 = min(P, p0 + per);
    int n = 0;
    for (int q = p0; q < p1; ++q) n += flag[q];
    // inclusive scan of n over the block
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int v = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    __shared__ int wsum[kScanThreads / 32];
    if (lane == 31) wsum[warp] = v;
    __syncthreads();
    if (warp == 0) {
        int w = wsum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += u;
        }
        wsum[lane] = w;
    }
    __syncthreads();
    int base = v - n + (warp > 0 ? wsum[warp - 1] : 0);
    for (int q = p0; q < p1; ++q)
        if (flag[q]) idx[base++] = q;
    if (threadIdx.x == kScanThreads - 1) count[0] = base;
}

// Per (sample, frame), kEm doubles: the frame's emission probabilities relative
// to the larger of the two, exp(log p_on - m) = mant_on 2^k_on and likewise for
// off (one of them is exactly 1), d(log p_on)/d phi, and m itself:
// {0: mant_on, 1: mant_off, 2: k_on, 3: k_off, 4..8: d(log p_on)/d phi, 9: m}.
constexpr int kEm = 10;

// exp(x) = mant 2^k for x <= 0 (mant in about [1, 2)); x = k ln2 + r with r
// formed by one fused multiply-add, whose error (|k| ulp-sized) is far below
// the log-space reference's own rounding. Probabilities below 2^-(2^24)
// relative are 0.
__device__ __forceinline__ void exp_split(double x, double* mant, double* k) {
    const double kd = floor(x * 1.4426950408889634);
    if (kd < -16777216.0) {
        *mant = 0.0;
        *k = 0.0;
        return;
    }
    *mant = exp(fma(-kd, 0.6931471805599453, x));
    *k = kd;
}

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
        double* o = out + (size_t)sf * kEm;
        // log p_on = -sum (d - v)^2 / 2var - c0, log p_off = -sum d^2 / 2var - c0;
        // their difference is formed without the large common terms
        const double off = -t[1] / twovar - c0;
        const double gap = (2.0 * t[0] - spot_sums[0]) / twovar;  // log p_on - log p_off
        if (gap <= 0.0) {
            exp_split(gap, &o[0], &o[2]);
            o[1] = 1.0;
            o[3] = 0.0;
            o[9] = off;
        } else {
            o[0] = 1.0;
            o[2] = 0.0;
            exp_split(-gap, &o[1], &o[3]);
            o[9] = off + gap;
        }
#pragma unroll
        for (int n = 0; n < kM; ++n) o[4 + n] = (t[2 + n] - spot_sums[1 + n]) / var;
    }
}

// A frame's emission terms for the double-float forward recursion: the
// mantissas (double-float) and exponents of p(on) and p(off) relative to the
// larger one, and d(log p_on)/d phi.
struct __align__(16) EmDf {
    float2 mant[2];
    int k[2];
    float2 q[kM];
};

// The gradient's emission terms from the double-float residuals, kDfTile
// samples of one frame per CTA (blockIdx.x = frame, blockIdx.y = sample
// tile): per sample sum d v and sum der_n d in double-float, then the terms
// emission_kernel forms except the frame's level (used by the log probability
// only), written as double-floats for forward_df_kernel.
constexpr int kDfTile = 4;
__global__ void __launch_bounds__(kEmitThreads) emission_df_kernel(const float2* __restrict__ dfd,
                                                                    const float2* __restrict__ vdf,
                                                                    const int* __restrict__ sup,
                                                                    const int* __restrict__ nsup,
                                                                    const double* __restrict__ spot_sums, int S, int F,
                                                                    int P, double twovar, double var,
                                                                    EmDf* __restrict__ out) {
    const int f = blockIdx.x, s0 = blockIdx.y * kDfTile;
    const int ns = min(kDfTile, S - s0);
    float2 acc[kDfTile][6];
#pragma unroll
    for (int a = 0; a < kDfTile; ++a)
#pragma unroll
        for (int n = 0; n < 6; ++n) acc[a][n] = make_float2(0.f, 0.f);
    const int n = *nsup;
    for (int i = threadIdx.x; i < n; i += kEmitThreads) {
        const int p = __ldg(sup + i);
        // every load of the iteration goes out before its arithmetic (a tile's
        // missing samples read 0 and add 0)
        float2 w[6], d[kDfTile];
#pragma unroll
        for (int a = 0; a < kDfTile; ++a)
            d[a] = a < ns ? __ldg(dfd + ((size_t)(s0 + a) * F + f) * P + p) : make_float2(0.f, 0.f);
#pragma unroll
        for (int n = 0; n < 6; ++n) w[n] = __ldg(vdf + (size_t)p * 6 + n);
#pragma unroll
        for (int a = 0; a < kDfTile; ++a)
#pragma unroll
            for (int n = 0; n < 6; ++n) df_acc_mul(acc[a][n], w[n], d[a]);
    }
#pragma unroll
    for (int a = 0; a < kDfTile; ++a)
#pragma unroll
        for (int n = 0; n < 6; ++n) acc[a][n] = df_two_sum(acc[a][n].x, acc[a][n].y);
    __shared__ float2 part[kEmitThreads / 32][kDfTile][6];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int a = 0; a < kDfTile; ++a)
#pragma unroll
        for (int n = 0; n < 6; ++n) {
            float2 v = acc[a][n];
            for (int o = 16; o > 0; o >>= 1) {
                float2 u;
                u.x = __shfl_down_sync(0xffffffffu, v.x, o);
                u.y = __shfl_down_sync(0xffffffffu, v.y, o);
                v = df_add(v, u);
            }
            if (lane == 0) part[warp][a][n] = v;
        }
    __syncthreads();
    if (threadIdx.x < ns) {
        const int a = threadIdx.x;
        double t[6];
#pragma unroll
        for (int n = 0; n < 6; ++n) {
            float2 v = part[0][a][n];
            for (int w = 1; w < kEmitThreads / 32; ++w) v = df_add(v, part[w][a][n]);
            t[n] = df_to(v);
        }
        EmDf* o = out + (size_t)(s0 + a) * F + f;
        const double gap = (2.0 * t[0] - spot_sums[0]) / twovar;  // log p_on - log p_off
        double m[2], k[2];
        if (gap <= 0.0) {
            exp_split(gap, &m[0], &k[0]);
            m[1] = 1.0;
            k[1] = 0.0;
        } else {
            m[0] = 1.0;
            k[0] = 0.0;
            exp_split(-gap, &m[1], &k[1]);
        }
        EmDf r;
        for (int i = 0; i < 2; ++i) {
            r.mant[i] = df_from(m[i]);
            r.k[i] = (int)k[i];
        }
#pragma unroll
        for (int n = 0; n < kM; ++n) r.q[n] = df_from((t[1 + n] - spot_sums[1 + n]) / var);
        *o = r;
    }
}

// One warp per sample. Lane l < 18 holds state j = l / 6 and component k =
// l % 6: k < 5 the derivative part D_jk = alpha_j dd_jk, k = 5 the probability
// alpha_j, both as x_jk 2^E_j with x_j5 in [0.5, 1) (E_j = kZeroExp when
// alpha_j = 0); lanes 18..31 repeat lanes 0..13. In the reference's terms
// alpha_j = exp(delta_j) up to a common factor and dd_jk is its derivative
// table, so per frame t (forward_algorithm.h:196-224)
//   alpha_j <- p_j(t) sum_i A_ij alpha_i,
//   D_jk    <- p_j(t) sum_i A_ij D_ik + [j = on] alpha_j d(log p_on(t))/d phi_k,
// and at the end log P = log sum_j alpha_j and the gradient is
// sum_j D_jk / sum_j alpha_j (forward_algorithm.h:240-259). The sum over i is
// aligned to the largest exponent among the states that can move to j; terms
// more than 2^1022 below it are dropped (the reference's exp underflows there).
constexpr int kZeroExp = -(1 << 29);

__device__ __forceinline__ double pow2i(int d) {  // 2^d for -1022 <= d <= 1023
    return __hiloint2double((d + 1023) << 20, 0);
}

__global__ void __launch_bounds__(32) forward_kernel(const double* __restrict__ em, int S, int F,
                                                      const double* __restrict__ A9,
                                                      const double* __restrict__ pi3, double* __restrict__ res) {
    const int s = blockIdx.x;
    const int lane = threadIdx.x;
    const int l = lane % 18;
    const int j = l / 6, k = l % 6;
    const unsigned full = 0xffffffffu;
    double Aj[3];
    bool nz[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        Aj[i] = A9[i * 3 + j];
        nz[i] = Aj[i] != 0.0;
    }
    const double* e = em + (size_t)s * F * kEm;
    // sum over the frames of the reference level m (lanes in parallel)
    double base = 0.0;
    for (int t = lane; t < F; t += 32) base += e[(size_t)t * kEm + 9];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) base += __shfl_xor_sync(full, base, o);

    const int mi = j == 0 ? 0 : 1;  // the bleached state emits like "off"
    const int ki = j == 0 ? 2 : 3;
    const bool has_de = j == 0 && k < 5;
    // normalise the new values y of this lane's state by the exponent of its
    // probability lane; returns the state's new exponent
    auto normalise = [&](double y, int Ebase, double* x) {
        const double y5 = __shfl_sync(full, y, j * 6 + 5);
        const int hi = __double2hiint(y5), lo = __double2loint(y5);
        if (hi == 0 && lo == 0) {
            *x = y;
            return kZeroExp;
        }
        const int sh = ((hi >> 20) & 0x7ff) - 1022;  // y5 = m 2^sh, m in [0.5, 1)
        *x = y * pow2i(-sh);
        return Ebase + sh;
    };
    // frame 0: alpha_j = pi_j p_j(0)
    double x;
    int E[3];
    {
        const double a = pi3[j] * e[mi];
        const double y = k == 5 ? a : (has_de ? a * e[4 + k] : 0.0);
        const int En = normalise(y, (int)e[ki], &x);
#pragma unroll
        for (int i = 0; i < 3; ++i) E[i] = __shfl_sync(full, En, i * 6 + 5);
    }
    // the next frame's loads go out one frame ahead
    double nm = 0.0, nk = 0.0, nq = 0.0;
    if (F > 1) {
        const double* et = e + kEm;
        nm = et[mi];
        nk = et[ki];
        nq = has_de ? et[4 + k] : 0.0;
    }
    for (int t = 1; t < F; ++t) {
        const double mant = nm, q = nq;
        const int ke = (int)nk;
        if (t + 1 < F) {
            const double* et = e + (size_t)(t + 1) * kEm;
            nm = et[mi];
            nk = et[ki];
            nq = has_de ? et[4 + k] : 0.0;
        }
        int Em = kZeroExp;
#pragma unroll
        for (int i = 0; i < 3; ++i)
            if (nz[i] && E[i] > Em) Em = E[i];
        double c[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const int d = E[i] - Em;
            c[i] = (d >= -1022 && d <= 0) ? Aj[i] * pow2i(d) : 0.0;
        }
        double xi[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) xi[i] = __shfl_sync(full, x, i * 6 + k);
        double y = fma(c[2], xi[2], fma(c[1], xi[1], c[0] * xi[0])) * mant;
        const double y05 = __shfl_sync(full, y, 5);
        y = fma(y05, q, y);
        const int En = normalise(y, Em + ke, &x);
#pragma unroll
        for (int i = 0; i < 3; ++i) E[i] = __shfl_sync(full, En, i * 6 + 5);
    }
    // log P and the gradient, the states aligned to the largest exponent
    const int Em = max(E[0], max(E[1], E[2]));
    const int d = E[j] - Em;
    const double v = (d >= -1022) ? x * pow2i(d) : 0.0;
    const double tot = v + __shfl_sync(full, v, (lane + 6) & 31) + __shfl_sync(full, v, (lane + 12) & 31);
    const double den = __shfl_sync(full, tot, 5);
    double* r = res + (size_t)s * 6;
    if (lane < 5) r[lane] = tot / den;
    if (lane == 5) r[5] = base + log(den) + (double)Em * 0.6931471805599453;
}

// The forward recursion of forward_kernel in double-float arithmetic, for
// the gradient only (the log probability is not formed): each lane's value a
// double-float mantissa with the state's exponent, the same alignment to the
// largest exponent among the states that reach j, terms more than 2^100 below
// it dropped (below the format's precision).
__global__ void __launch_bounds__(32) forward_df_kernel(const EmDf* __restrict__ em, int S, int F,
                                                         const double* __restrict__ A9, const double* __restrict__ pi3,
                                                         double* __restrict__ res) {
    const int s = blockIdx.x;
    const int lane = threadIdx.x;
    const int l = lane % 18;
    const int j = l / 6, k = l % 6;
    const unsigned full = 0xffffffffu;
    float2 Aj[3];
    bool nz[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        Aj[i] = df_from(A9[i * 3 + j]);
        nz[i] = A9[i * 3 + j] != 0.0;
    }
    const EmDf* e = em + (size_t)s * F;
    const int mi = j == 0 ? 0 : 1;  // the bleached state emits like "off"
    const bool has_de = j == 0 && k < 5;
    auto shfl2 = [&](float2 v, int src) {
        return make_float2(__shfl_sync(full, v.x, src), __shfl_sync(full, v.y, src));
    };
    // normalise the new values y of this lane's state by the exponent of its
    // probability lane; returns the state's new exponent
    // (branch-free: the lanes of a state whose probability is 0 must not
    // diverge from the others)
    auto normalise = [&](float2 y, int Ebase, float2* x) {
        const float2 y5 = shfl2(y, j * 6 + 5);
        const int ex = (__float_as_int(y5.x) >> 23) & 0xff;
        const bool zero = y5.x == 0.f || ex == 0 || Ebase == kZeroExp;
        const int sh = ex - 126;  // y5 = m 2^sh, m in [0.5, 1)
        const float sc = zero ? 1.f : pow2f(-sh);
        *x = make_float2(y.x * sc, y.y * sc);
        return zero ? kZeroExp : Ebase + sh;
    };
    float2 x;
    int E[3];
    {
        const float2 a = df_mul(df_from(pi3[j]), e[0].mant[mi]);
        const float2 y = k == 5 ? a : (has_de ? df_mul(a, e[0].q[k]) : make_float2(0.f, 0.f));
        const int En = normalise(y, pi3[j] == 0.0 ? kZeroExp : e[0].k[mi], &x);
#pragma unroll
        for (int i = 0; i < 3; ++i) E[i] = __shfl_sync(full, En, i * 6 + 5);
    }
    // the frames' terms pass through shared memory 32 at a time: the next
    // chunk is loaded into registers while this one is used, and stored at
    // its end (a chain step is shorter than a load's latency)
    const int kq = k < 5 ? k : 0;
    const float qmask = has_de ? 1.f : 0.f;
    __shared__ __align__(16) EmDf chunk[2][32];
    float4 nxt[4];
    auto fetch = [&](int c) {
        const int t = c * 32 + lane;
        const float4* src = reinterpret_cast<const float4*>(e + (t < F ? t : F - 1));
#pragma unroll
        for (int w = 0; w < 4; ++w) nxt[w] = src[w];
    };
    auto store = [&](int slot) {
        float4* dst = reinterpret_cast<float4*>(&chunk[slot][lane]);
#pragma unroll
        for (int w = 0; w < 4; ++w) dst[w] = nxt[w];
    };
    const int nchunk = (F + 31) / 32;
    fetch(0);
    store(0);
    __syncwarp();
    for (int c = 0; c < nchunk; ++c) {
        if (c + 1 < nchunk) fetch(c + 1);
        const EmDf* cur = chunk[c & 1];
        const int t1 = min(F, c * 32 + 32);
        for (int t = max(1, c * 32); t < t1; ++t) {
            const EmDf& et = cur[t - c * 32];
            const float2 mant = et.mant[mi];
            const float2 qv = et.q[kq];
            const float2 q = make_float2(qv.x * qmask, qv.y * qmask);
            const int ke = et.k[mi];
            int Em = kZeroExp;
#pragma unroll
            for (int i = 0; i < 3; ++i) Em = (nz[i] && E[i] > Em) ? E[i] : Em;
            float2 y = make_float2(0.f, 0.f);
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const float2 xi = shfl2(x, i * 6 + k);
                const int d = E[i] - Em;
                const bool use = nz[i] && E[i] != kZeroExp && d >= -100;
                const float sc = use ? pow2f(d < -126 ? -126 : d) : 0.f;
                float2 tm = df_mul(Aj[i], xi);
                tm.x *= sc;
                tm.y *= sc;
                y = df_add(y, tm);
            }
            y = df_mul(y, mant);
            const float2 y05 = shfl2(y, 5);
            y = df_add(y, df_mul(y05, q));
            const int En = normalise(y, (Em == kZeroExp || ke == kZeroExp) ? kZeroExp : Em + ke, &x);
#pragma unroll
            for (int i = 0; i < 3; ++i) E[i] = __shfl_sync(full, En, i * 6 + 5);
        }
        __syncwarp();
        if (c + 1 < nchunk) store((c + 1) & 1);
        __syncwarp();
    }
    // the gradient, the states aligned to the largest exponent
    const int Em = max(E[0], max(E[1], E[2]));
    const int d = E[j] - Em;
    const double v = (d >= -1022 && E[j] != kZeroExp) ? df_to(x) * ldexp(1.0, d) : 0.0;
    const double tot = v + __shfl_sync(full, v, (lane + 6) & 31) + __shfl_sync(full, v, (lane + 12) & 31);
    const double den = __shfl_sync(full, tot, 5);
    double* r = res + (size_t)s * 6;
    if (lane < 5) r[lane] = tot / den;
    if (lane == 5) r[5] = 0.0;
}

}  // namespace

int launch_threeb_residual(const double* bg, const double* pix, int S, int F, int P, float2* dfd, void* stream) {
    const long long n = (long long)S * F * P;
    if (n == 0) return 0;
    residual_df_kernel<<<(unsigned)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(bg, pix, F, P, n,
                                                                                                    dfd);
    return (int)cudaGetLastError();
}

int launch_threeb(const double* bg, const double* pix, const int* pixels, int S, int F, int P, const double* phi_dev,
                  double zf, double variance, double c0, const double* A_dev, const double* pi_dev,
                  double* val, double* der, double* em, double* res, const float2* dfd, float2* vdf, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nblk = (P + kPixThreads - 1) / kPixThreads;
    double* sums = res + (size_t)S * 6;  // 6 doubles after the per-sample results, then the blocks' partials
    // the double-float path's support flags and list share the table's buffer:
    // vdf [P][6] float2, then P flag bytes, then the P indices and the count
    unsigned char* flag = dfd ? reinterpret_cast<unsigned char*>(vdf + (size_t)P * 6) : nullptr;
    int* sup = dfd ? reinterpret_cast<int*>(flag + (((size_t)P + 15) & ~(size_t)15)) : nullptr;
    spot_pixels_kernel<<<nblk, kPixThreads, 0, st>>>(pixels, P, phi_dev, zf, val, der, dfd ? vdf : nullptr,
                                                     sums + 6, flag);
    spot_sums_kernel<<<1, 32, 0, st>>>(sums + 6, nblk, sums);
    if (dfd) {
        support_compact_kernel<<<1, kScanThreads, 0, st>>>(flag, P, sup, sup + P);
        EmDf* emd = reinterpret_cast<EmDf*>(em);  // 64 B per (sample, frame), within the FP64 path's 80
        emission_df_kernel<<<dim3((unsigned)F, (unsigned)((S + kDfTile - 1) / kDfTile)), kEmitThreads, 0, st>>>(
            dfd, vdf, sup, sup + P, sums, S, F, P, 2 * variance, variance, emd);
        forward_df_kernel<<<S, 32, 0, st>>>(emd, S, F, A_dev, pi_dev, res);
        return (int)cudaGetLastError();
    }
    emission_kernel<<<(unsigned)((long long)S * F), kEmitThreads, 0, st>>>(bg, pix, val, der, sums, F, P,
                                                                           2 * variance, variance, c0, em);
    forward_kernel<<<S, 32, 0, st>>>(em, S, F, A_dev, pi_dev, res);
    return (int)cudaGetLastError();
}

}  // namespace rfba

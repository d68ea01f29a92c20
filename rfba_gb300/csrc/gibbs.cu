// 3B Gibbs sampling of the spot states (sm_103a, FP64).
//
// GibbsSampler2::next (RFBA Main/sampled_multispot.h:658-690) draws the
// on / off / bleached state of every spot in every frame given the spots'
// positions and the data, one spot at a time: remove the spot from the
// current sample's intensities (over the spot's mask, in the frames where it
// is on), compute each frame's log probability with the spot on and off over
// its mask (SpotWithBackgroundMasked, spot_with_background.hh:98-137), run the
// forward filter of the 3-state chain (forward_algorithm_delta2,
// forward_algorithm.h:385-431), draw the state sequence backwards
// (backward_sampling, forward_algorithm.h:546-570) and add the spot back with
// its new states. NegativeFreeEnergy (multispot5.cc:335-405) runs the same
// sampler under a slowly growing noise variance; FitSpots (multispot5.cc:
// 1591-1604) keeps its draws as the background samples of the spot optimiser.
//
// One cooperative kernel runs a whole chain: the frames are dealt out to the
// CTAs, which do the per-frame work (remove / add over the mask, the two sums
// of squares, the emission probabilities) in parallel; after a grid barrier
// one warp of every CTA runs the forward filter and the backward draw over all
// frames from the same emission table and random counters (so every CTA draws
// the same states, and no second barrier is needed), and every CTA adds the
// spot back into its own frames. A frame's state is only ever read by the CTA
// that owns the frame, and the emission table alternates between two buffers
// from one spot update to the next. The filter runs
// on probabilities, each state's value a mantissa with its own power-of-two
// exponent (no exp or log in the sequential chain; the frames' emission terms
// are split into mantissa and exponent in parallel beforehand), which is the
// reference's log-space recursion in other coordinates. The draw uses
// Philox4x32-10 keyed by the caller's seed with counter (frame, spot, sweep,
// draw): the reference's distribution, not its MT19937 stream. Grid barriers
// wait at most about two seconds of %globaltimer, then record a failure and
// leave the kernel.
#include <cuda_runtime.h>
#include <cstdint>

#include "philox.h"
#include "srrf_internal.h"

namespace rfba {
namespace {

constexpr int kGibbsThreads = 256;
constexpr int kZeroExp = -(1 << 29);
constexpr unsigned long long kBarrierNs = 2000000000ull;

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ double pow2i(int d) {  // 2^d, -1022 <= d <= 1023
    return __hiloint2double((d + 1023) << 20, 0);
}

// exp(x) = mant 2^k for x <= 0 (mant in [1, 2)): x = k ln2 + r with r by one
// fused multiply-add. Relative probabilities below 2^-(2^24) are 0.
__device__ __forceinline__ void exp_split(double x, double* mant, int* k) {
    const double kd = floor(x * 1.4426950408889634);
    if (kd < -16777216.0) {
        *mant = 0.0;
        *k = kZeroExp;
        return;
    }
    *mant = exp(fma(-kd, 0.6931471805599453, x));
    *k = (int)kd;
}

// Grid barrier over co-resident CTAs (cooperative launch). False when the
// wait gave up; the caller then leaves the kernel.
__device__ bool grid_barrier(unsigned int* count, unsigned int* gen, unsigned int nblocks) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        s_ok = 1;
        __threadfence();
        const unsigned int g = *((volatile unsigned int*)gen);
        if (atomicAdd(count, 1u) == nblocks - 1) {
            atomicExch(count, 0u);
            __threadfence();
            atomicAdd(gen, 1u);
        } else {
            const unsigned long long t0 = gtimer();
            int i = 0;
            while (*((volatile unsigned int*)gen) == g) {
                if ((++i & 63) == 0 && gtimer() - t0 > kBarrierNs) {
                    s_ok = 0;
                    break;
                }
                if (i > (1 << 30)) {
                    s_ok = 0;
                    break;
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
    return s_ok != 0;
}

__device__ __forceinline__ double block_sum(double v, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < kGibbsThreads / 32; ++i) t += red[i];
    return t;  // valid in thread 0
}

__global__ void __launch_bounds__(kGibbsThreads) gibbs_chain_kernel(const GibbsParams g) {
    extern __shared__ double gsm[];
    // shared: per frame and state the forward value's mantissa and exponent,
    // the frame's uniform for the backward draw, the frames' emission terms,
    // and the spot's drawn states
    double* xs = gsm;                                          // [F][3]
    int* es = reinterpret_cast<int*>(xs + (size_t)3 * g.F);    // [F][3]
    double* us = reinterpret_cast<double*>(es + ((3 * g.F + 1) & ~1));  // [F]
    double* emc = us + g.F;                                    // [F][4]
    unsigned char* sts = reinterpret_cast<unsigned char*>(emc + (size_t)4 * g.F);  // [F]
    __shared__ double red[kGibbsThreads / 32];
    const int c = blockIdx.x, G = gridDim.x;
    const int F = g.F, P = g.P, K = g.K;
    // states and emission terms cross CTAs: read them past L1
    const volatile unsigned char* vstate = g.state;

    for (int d = 0; d < g.n_draws; ++d) {
        const double var = g.var_draw ? g.var_draw[d] : g.variance;
        const double twovar = 2 * var;
        for (int it = 0; it < g.sweeps; ++it) {
            for (int k = 0; k < K; ++k) {
                // the emission table alternates between two buffers from one spot
                // update to the next: a CTA can start writing the next update's
                // terms while a slower one still reads this update's
                const unsigned long long upd = ((unsigned long long)d * g.sweeps + it) * K + k;
                double* emb = g.em + (size_t)(upd & 1) * 4 * F;
                const int m0 = g.moff[k], m1 = g.moff[k + 1];
                const int npix = m1 - m0;
                const double* vk = g.si + (size_t)k * P;
                const double cst = npix * log(2 * 3.14159265358979323846 * var) / 2;
                // phase A: remove spot k where it is on; the frame's two sums
                for (int f = c; f < F; f += G) {
                    const bool on = vstate[(size_t)k * F + f] == 0;
                    double* cur = g.cur + (size_t)f * P;
                    const double* dat = g.pix + (size_t)f * P;
                    double soff = 0.0, son = 0.0;
                    for (int q = m0 + threadIdx.x; q < m1; q += kGibbsThreads) {
                        const int p = g.midx[q];
                        const double v = vk[p];
                        double cv = cur[p];
                        if (on) {
                            cv -= v;
                            cur[p] = cv;
                        }
                        const double e0 = dat[p] - cv;
                        const double e1 = dat[p] - (cv + v);
                        soff += e0 * e0;
                        son += e1 * e1;
                    }
                    const double toff = block_sum(soff, red);
                    const double ton = block_sum(son, red);
                    if (threadIdx.x == 0) {
                        const double lon = -ton / twovar - cst;
                        const double loff = -toff / twovar - cst;
                        const double m = lon > loff ? lon : loff;
                        double mo, mf;
                        int ko, kf;
                        exp_split(lon - m, &mo, &ko);
                        exp_split(loff - m, &mf, &kf);
                        double* em = emb + (size_t)f * 4;
                        em[0] = mo;
                        em[1] = (double)ko;
                        em[2] = mf;
                        em[3] = (double)kf;
                        if (g.rec_lp && d == 0 && it == 0) {
                            g.rec_lp[((size_t)k * F + f) * 2] = lon;
                            g.rec_lp[((size_t)k * F + f) * 2 + 1] = loff;
                        }
                    }
                }
                if (!grid_barrier(g.bar, g.bar + 1, G)) {
                    if (threadIdx.x == 0) atomicCAS(g.err, 0ull, (0x47ull << 56) | (unsigned long long)k);
                    return;
                }
                // phase B: forward filter and backward draw, run by warp 0 of every
                // CTA on the same inputs and counters, so every CTA draws the same
                // states and only the barrier above is needed per spot
                if (threadIdx.x < 32) {
                    const int lane = threadIdx.x;
                    const unsigned full = 0xffffffffu;
                    for (int i = lane; i < 4 * F; i += 32) emc[i] = __ldcg(emb + i);
                    // uniforms of this spot's draw, one per frame
                    const unsigned long long ctr = (unsigned long long)d * g.sweeps + it + g.draw_base;
                    for (int f = lane; f < F; f += 32) {
                        uint32_t cc[4] = {(uint32_t)f, (uint32_t)k, (uint32_t)ctr, (uint32_t)(ctr >> 32)};
                        Philox::gen(cc, (uint32_t)g.seed, (uint32_t)(g.seed >> 32));
                        us[f] = u53(cc[0], cc[1]);
                    }
                    __syncwarp();
                    // the recursion runs on the three lanes that carry a state; the
                    // FP64 pipe of this GPU is narrow, so the other lanes stay idle
                    if (lane < 3) {
                        const unsigned m3 = 0x7u;
                        const int j = lane;
                        double Aj[3];
                        bool nz[3];
#pragma unroll
                        for (int i = 0; i < 3; ++i) {
                            Aj[i] = g.A[i * 3 + j];
                            nz[i] = Aj[i] != 0.0;
                        }
                        const int mi = j == 0 ? 0 : 2;  // "off" and bleached emit alike
                        // frame 0
                        double x;
                        int E;
                        {
                            const double y = g.pi[j] * emc[mi];
                            if (y == 0.0) {
                                x = 0.0;
                                E = kZeroExp;
                            } else {
                                int sh;
                                x = frexp(y, &sh);
                                E = (int)emc[mi + 1] + sh;
                            }
                        }
                        xs[j] = x;
                        es[j] = E;
                        int Ev[3];
#pragma unroll
                        for (int i = 0; i < 3; ++i) Ev[i] = __shfl_sync(m3, E, i);
                        for (int t = 1; t < F; ++t) {
                            const double mant = emc[(size_t)t * 4 + mi];
                            const int ke = (int)emc[(size_t)t * 4 + mi + 1];
                            int Em = kZeroExp;
#pragma unroll
                            for (int i = 0; i < 3; ++i)
                                if (nz[i] && Ev[i] > Em) Em = Ev[i];
                            double xi[3];
#pragma unroll
                            for (int i = 0; i < 3; ++i) xi[i] = __shfl_sync(m3, x, i);
                            double y = 0.0;
#pragma unroll
                            for (int i = 0; i < 3; ++i) {
                                const int dd = Ev[i] - Em;
                                if (nz[i] && dd >= -1022) y = fma(Aj[i] * pow2i(dd), xi[i], y);
                            }
                            y *= mant;
                            if (y == 0.0 || Em == kZeroExp || ke == kZeroExp) {
                                x = 0.0;
                                E = kZeroExp;
                            } else {
                                int sh;
                                x = frexp(y, &sh);
                                E = Em + ke + sh;
                            }
                            xs[(size_t)t * 3 + j] = x;
                            es[(size_t)t * 3 + j] = E;
#pragma unroll
                            for (int i = 0; i < 3; ++i) Ev[i] = __shfl_sync(m3, E, i);
                        }
                    }
                    __syncwarp();
                    // filtering distribution per frame (trace mode, first sweep)
                    if (c == 0 && g.rec_filt && d == 0 && it == 0) {
                        for (int t = lane; t < F; t += 32) {
                            const int* e3 = es + (size_t)t * 3;
                            const int Em = max(e3[0], max(e3[1], e3[2]));
                            double w[3], tot = 0.0;
                            for (int i = 0; i < 3; ++i) {
                                const int dd = e3[i] - Em;
                                w[i] = dd >= -1022 ? xs[(size_t)t * 3 + i] * pow2i(dd) : 0.0;
                                tot += w[i];
                            }
                            for (int i = 0; i < 3; ++i) g.rec_filt[((size_t)k * F + t) * 3 + i] = w[i] / tot;
                        }
                    }
                    // backward draw (select_random_element on the unscaled weights).
                    // The lanes first tabulate, for every frame and each state the
                    // next frame may hold (index 3: none, for the last frame), the
                    // cumulative thresholds of states 0 and 1 as fractions of the
                    // total; the sequential walk then only compares its uniform
                    // with a table entry. The table reuses the emission staging area.
                    float2* thr = reinterpret_cast<float2*>(emc);  // [F][4]
                    for (int t = lane; t < F; t += 32) {
                        const double* x3 = xs + (size_t)t * 3;
                        const int* e3 = es + (size_t)t * 3;
                        for (int nx = 0; nx < 4; ++nx) {
                            int Em = kZeroExp;
                            for (int i = 0; i < 3; ++i)
                                if ((nx == 3 || g.A[i * 3 + nx] != 0.0) && x3[i] != 0.0 && e3[i] > Em) Em = e3[i];
                            double a[3], tot = 0.0;
                            for (int i = 0; i < 3; ++i) {
                                const double tr = nx == 3 ? 1.0 : g.A[i * 3 + nx];
                                const int dd = e3[i] - Em;
                                a[i] = (tr != 0.0 && x3[i] != 0.0 && dd >= -1022) ? x3[i] * pow2i(dd) * tr : 0.0;
                                tot += a[i];
                            }
                            // no weight at all: the walk takes state 0, as a zero total does
                            thr[(size_t)t * 4 + nx] =
                                tot > 0.0 ? make_float2((float)(a[0] / tot), (float)((a[0] + a[1]) / tot))
                                          : make_float2(1.f, 1.f);
                        }
                    }
                    __syncwarp();
                    if (lane == 0) {
                        int next = 3;
                        for (int t = F - 1; t >= 0; --t) {
                            const float2 th = thr[(size_t)t * 4 + next];
                            const double u = us[t];
                            const int sdraw = u <= (double)th.x ? 0 : (u <= (double)th.y ? 1 : 2);
                            sts[t] = (unsigned char)sdraw;
                            next = sdraw;
                        }
                    }
                }
                __syncthreads();
                // phase C: record the drawn states of this CTA's frames and add spot
                // k back where it is on
                for (int f = c; f < F; f += G) {
                    if (threadIdx.x == 0) g.state[(size_t)k * F + f] = sts[f];
                    if (sts[f] != 0) continue;
                    double* cur = g.cur + (size_t)f * P;
                    for (int q = m0 + threadIdx.x; q < m1; q += kGibbsThreads) {
                        const int p = g.midx[q];
                        cur[p] += vk[p];
                    }
                }
                __syncthreads();
            }
        }
        // the draw: states, intensities (optionally without one spot), the sum
        // of squared residuals over all pixels
        for (int f = c; f < F; f += G) {
            if (g.out_state)
                for (int k = threadIdx.x; k < K; k += kGibbsThreads)
                    g.out_state[((size_t)d * K + k) * F + f] = vstate[(size_t)k * F + f];
            const double* cur = g.cur + (size_t)f * P;
            const bool ex = g.exclude_spot >= 0 && vstate[(size_t)g.exclude_spot * F + f] == 0;
            const double* vx = ex ? g.si + (size_t)g.exclude_spot * P : nullptr;
            double* o = g.out_int ? g.out_int + ((size_t)d * F + f) * P : nullptr;
            const double* dat = g.pix + (size_t)f * P;
            double se = 0.0;
            for (int p = threadIdx.x; p < P; p += kGibbsThreads) {
                const double cv = cur[p];
                if (o) o[p] = ex ? cv - vx[p] : cv;
                const double e = dat[p] - cv;
                se += e * e;
            }
            if (g.out_err) {
                const double t = block_sum(se, red);
                if (threadIdx.x == 0) g.out_err[(size_t)d * F + f] = t;
            }
        }
        __syncthreads();
    }
}

// Spot intensities at every pixel (compute_spot_intensity with spot_shape,
// storm.h:229-235): exp(s) * brightness / (blur sqrt(2 pi)), s = -|x - mu|^2 /
// (2 blur^2) with the z difference divided by the z factor.
__global__ void spot_intensity_kernel(const int* __restrict__ pixels, int P, const double* __restrict__ spots, int K,
                                      double zf, double* __restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)K * P) return;
    const int k = (int)(i / P), p = (int)(i % P);
    const double* phi = spots + (size_t)k * 5;
    const double d0 = pixels[3 * p] - phi[2], d1 = pixels[3 * p + 1] - phi[3], d2 = (pixels[3 * p + 2] - phi[4]) / zf;
    const double s = -(d0 * d0 + d1 * d1 + d2 * d2) / (2 * phi[1] * phi[1]);
    const double r_2_pi = sqrt(2 * 3.14159265358979323846);
    out[i] = exp(s) * phi[0] / (phi[1] * r_2_pi);
}

}  // namespace

size_t gibbs_smem_bytes(int F) {
    return (size_t)F * 3 * sizeof(double) + (size_t)((3 * F + 1) & ~1) * sizeof(int) + (size_t)F * sizeof(double) +
           (size_t)F * 4 * sizeof(double) + (size_t)F;
}

int gibbs_max_blocks(int F, int* out) {
    const size_t smem = gibbs_smem_bytes(F);
    cudaError_t e = cudaFuncSetAttribute(gibbs_chain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    int dev = 0, sms = 0, per = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return (int)e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return (int)e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, gibbs_chain_kernel, kGibbsThreads, smem)) !=
        cudaSuccess)
        return (int)e;
    *out = per * sms;
    return 0;
}

int launch_gibbs(const GibbsParams& p, int grid, void* stream) {
    const size_t smem = gibbs_smem_bytes(p.F);
    cudaError_t e = cudaFuncSetAttribute(gibbs_chain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    GibbsParams q = p;
    void* args[] = {&q};
    e = cudaLaunchCooperativeKernel((const void*)gibbs_chain_kernel, dim3(grid), dim3(kGibbsThreads), args, smem,
                                    static_cast<cudaStream_t>(stream));
    return (int)e;
}

int launch_spot_intensity(const int* pixels, int P, const double* spots, int K, double zf, double* out, void* stream) {
    const long long n = (long long)K * P;
    if (n == 0) return 0;
    spot_intensity_kernel<<<(unsigned)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(pixels, P, spots,
                                                                                                      K, zf, out);
    return (int)cudaGetLastError();
}

}  // namespace rfba

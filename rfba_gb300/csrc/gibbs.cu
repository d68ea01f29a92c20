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
// One cooperative kernel runs a whole chain (or several independent chains
// side by side, each on its own share of the CTAs): the frames are dealt out to the
// CTAs, which do the per-frame work (remove / add over the mask, the two sums
// of squares, the emission terms) in parallel; after a grid barrier one warp
// of every CTA runs the forward filter and the backward draw over all frames
// from the same emission table and random counters (so every CTA draws the
// same states, and no second barrier is needed), and every CTA adds the spot
// back into its own frames. A frame's state is only ever read by the CTA that
// owns the frame, and the emission table alternates between two buffers from
// one spot update to the next. The filter and the draw's thresholds are those
// of ffbs.cuh (double-float forward values with power-of-two exponents; the
// draw a walk through a per-frame decision table, each entry the state the
// frame takes for each state of the next frame). The draw uses Philox4x32-10
// keyed by the caller's seed with counter (frame, spot, sweep, draw): the
// reference's distribution, not its MT19937 stream. The grid barrier counts
// arrivals on a counter that only grows and waits at most about two seconds
// of %globaltimer, then records a failure and leaves the kernel.
#include <cuda_runtime.h>
#include <cstdint>

#include "ffbs.cuh"
#include "philox.h"
#include "srrf_internal.h"

namespace rfba {
namespace {

using ffbs::kZeroExp;

constexpr int kGibbsThreads = 256;
constexpr int kBatch = 8;  // mask pixels a thread gathers at once
constexpr unsigned long long kBarrierNs = 2000000000ull;

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid barrier over co-resident CTAs (cooperative launch) on a counter that
// only grows: barrier b (0, 1, ...) is passed once the counter reaches
// (b + 1) * nblocks. False when the wait gave up; the caller then leaves the
// kernel.
__device__ bool grid_barrier(unsigned int* count, unsigned int target) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        s_ok = 1;
        __threadfence();
        atomicAdd(count, 1u);
        const unsigned long long t0 = gtimer();
        int i = 0;
        for (;;) {
            unsigned int v;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(count) : "memory");
            if ((int)(v - target) >= 0) break;
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
    __syncthreads();
    return s_ok != 0;
}

// Sums of a and b over the CTA, valid in thread 0.
__device__ __forceinline__ void block_sum2(double& a, double& b, double2* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[w] = make_double2(a, b);
    __syncthreads();
    if (w == 0) {
        double2 v = lane < kGibbsThreads / 32 ? red[lane] : make_double2(0.0, 0.0);
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) {
            v.x += __shfl_down_sync(0xffffffffu, v.x, o);
            v.y += __shfl_down_sync(0xffffffffu, v.y, o);
        }
        a = v.x;
        b = v.y;
    }
}

// A frame's emission terms as phase A publishes them for phase B.
struct EmFrame {
    float2 m[2];  // double-float mantissas: on, off
    int k[2];     // exponents: on, off
    int pad[2];
};

// Several independent chains may share one launch: chain i runs on CTAs
// [i G, (i + 1) G) with its own parameters, scratch and barrier counter.
__global__ void __launch_bounds__(kGibbsThreads) gibbs_chain_kernel(const GibbsParams* __restrict__ chains,
                                                                     int nchains) {
    extern __shared__ double gsm[];
    const int G = gridDim.x / nchains;
    const int c = blockIdx.x % G;
    const GibbsParams& g = chains[blockIdx.x / G];
    const int F = g.F, P = g.P, K = g.K;
    // shared: per frame and state the forward value (double-float mantissa,
    // exponent), the frames' emission terms, the backward draw's decision table
    // (drawn state per frame and next state) and the spot's drawn states
    float2* xs = reinterpret_cast<float2*>(gsm);   // [F][3]
    float2* emf = xs + (size_t)3 * F;              // [F][2]
    int* es = reinterpret_cast<int*>(emf + (size_t)2 * F);  // [F][3]
    int* emk = es + (size_t)3 * F;                 // [F][2]
    unsigned char* sel = reinterpret_cast<unsigned char*>(emk + (size_t)2 * F);  // [F][4]
    unsigned char* sts = sel + (size_t)4 * F;      // [F]
    __shared__ double2 red[kGibbsThreads / 32];
    // states and emission terms cross CTAs: read them past L1
    const volatile unsigned char* vstate = g.state;
    EmFrame* em_all = reinterpret_cast<EmFrame*>(g.em);
    float Af[9];
    unsigned nzA;
    ffbs::transition_floats(g.A, Af, &nzA);

    for (int d = 0; d < g.n_draws; ++d) {
        const double var = g.var_draw ? g.var_draw[d] : g.variance;
        const double twovar = 2 * var;
        const double log_norm = log(2 * 3.14159265358979323846 * var);
        for (int it = 0; it < g.sweeps; ++it) {
            for (int k = 0; k < K; ++k) {
                // the emission table alternates between two buffers from one spot
                // update to the next: a CTA can start writing the next update's
                // terms while a slower one still reads this update's
                const unsigned long long upd = ((unsigned long long)d * g.sweeps + it) * K + k;
                EmFrame* emb = em_all + (size_t)(upd & 1) * F;
                const int m0 = g.moff[k], m1 = g.moff[k + 1];
                const int npix = m1 - m0;
                const double* vk = g.si + (size_t)k * P;
                const double cst = npix * log_norm / 2;
                // phase A: remove spot k where it is on; the frame's two sums
                for (int f = c; f < F; f += G) {
                    const bool on = vstate[(size_t)k * F + f] == 0;
                    double* cur = g.cur + (size_t)f * P;
                    const double* dat = g.pix + (size_t)f * P;
                    double soff = 0.0, son = 0.0;
                    for (int q0 = m0 + threadIdx.x; q0 < m1; q0 += kGibbsThreads * kBatch) {
                        // a spot's mask holds no pixel twice, so the gathers of one
                        // batch are independent of its stores
                        int pp[kBatch];
                        double v[kBatch], cv[kBatch], dv[kBatch];
#pragma unroll
                        for (int b = 0; b < kBatch; ++b) {
                            const int q = q0 + b * kGibbsThreads;
                            pp[b] = q < m1 ? __ldg(g.midx + q) : -1;
                        }
#pragma unroll
                        for (int b = 0; b < kBatch; ++b) {
                            const int p = pp[b] < 0 ? 0 : pp[b];
                            v[b] = __ldg(vk + p);
                            cv[b] = cur[p];
                            dv[b] = __ldg(dat + p);
                        }
#pragma unroll
                        for (int b = 0; b < kBatch; ++b) {
                            if (pp[b] < 0) continue;
                            if (on) {
                                cv[b] -= v[b];
                                cur[pp[b]] = cv[b];
                            }
                            const double e0 = dv[b] - cv[b];
                            const double e1 = dv[b] - (cv[b] + v[b]);
                            soff += e0 * e0;
                            son += e1 * e1;
                        }
                    }
                    block_sum2(soff, son, red);
                    if (threadIdx.x == 0) {
                        const double lon = -son / twovar - cst;
                        const double loff = -soff / twovar - cst;
                        EmFrame fr;
                        ffbs::emission_terms(lon, loff, fr.m, fr.k);
                        fr.pad[0] = fr.pad[1] = 0;
                        emb[f] = fr;
                        if (g.rec_lp && d == 0 && it == 0) {
                            g.rec_lp[((size_t)k * F + f) * 2] = lon;
                            g.rec_lp[((size_t)k * F + f) * 2 + 1] = loff;
                        }
                    }
                }
                if (!grid_barrier(g.bar, (unsigned int)((upd + 1) * (unsigned long long)G))) {
                    if (threadIdx.x == 0) atomicCAS(g.err, 0ull, (0x47ull << 56) | (unsigned long long)k);
                    return;
                }
                // phase B: forward filter and backward draw, run by every CTA on the
                // same inputs and counters, so every CTA draws the same states and
                // only the barrier above is needed per spot. The emission terms are
                // staged and the decision table filled by all threads; the filter
                // (warp 0) and the walk through the table (thread 0) are sequential.
                for (int t = threadIdx.x; t < F; t += kGibbsThreads) {
                    const float4 a = __ldcg(reinterpret_cast<const float4*>(emb + t));
                    const int4 b = __ldcg(reinterpret_cast<const int4*>(emb + t) + 1);
                    emf[2 * t] = make_float2(a.x, a.y);
                    emf[2 * t + 1] = make_float2(a.z, a.w);
                    emk[2 * t] = b.x;
                    emk[2 * t + 1] = b.y;
                }
                __syncthreads();
                if (threadIdx.x < 32) ffbs::forward_filter(threadIdx.x, F, g.A, g.pi, emf, emk, xs, es);
                __syncthreads();
                // filtering distribution per frame (trace mode, first sweep)
                if (c == 0 && g.rec_filt && d == 0 && it == 0)
                    for (int t = threadIdx.x; t < F; t += kGibbsThreads)
                        ffbs::filter_probs(t, xs, es, g.rec_filt + ((size_t)k * F + t) * 3);
                // decision table: the state frame t draws for each state the next
                // frame holds, from the frame's uniform (counter: frame, spot, sweep
                // and draw)
                const unsigned long long ctr = (unsigned long long)d * g.sweeps + it + g.draw_base;
                for (int t = threadIdx.x; t < F; t += kGibbsThreads) {
                    uint32_t cc[4] = {(uint32_t)t, (uint32_t)k, (uint32_t)ctr, (uint32_t)(ctr >> 32)};
                    Philox::gen(cc, (uint32_t)g.seed, (uint32_t)(g.seed >> 32));
                    ffbs::frame_draws(t, ffbs::uniform53(cc[0], cc[1]), xs, es, Af, nzA, sel + 4 * t);
                }
                __syncthreads();
                if (threadIdx.x < 32) ffbs::walk_decisions(threadIdx.x, F, sel, sts);
                __syncthreads();
                // phase C: record the drawn states of this CTA's frames and add spot
                // k back where it is on
                for (int f = c; f < F; f += G) {
                    if (threadIdx.x == 0) g.state[(size_t)k * F + f] = sts[f];
                    if (sts[f] != 0) continue;
                    double* cur = g.cur + (size_t)f * P;
                    for (int q0 = m0 + threadIdx.x; q0 < m1; q0 += kGibbsThreads * kBatch) {
                        int pp[kBatch];
                        double v[kBatch], cv[kBatch];
#pragma unroll
                        for (int b = 0; b < kBatch; ++b) {
                            const int q = q0 + b * kGibbsThreads;
                            pp[b] = q < m1 ? __ldg(g.midx + q) : -1;
                        }
#pragma unroll
                        for (int b = 0; b < kBatch; ++b) {
                            const int p = pp[b] < 0 ? 0 : pp[b];
                            v[b] = __ldg(vk + p);
                            cv[b] = cur[p];
                        }
#pragma unroll
                        for (int b = 0; b < kBatch; ++b)
                            if (pp[b] >= 0) cur[pp[b]] = cv[b] + v[b];
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
            double se = 0.0, unused = 0.0;
            for (int p = threadIdx.x; p < P; p += kGibbsThreads) {
                const double cv = cur[p];
                if (o) o[p] = ex ? cv - vx[p] : cv;
                const double e = dat[p] - cv;
                se += e * e;
            }
            if (g.out_err) {
                block_sum2(se, unused, red);
                if (threadIdx.x == 0) g.out_err[(size_t)d * F + f] = se;
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
    // forward values 24 B, emission terms 16 + 8 B, exponents 12 B, decision
    // table 4 B and drawn state 1 B per frame
    return ((size_t)F * 65 + 15) & ~(size_t)15;
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

int launch_gibbs(const GibbsParams* chains_dev, int nchains, int grid_per_chain, int F, void* stream) {
    const size_t smem = gibbs_smem_bytes(F);
    cudaError_t e = cudaFuncSetAttribute(gibbs_chain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    const GibbsParams* q = chains_dev;
    int n = nchains;
    void* args[] = {&q, &n};
    e = cudaLaunchCooperativeKernel((const void*)gibbs_chain_kernel, dim3(grid_per_chain * nchains), dim3(kGibbsThreads),
                                    args, smem, static_cast<cudaStream_t>(stream));
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

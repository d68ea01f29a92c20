// Host side of the 3B (Bayesian blinking and bleaching) entry points of
// librfba_srrf.so: the spot gradient and its optimiser, the Gibbs sampler, the
// free energy and the main-loop pass (RFBA Main/multispot5.cc,
// sampled_multispot.h), each staging its data on the context's device scratch
// and driving the kernels of threeb.cu and gibbs.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <set>
#include <string>
#include <vector>

#include "cg_only.h"
#include "context.h"

namespace rfba {

// ---- 3B spot gradient ------------------------------------------------------

static int threeb_validate(const rfba_3b_model* m, int S, int F, int P, int ptr_flags) {
    if (S < 1 || F < 1 || P < 1 || (long long)S * F >= (1LL << 31) || !(m->variance > 0) || m->z_factor == 0) {
        set_error("bad sizes or model (S, F, P >= 1, S*F < 2^31, variance > 0, z_factor != 0)");
        return RFBA_ERR_INVALID;
    }
    if (ptr_flags != RFBA_HOST_PTRS && ptr_flags != RFBA_DEVICE_PTRS) {
        set_error("ptr_flags must be RFBA_HOST_PTRS or RFBA_DEVICE_PTRS");
        return RFBA_ERR_INVALID;
    }
    for (int n = 0; n < 12; ++n) {
        const double v = n < 9 ? m->A[n] : m->pi[n - 9];
        if (!(v >= 0 && v <= 1)) {
            set_error("transition and initial probabilities must lie in [0, 1]");
            return RFBA_ERR_INVALID;
        }
    }
    return RFBA_OK;
}

struct ThreeBData {
    const double* bg = nullptr;
    const double* pix = nullptr;
    const int* pixels = nullptr;
    int S = 0, F = 0, P = 0;
};

// Scratch for one evaluation, and the data on the device (copied in once when
// the caller's pointers are host memory).
static int threeb_stage(rfba_ctx* ctx, const double* sample_bg, const double* pixel_intensities, const int* pixels,
                        int S, int F, int P, int ptr_flags, cudaStream_t st, ThreeBData* d) {
    int s;
    const size_t nbg = (size_t)S * F * P, npix = (size_t)F * P;
    if ((s = ctx->tb_val.ensure((size_t)P * 8, "3B spot table")) || (s = ctx->tb_der.ensure((size_t)P * 40, "3B spot table")) ||
        (s = ctx->tb_em.ensure((size_t)S * F * 80, "3B emissions")) || (s = ctx->tb_res.ensure((size_t)S * 48 + 48, "3B results")) ||
        (s = ctx->tb_par.ensure(17 * 8, "3B parameters")))
        return s;
    d->bg = sample_bg;
    d->pix = pixel_intensities;
    d->pixels = pixels;
    d->S = S;
    d->F = F;
    d->P = P;
    if (ptr_flags == RFBA_HOST_PTRS) {
        if ((s = ctx->tb_bg.ensure(nbg * 8, "3B samples")) || (s = ctx->tb_pix.ensure(npix * 8, "3B data")) ||
            (s = ctx->tb_pixels.ensure((size_t)P * 12, "3B mask")))
            return s;
        RFBA_CUDA(cudaMemcpyAsync(ctx->tb_bg.p, sample_bg, nbg * 8, cudaMemcpyHostToDevice, st), "samples copy");
        RFBA_CUDA(cudaMemcpyAsync(ctx->tb_pix.p, pixel_intensities, npix * 8, cudaMemcpyHostToDevice, st), "data copy");
        RFBA_CUDA(cudaMemcpyAsync(ctx->tb_pixels.p, pixels, (size_t)P * 12, cudaMemcpyHostToDevice, st), "mask copy");
        d->bg = static_cast<const double*>(ctx->tb_bg.p);
        d->pix = static_cast<const double*>(ctx->tb_pix.p);
        d->pixels = static_cast<const int*>(ctx->tb_pixels.p);
    }
    return RFBA_OK;
}

// One evaluation at `spot` (brightness and blur > 0) on staged data: the four
// kernels, the samples' results back, their mean plus the priors' derivatives.
static int threeb_eval(rfba_ctx* ctx, const rfba_3b_model* m, const ThreeBData& d, const double* spot, double* out,
                       double* log_prob, cudaStream_t st) {
    const int S = d.S, F = d.F, P = d.P;
    // parameters: spot, A (row-major), pi
    double par[17];
    for (int n = 0; n < 5; ++n) par[n] = spot[n];
    for (int n = 0; n < 9; ++n) par[5 + n] = m->A[n];
    for (int n = 0; n < 3; ++n) par[14 + n] = m->pi[n];
    RFBA_CUDA(cudaMemcpyAsync(ctx->tb_par.p, par, sizeof par, cudaMemcpyHostToDevice, st), "parameter upload");
    const unsigned int n_pix = (unsigned int)P;
    const double c0 = n_pix * ::log(2 * M_PI * m->variance) / 2;  // spot_with_background.hh:126-127
    const double* dpar = static_cast<const double*>(ctx->tb_par.p);
    int e = launch_threeb(d.bg, d.pix, d.pixels, S, F, P, dpar, m->z_factor, m->variance, c0, dpar + 5, dpar + 14,
                          static_cast<double*>(ctx->tb_val.p), static_cast<double*>(ctx->tb_der.p),
                          static_cast<double*>(ctx->tb_em.p), static_cast<double*>(ctx->tb_res.p), st);
    if (e) return cuda_fail((cudaError_t)e, "3B spot gradient launch");
    ctx->launches += 4;
    std::vector<double> res((size_t)S * 6);
    RFBA_CUDA(cudaMemcpyAsync(res.data(), ctx->tb_res.p, res.size() * 8, cudaMemcpyDeviceToHost, st), "result copy");
    RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    double sum[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < S; ++i)
        for (int n = 0; n < 5; ++n) sum[n] += res[(size_t)i * 6 + n];
    // storm.h:431-434: derivatives of the log-normal priors on brightness and blur
    auto dlln = [&](double x, double mu, double sg) { return -(1 + (std::log(x) - mu) / (sg * sg)) / x; };
    const double prior[5] = {dlln(spot[0], m->mu_brightness, m->sigma_brightness),
                             dlln(spot[1], m->mu_blur, m->sigma_blur), 0, 0, 0};
    for (int n = 0; n < 5; ++n) out[n] = -(sum[n] / (double)S + prior[n]);
    if (log_prob)
        for (int i = 0; i < S; ++i) log_prob[i] = res[(size_t)i * 6 + 5];
    return RFBA_OK;
}


// ---- 3B Gibbs sampler -------------------------------------------------------

// getBall (multispot5.cc:1259-1272): the integer offsets p, z outermost then y
// then x over [-r, r] with r = ceil(radius + 1), kept when |p|^2 (unsigned)
// <= radius^2 in float.
static std::vector<int> ball(float radius) {
    std::vector<int> pts;
    const int r = (int)std::ceil(radius + 1);
    for (int z = -r; z <= r; ++z)
        for (int y = -r; y <= r; ++y)
            for (int x = -r; x <= r; ++x) {
                const unsigned int m2 = (unsigned int)(x * x) + (unsigned int)(y * y) + (unsigned int)(z * z);
                if ((float)m2 <= radius * radius) {
                    pts.push_back(x);
                    pts.push_back(y);
                    pts.push_back(z);
                }
            }
    return pts;
}

// ir_rounded3D (multispot5.cc:989-995): round half away from zero.
static int round_away(double v) { return static_cast<int>(v > 0.0 ? v + 0.5 : v - 0.5); }

// Masks and pixel/spot validation shared by the Gibbs entry points. Masks are
// host copies (read back when the caller's pointers are device memory).
static int gibbs_masks(const int* moff, const int* midx, int K, int P, int ptr_flags, cudaStream_t st,
                       std::vector<int>* hoff, std::vector<int>* hidx) {
    hoff->assign((size_t)K + 1, 0);
    if (ptr_flags == RFBA_HOST_PTRS)
        std::memcpy(hoff->data(), moff, ((size_t)K + 1) * sizeof(int));
    else {
        RFBA_CUDA(cudaMemcpyAsync(hoff->data(), moff, ((size_t)K + 1) * sizeof(int), cudaMemcpyDeviceToHost, st),
                  "mask offsets read-back");
        RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    }
    if ((*hoff)[0] != 0) {
        set_error("mask_offsets[0] must be 0");
        return RFBA_ERR_INVALID;
    }
    for (int k = 0; k < K; ++k)
        if ((*hoff)[k + 1] < (*hoff)[k]) {
            set_error("mask_offsets must not decrease");
            return RFBA_ERR_INVALID;
        }
    const size_t nnz = (size_t)(*hoff)[K];
    hidx->assign(nnz, 0);
    if (nnz) {
        if (ptr_flags == RFBA_HOST_PTRS)
            std::memcpy(hidx->data(), midx, nnz * sizeof(int));
        else {
            RFBA_CUDA(cudaMemcpyAsync(hidx->data(), midx, nnz * sizeof(int), cudaMemcpyDeviceToHost, st),
                      "mask read-back");
            RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
        }
    }
    // every index inside [0, P), no pixel twice in one spot's mask (a spot's
    // pixels are updated in parallel)
    std::vector<int> seen((size_t)P, -1);
    for (int k = 0; k < K; ++k)
        for (int q = (*hoff)[k]; q < (*hoff)[k + 1]; ++q) {
            const int p = (*hidx)[q];
            if (p < 0 || p >= P) {
                set_error("mask pixel index outside [0, P)");
                return RFBA_ERR_INVALID;
            }
            if (seen[p] == k) {
                set_error("a pixel appears twice in one spot's mask");
                return RFBA_ERR_INVALID;
            }
            seen[p] = k;
        }
    return RFBA_OK;
}

struct GibbsCall {
    int K = 0, F = 0, P = 0;
    int sweeps = 1, n_draws = 1;
    unsigned long long seed = 0;
    int exclude = -1;
    const double* var_draw = nullptr;  // host, n_draws
    bool want_state = false, want_int = false, want_err = false, trace = false;
};

// Stage the data, compute the spot intensities, run one chain from all spots
// off. Outputs stay in the context's gb_* buffers; returns after the kernel
// has finished and its status has been read.
static int gibbs_run(rfba_ctx* ctx, const rfba_3b_model* m, const double* pix, const int* pixels,
                     const double* spots, const std::vector<int>& hoff, const std::vector<int>& hidx,
                     const GibbsCall& c, int ptr_flags, cudaStream_t st) {
    int s;
    const size_t K = (size_t)c.K, F = (size_t)c.F, P = (size_t)c.P, nnz = hidx.size();
    if ((s = ctx->gb_moff.ensure((K + 1) * 4, "3B mask offsets")) || (s = ctx->gb_midx.ensure(nnz * 4 + 4, "3B masks")) ||
        (s = ctx->gb_si.ensure(K * P * 8 + 8, "3B spot intensities")) ||
        (s = ctx->gb_state.ensure(K * F + 1, "3B spot states")) || (s = ctx->gb_cur.ensure(F * P * 8, "3B sample intensities")) ||
        (s = ctx->gb_em.ensure(F * 64, "3B emissions")) || (s = ctx->gb_bar.ensure(256, "3B barrier")))
        return s;
    const double* dpix = pix;
    const int* dpixels = pixels;
    const double* dspots = spots;
    if (ptr_flags == RFBA_HOST_PTRS) {
        if ((s = ctx->gb_pix.ensure(F * P * 8, "3B data")) || (s = ctx->gb_pixels.ensure(P * 12, "3B pixels")) ||
            (s = ctx->gb_spots.ensure(K * 40 + 8, "3B spots")))
            return s;
        RFBA_CUDA(cudaMemcpyAsync(ctx->gb_pix.p, pix, F * P * 8, cudaMemcpyHostToDevice, st), "data copy");
        RFBA_CUDA(cudaMemcpyAsync(ctx->gb_pixels.p, pixels, P * 12, cudaMemcpyHostToDevice, st), "pixels copy");
        if (K) RFBA_CUDA(cudaMemcpyAsync(ctx->gb_spots.p, spots, K * 40, cudaMemcpyHostToDevice, st), "spots copy");
        dpix = static_cast<const double*>(ctx->gb_pix.p);
        dpixels = static_cast<const int*>(ctx->gb_pixels.p);
        dspots = static_cast<const double*>(ctx->gb_spots.p);
    }
    RFBA_CUDA(cudaMemcpyAsync(ctx->gb_moff.p, hoff.data(), (K + 1) * 4, cudaMemcpyHostToDevice, st), "mask offsets copy");
    if (nnz) RFBA_CUDA(cudaMemcpyAsync(ctx->gb_midx.p, hidx.data(), nnz * 4, cudaMemcpyHostToDevice, st), "mask copy");
    if (K) {
        int e = launch_spot_intensity(dpixels, c.P, dspots, c.K, m->z_factor, static_cast<double*>(ctx->gb_si.p), st);
        if (e) return cuda_fail((cudaError_t)e, "3B spot intensity launch");
        ++ctx->launches;
    }
    // all spots off (state 2), no spot intensity in the current sample
    RFBA_CUDA(cudaMemsetAsync(ctx->gb_state.p, 2, K * F + 1, st), "state init");
    RFBA_CUDA(cudaMemsetAsync(ctx->gb_cur.p, 0, F * P * 8, st), "sample init");
    RFBA_CUDA(cudaMemsetAsync(ctx->gb_bar.p, 0, 256, st), "barrier init");
    RFBA_CUDA(cudaMemsetAsync(ctx->errw.p, 0, 8, st), "status clear");
    const size_t nd = (size_t)c.n_draws;
    if (c.var_draw) {
        if ((s = ctx->gb_var.ensure(nd * 8, "3B variance schedule"))) return s;
        RFBA_CUDA(cudaMemcpyAsync(ctx->gb_var.p, c.var_draw, nd * 8, cudaMemcpyHostToDevice, st), "schedule copy");
    }
    if (c.want_state && (s = ctx->gb_ostate.ensure(nd * K * F + 1, "3B drawn states"))) return s;
    if (c.want_int && (s = ctx->gb_oint.ensure(nd * F * P * 8, "3B drawn intensities"))) return s;
    if (c.want_err && (s = ctx->gb_oerr.ensure(nd * F * 8, "3B residual sums"))) return s;
    if (c.trace && ((s = ctx->gb_lp.ensure(K * F * 16 + 16, "3B trace")) || (s = ctx->gb_filt.ensure(K * F * 24 + 24, "3B trace"))))
        return s;
    GibbsParams g;
    std::memset(&g, 0, sizeof g);
    g.pix = dpix;
    g.si = static_cast<const double*>(ctx->gb_si.p);
    g.moff = static_cast<const int*>(ctx->gb_moff.p);
    g.midx = static_cast<const int*>(ctx->gb_midx.p);
    g.K = c.K;
    g.F = c.F;
    g.P = c.P;
    for (int n = 0; n < 9; ++n) g.A[n] = m->A[n];
    for (int n = 0; n < 3; ++n) g.pi[n] = m->pi[n];
    g.variance = m->variance;
    g.var_draw = c.var_draw ? static_cast<const double*>(ctx->gb_var.p) : nullptr;
    g.sweeps = c.sweeps;
    g.n_draws = c.n_draws;
    g.seed = c.seed;
    g.draw_base = 0;
    g.state = static_cast<unsigned char*>(ctx->gb_state.p);
    g.cur = static_cast<double*>(ctx->gb_cur.p);
    g.em = static_cast<double*>(ctx->gb_em.p);
    g.bar = static_cast<unsigned int*>(ctx->gb_bar.p);
    g.err = static_cast<unsigned long long*>(ctx->errw.p);
    g.out_state = c.want_state ? static_cast<unsigned char*>(ctx->gb_ostate.p) : nullptr;
    g.out_int = c.want_int ? static_cast<double*>(ctx->gb_oint.p) : nullptr;
    g.exclude_spot = c.exclude;
    g.out_err = c.want_err ? static_cast<double*>(ctx->gb_oerr.p) : nullptr;
    g.rec_lp = c.trace ? static_cast<double*>(ctx->gb_lp.p) : nullptr;
    g.rec_filt = c.trace ? static_cast<double*>(ctx->gb_filt.p) : nullptr;
    int maxb = 0;
    int e = gibbs_max_blocks(c.F, &maxb);
    if (e) return cuda_fail((cudaError_t)e, "3B Gibbs occupancy");
    if (maxb < 1) {
        set_error("3B Gibbs kernel does not fit on an SM");
        return RFBA_ERR_UNSUPPORTED;
    }
    const int grid = std::min(std::min(c.F, maxb), ctx->sm_count);
    e = launch_gibbs(g, grid, st);
    if (e) return cuda_fail((cudaError_t)e, "3B Gibbs launch");
    ++ctx->launches;
    unsigned long long w = 0;
    RFBA_CUDA(cudaMemcpyAsync(&w, ctx->errw.p, 8, cudaMemcpyDeviceToHost, st), "status read");
    RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    if (w) {
        RFBA_CUDA(cudaMemsetAsync(ctx->errw.p, 0, 8, st), "status clear");
        char buf[160];
        std::snprintf(buf, sizeof buf, "3B Gibbs sampler: a grid barrier gave up (spot %llu)", w & 0xffffffffffffull);
        set_error(buf);
        return RFBA_ERR_TIMEOUT;
    }
    return RFBA_OK;
}

static int gibbs_check(rfba_ctx* ctx, const rfba_3b_model* m, int K, int F, int P, int ptr_flags) {
    if (!ctx || !m) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    if (K < 0 || F < 1 || P < 1 || F > 2048 || (long long)F * P >= (1LL << 40) / 8) {
        set_error("bad sizes (K >= 0, 1 <= F <= 2048, P >= 1)");
        return RFBA_ERR_INVALID;
    }
    return threeb_validate(m, 1, F, P, ptr_flags);
}

static void copy_out(void* dst, const void* src, size_t n, int ptr_flags, cudaStream_t st, int* s) {
    if (*s || !dst || n == 0) return;
    const cudaError_t e = cudaMemcpyAsync(dst, src, n, ptr_flags == RFBA_HOST_PTRS ? cudaMemcpyDeviceToHost
                                                                                  : cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) *s = cuda_fail(e, "3B Gibbs output copy");
}

// variance_from_sample (multispot5.cc:321-328)
static double variance_from_sample(double sample, double samples, double base_sigma, double scale_pow) {
    const double scale = std::pow(1.25, sample * 1. / samples * scale_pow);
    const double sigma = base_sigma * scale;
    return sigma * sigma;
}

// log_log_normal (storm.h:417-420) with the reference's ln (forward_algorithm.h:34-40)
static double ref_ln(double x) { return x == 0 ? -1e100 : std::log(x); }
static double log_log_normal(double x, double mu, double sigma) {
    const double a = ref_ln(x) - mu;
    return -(a * a) / (2 * (sigma * sigma)) - ref_ln(x) - ref_ln(sigma * std::sqrt(2 * M_PI));
}

}  // namespace rfba

using namespace rfba;

extern "C" {

int rfba_3b_spot_masks(const int* pixels, int P, const double* spots, int K, int* mask_offsets, int* mask_pixels,
                       long long cap, long long* nnz) {
    if (!pixels || P < 1 || K < 0 || (K > 0 && !spots) || !mask_offsets || !nnz) {
        set_error("null argument or bad sizes");
        return RFBA_ERR_INVALID;
    }
    // pixels must be in the reference's Ref3D order (z, then y, then x)
    auto less = [&](int a, int b) {
        const int* p = pixels + 3 * a;
        const int* q = pixels + 3 * b;
        return p[2] < q[2] || (p[2] == q[2] && p[1] < q[1]) || (p[2] == q[2] && p[1] == q[1] && p[0] < q[0]);
    };
    for (int i = 1; i < P; ++i)
        if (!less(i - 1, i)) {
            set_error("pixels must be sorted by (z, y, x) without repeats");
            return RFBA_ERR_INVALID;
        }
    long long n = 0;
    mask_offsets[0] = 0;
    for (int k = 0; k < K; ++k) {
        const double* sp = spots + 5 * (size_t)k;
        const std::vector<int> b = ball((float)(sp[1] * 6 + 1));
        const int ox = round_away(sp[2]), oy = round_away(sp[3]), oz = round_away(sp[4]);
        for (size_t j = 0; j < b.size(); j += 3) {
            const int t[3] = {b[j] + ox, b[j + 1] + oy, b[j + 2] + oz};
            int lo = 0, hi = P;  // lower_bound
            while (lo < hi) {
                const int mid = (lo + hi) / 2;
                const int* q = pixels + 3 * mid;
                const bool lt = q[2] < t[2] || (q[2] == t[2] && q[1] < t[1]) || (q[2] == t[2] && q[1] == t[1] && q[0] < t[0]);
                if (lt)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            if (lo < P && pixels[3 * lo] == t[0] && pixels[3 * lo + 1] == t[1] && pixels[3 * lo + 2] == t[2]) {
                if (mask_pixels && n < cap) mask_pixels[n] = lo;
                ++n;
            }
        }
        if (n > INT32_MAX) {
            set_error("masks too large");
            return RFBA_ERR_INVALID;
        }
        mask_offsets[k + 1] = (int)n;
    }
    *nnz = n;
    return RFBA_OK;
}

int rfba_3b_gibbs_sample(rfba_ctx* ctx, const rfba_3b_model* m, const double* pixel_intensities, const int* pixels,
                         const double* spots, const int* mask_offsets, const int* mask_pixels, int K, int F, int P,
                         int sweeps, int n_draws, unsigned long long seed, int exclude_spot, uint8_t* states,
                         double* sample_intensities, int ptr_flags, void* stream) {
    int s;
    if ((s = gibbs_check(ctx, m, K, F, P, ptr_flags))) return s;
    if (!pixel_intensities || !pixels || (K > 0 && (!spots || !mask_pixels)) || !mask_offsets || sweeps < 1 ||
        n_draws < 1 || exclude_spot >= K || exclude_spot < -1) {
        set_error("null argument, or sweeps / n_draws < 1, or exclude_spot outside [-1, K)");
        return RFBA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if ((s = order_streams(ctx, st))) return s;
    std::vector<int> hoff, hidx;
    if ((s = gibbs_masks(mask_offsets, mask_pixels, K, P, ptr_flags, st, &hoff, &hidx))) return s;
    GibbsCall c;
    c.K = K;
    c.F = F;
    c.P = P;
    c.sweeps = sweeps;
    c.n_draws = n_draws;
    c.seed = seed;
    c.exclude = exclude_spot;
    c.want_state = states != nullptr;
    c.want_int = sample_intensities != nullptr;
    if ((s = gibbs_run(ctx, m, pixel_intensities, pixels, spots, hoff, hidx, c, ptr_flags, st))) return s;
    copy_out(states, ctx->gb_ostate.p, (size_t)n_draws * K * F, ptr_flags, st, &s);
    copy_out(sample_intensities, ctx->gb_oint.p, (size_t)n_draws * F * P * 8, ptr_flags, st, &s);
    if (s) return s;
    RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    return RFBA_OK;
}

// Seed of spot `s`'s draws in pass `pass` of rfba_3b_optimise_pass: SplitMix64
// (Steele, Lea, Flood, OOPSLA 2014) of the caller's seed mixed with both.
static unsigned long long pass_seed(unsigned long long seed, int pass, int s) {
    unsigned long long z = seed ^ ((unsigned long long)(unsigned)pass << 32) ^ (unsigned long long)(unsigned)s;
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

unsigned long long rfba_3b_pass_seed(unsigned long long seed, int pass, int s) { return pass_seed(seed, pass, s); }

// One pass of FitSpots::optimize_each_spot_in_turn_for_several_passes
// (multispot5.cc:1511-1690).
int rfba_3b_optimise_pass(rfba_ctx* ctx, const rfba_3b_model* m, const double* pixel_intensities, const int* pixels,
                          int F, int P, double* spots, int* nspots, int pass, int main_samples, int sweeps,
                          int cg_max_iterations, const double limit[5], double position_extra_radius,
                          unsigned long long seed, int* evaluations) {
    int s;
    if (!nspots || !spots || !limit || !pixel_intensities || !pixels) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    int K = *nspots;
    if ((s = gibbs_check(ctx, m, K, F, P, RFBA_HOST_PTRS))) return s;
    if (main_samples < 1 || sweeps < 1 || cg_max_iterations < 0) {
        set_error("main_samples and sweeps must be >= 1, cg_max_iterations >= 0");
        return RFBA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    if ((s = order_streams(ctx, st))) return s;
    // masks of every spot (multispot5.cc:1518-1521)
    std::vector<int> off((size_t)K + 1);
    long long nnz = 0;
    if ((s = rfba_3b_spot_masks(pixels, P, spots, K, off.data(), nullptr, 0, &nnz))) return s;
    std::vector<int> idx((size_t)nnz);
    if ((s = rfba_3b_spot_masks(pixels, P, spots, K, off.data(), idx.data(), nnz, &nnz))) return s;
    std::vector<std::vector<int> > masks((size_t)K);
    for (int k = 0; k < K; ++k) masks[k].assign(idx.begin() + off[k], idx.begin() + off[k + 1]);
    // allowed area: the pixels dilated by getBall(extra_radius) (multispot5.cc:1280-1290)
    std::set<long long> allowed;
    auto key = [](int x, int y, int z) {
        return ((long long)(x + (1 << 20)) << 42) | ((long long)(y + (1 << 20)) << 21) | (long long)(z + (1 << 20));
    };
    const bool use_prior = position_extra_radius >= 0;
    if (use_prior) {
        const std::vector<int> b = ball((float)position_extra_radius);
        for (int p = 0; p < P; ++p)
            for (size_t j = 0; j < b.size(); j += 3)
                allowed.insert(key(pixels[3 * p] + b[j], pixels[3 * p + 1] + b[j + 1], pixels[3 * p + 2] + b[j + 2]));
    }
    // the sweep order (multispot5.cc:1541-1560): by x or y position, ascending
    // or descending; the reference's third branch repeats `% 4 == 1` and is never
    // taken, so passes 2 and 3 both sort by descending y
    std::vector<int> order((size_t)K);
    for (int k = 0; k < K; ++k) order[k] = k;
    std::vector<std::array<double, 5> > sp((size_t)K);
    for (int k = 0; k < K; ++k)
        for (int n = 0; n < 5; ++n) sp[k][n] = spots[5 * k + n];
    const int mode = pass % 4 == 0 ? 0 : pass % 4 == 1 ? 1 : 2;
    const int first = mode == 2 ? 3 : 2, second = first == 2 ? 3 : 2;
    std::sort(order.begin(), order.end(), [&](int a, int b) {
        const double fa = sp[a][first], fb = sp[b][first];
        const bool desc = mode != 0;
        if (desc ? fa > fb : fa < fb) return true;
        if (fa == fb) return desc ? sp[a][second] > sp[b][second] : sp[a][second] < sp[b][second];
        return false;
    });
    {
        std::vector<std::array<double, 5> > t((size_t)K);
        for (int k = 0; k < K; ++k) t[k] = sp[order[k]];
        sp.swap(t);
        // masks stay where they were: the reference swaps tmp_spot_pixels[i]
        // with spot_pixels[i], not spot_pixels[index[i]] (multispot5.cc:1570), so
        // a spot's mask is the one at its new position until it is optimised
    }
    // data on the device once
    const size_t FP = (size_t)F * P;
    if ((s = ctx->gb_pix.ensure(FP * 8, "3B data")) || (s = ctx->gb_pixels.ensure((size_t)P * 12, "3B pixels")) ||
        (s = ctx->gb_spots.ensure((size_t)K * 40 + 8, "3B spots")))
        return s;
    RFBA_CUDA(cudaMemcpyAsync(ctx->gb_pix.p, pixel_intensities, FP * 8, cudaMemcpyHostToDevice, st), "data copy");
    RFBA_CUDA(cudaMemcpyAsync(ctx->gb_pixels.p, pixels, (size_t)P * 12, cudaMemcpyHostToDevice, st), "pixels copy");
    int evals = 0;
    for (int k = 0; k < K; ++k) {
        // a fresh sampler for this spot: main_samples draws, the spot taken off
        // them (multispot5.cc:1591-1608)
        std::vector<int> hoff((size_t)K + 1, 0), hidx;
        for (int j = 0; j < K; ++j) {
            hidx.insert(hidx.end(), masks[j].begin(), masks[j].end());
            hoff[j + 1] = (int)hidx.size();
        }
        std::vector<double> flat((size_t)K * 5);
        for (int j = 0; j < K; ++j)
            for (int n = 0; n < 5; ++n) flat[5 * j + n] = sp[j][n];
        RFBA_CUDA(cudaMemcpyAsync(ctx->gb_spots.p, flat.data(), flat.size() * 8, cudaMemcpyHostToDevice, st),
                  "spots copy");
        GibbsCall c;
        c.K = K;
        c.F = F;
        c.P = P;
        c.sweeps = sweeps;
        c.n_draws = main_samples;
        c.seed = pass_seed(seed, pass, k);
        c.exclude = k;
        c.want_int = true;
        if ((s = gibbs_run(ctx, m, static_cast<const double*>(ctx->gb_pix.p), static_cast<const int*>(ctx->gb_pixels.p),
                           static_cast<const double*>(ctx->gb_spots.p), hoff, hidx, c, RFBA_DEVICE_PTRS, st)))
            return s;
        // optimise the spot on those samples (multispot5.cc:1611-1636)
        ThreeBData d;
        if ((s = threeb_stage(ctx, static_cast<const double*>(ctx->gb_oint.p), static_cast<const double*>(ctx->gb_pix.p),
                              static_cast<const int*>(ctx->gb_pixels.p), main_samples, F, P, RFBA_DEVICE_PTRS, st, &d)))
            return s;
        auto grad = [&](const double* x, double* g) -> int {
            if (x[0] <= 0 || x[1] <= 0) {
                for (int n = 0; n < 5; ++n) g[n] = std::numeric_limits<double>::quiet_NaN();
                return RFBA_OK;
            }
            return threeb_eval(ctx, m, d, x, g, nullptr, st);
        };
        CgOnly5 cg;
        if ((s = cg.start(sp[k].data(), limit, grad))) return s;
        cg.max_iterations = cg_max_iterations;
        if ((s = cg.run(grad))) return s;
        evals += cg.evaluations;
        for (int n = 0; n < 5; ++n) sp[k][n] = cg.x[n];
        // new mask; eject the spot if it has no pixels or left the allowed area
        // (multispot5.cc:1651-1674)
        int o2[2];
        long long n2 = 0;
        if ((s = rfba_3b_spot_masks(pixels, P, sp[k].data(), 1, o2, nullptr, 0, &n2))) return s;
        masks[k].assign((size_t)n2, 0);
        if (n2 && (s = rfba_3b_spot_masks(pixels, P, sp[k].data(), 1, o2, masks[k].data(), n2, &n2))) return s;
        const bool zero_prior =
            use_prior && !allowed.count(key(round_away(sp[k][2]), round_away(sp[k][3]), round_away(sp[k][4])));
        if (masks[k].empty() || zero_prior) {
            sp.erase(sp.begin() + k);
            masks.erase(masks.begin() + k);
            --K;
            --k;
        }
    }
    for (int k = 0; k < K; ++k)
        for (int n = 0; n < 5; ++n) spots[5 * k + n] = sp[k][n];
    *nspots = K;
    if (evaluations) *evaluations = evals;
    return RFBA_OK;
}

int rfba_3b_gibbs_trace(rfba_ctx* ctx, const rfba_3b_model* m, const double* pixel_intensities, const int* pixels,
                        const double* spots, const int* mask_offsets, const int* mask_pixels, int K, int F, int P,
                        unsigned long long seed, uint8_t* states, double* log_prob, double* filtered, int ptr_flags,
                        void* stream) {
    int s;
    if ((s = gibbs_check(ctx, m, K, F, P, ptr_flags))) return s;
    if (!pixel_intensities || !pixels || (K > 0 && (!spots || !mask_pixels)) || !mask_offsets) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if ((s = order_streams(ctx, st))) return s;
    std::vector<int> hoff, hidx;
    if ((s = gibbs_masks(mask_offsets, mask_pixels, K, P, ptr_flags, st, &hoff, &hidx))) return s;
    GibbsCall c;
    c.K = K;
    c.F = F;
    c.P = P;
    c.seed = seed;
    c.want_state = true;
    c.trace = true;
    if ((s = gibbs_run(ctx, m, pixel_intensities, pixels, spots, hoff, hidx, c, ptr_flags, st))) return s;
    copy_out(states, ctx->gb_ostate.p, (size_t)K * F, ptr_flags, st, &s);
    copy_out(log_prob, ctx->gb_lp.p, (size_t)K * F * 16, ptr_flags, st, &s);
    copy_out(filtered, ctx->gb_filt.p, (size_t)K * F * 24, ptr_flags, st, &s);
    if (s) return s;
    RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    return RFBA_OK;
}

int rfba_3b_free_energy(rfba_ctx* ctx, const rfba_3b_model* m, const double* pixel_intensities, const int* pixels,
                        const double* spots, const int* mask_offsets, const int* mask_pixels, int K, int F, int P,
                        int samples, int sweeps, unsigned long long seed, double* value, double* residuals,
                        int ptr_flags, void* stream) {
    int s;
    if ((s = gibbs_check(ctx, m, K, F, P, ptr_flags))) return s;
    if (!pixel_intensities || !pixels || (K > 0 && (!spots || !mask_pixels)) || !mask_offsets || !value ||
        samples < 1 || sweeps < 1) {
        set_error("null argument, or samples / sweeps < 1");
        return RFBA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if ((s = order_streams(ctx, st))) return s;
    std::vector<int> hoff, hidx;
    if ((s = gibbs_masks(mask_offsets, mask_pixels, K, P, ptr_flags, st, &hoff, &hidx))) return s;
    // the spots on the host, for the priors
    std::vector<double> hsp((size_t)K * 5);
    if (K) {
        if (ptr_flags == RFBA_HOST_PTRS)
            std::memcpy(hsp.data(), spots, hsp.size() * 8);
        else {
            RFBA_CUDA(cudaMemcpyAsync(hsp.data(), spots, hsp.size() * 8, cudaMemcpyDeviceToHost, st), "spots read-back");
            RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
        }
    }
    // NegativeFreeEnergy::compute_with_mask (multispot5.cc:335-405): slow-growth
    // thermodynamic integration over `samples` draws, draw i taken at the
    // variance of step i - 1 and differentiated by a five-point stencil
    const double base_sigma = std::sqrt(m->variance);
    const double scale_pow = 100.0;
    std::vector<double> var2((size_t)samples);
    for (int i = 0; i < samples; ++i) var2[i] = variance_from_sample(i - 1, samples, base_sigma, scale_pow);
    GibbsCall c;
    c.K = K;
    c.F = F;
    c.P = P;
    c.sweeps = sweeps;
    c.n_draws = samples;
    c.seed = seed;
    c.var_draw = var2.data();
    c.want_err = true;
    if ((s = gibbs_run(ctx, m, pixel_intensities, pixels, spots, hoff, hidx, c, ptr_flags, st))) return s;
    std::vector<double> err((size_t)samples * F);
    RFBA_CUDA(cudaMemcpyAsync(err.data(), ctx->gb_oerr.p, err.size() * 8, cudaMemcpyDeviceToHost, st),
              "residual read-back");
    RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    const unsigned int npixels = (unsigned int)P, nframes = (unsigned int)F;
    double sum = 0;
    for (int sample = 0; sample < samples; sample++) {
        const double var1 = variance_from_sample(sample - 2, samples, base_sigma, scale_pow);
        const double var2s = variance_from_sample(sample - 1, samples, base_sigma, scale_pow);
        const double var3 = variance_from_sample(sample + 1, samples, base_sigma, scale_pow);
        const double var4 = variance_from_sample(sample + 2, samples, base_sigma, scale_pow);
        double err_sum = 0;
        for (int f = 0; f < F; ++f) err_sum -= err[(size_t)sample * F + f];
        if (residuals) residuals[sample] = -err_sum;
        const double e1 = err_sum / (2 * var1) - npixels * nframes * ::log(2 * M_PI * var1) / 2;
        const double e2 = err_sum / (2 * var2s) - npixels * nframes * ::log(2 * M_PI * var2s) / 2;
        const double e3 = err_sum / (2 * var3) - npixels * nframes * ::log(2 * M_PI * var3) / 2;
        const double e4 = err_sum / (2 * var4) - npixels * nframes * ::log(2 * M_PI * var4) / 2;
        sum += (-e1 + 8 * e2 - 8 * e3 + e4) / 12;
    }
    const double log_final =
        (::log(variance_from_sample(samples, samples, base_sigma, scale_pow) * 2 * M_PI) / 2) * npixels * nframes;
    double priors = 0;
    for (int i = 0; i < K; i++) {
        priors += log_log_normal(hsp[i * 5 + 0], m->mu_brightness, m->sigma_brightness);
        priors += log_log_normal(hsp[i * 5 + 1], m->mu_blur, m->sigma_blur);
    }
    *value = -(sum + priors - log_final);
    return RFBA_OK;
}


// SpotNegProbabilityDiffWithSampledBackground::operator() (multispot5.cc:616-664)
int rfba_3b_spot_gradient(rfba_ctx* ctx, const rfba_3b_model* m, const double* sample_bg,
                          const double* pixel_intensities, const int* pixels, int S, int F, int P, const double spot[5],
                          double out[5], double* log_prob, int ptr_flags, void* stream) {
    if (!ctx || !m || !sample_bg || !pixel_intensities || !pixels || !spot || !out) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    int s;
    if ((s = threeb_validate(m, S, F, P, ptr_flags))) return s;
    if (spot[0] <= 0 || spot[1] <= 0) {  // multispot5.cc:618-619
        for (int n = 0; n < 5; ++n) out[n] = std::numeric_limits<double>::quiet_NaN();
        return RFBA_OK;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if ((s = order_streams(ctx, st))) return s;
    ThreeBData d;
    if ((s = threeb_stage(ctx, sample_bg, pixel_intensities, pixels, S, F, P, ptr_flags, st, &d))) return s;
    return threeb_eval(ctx, m, d, spot, out, log_prob, st);
}

// The spot optimisation of multispot5.cc:1614-1636: ConjugateGradientOnly<5>
// (conjugate_gradient_only.h) from `spot` with motion limits `limit`, its
// gradient the spot-gradient evaluation above on data staged once.
int rfba_3b_optimise_spot(rfba_ctx* ctx, const rfba_3b_model* m, const double* sample_bg,
                          const double* pixel_intensities, const int* pixels, int S, int F, int P, const double spot[5],
                          const double limit[5], int max_iterations, double spot_out[5], int* iterations,
                          int* evaluations, int ptr_flags, void* stream) {
    if (!ctx || !m || !sample_bg || !pixel_intensities || !pixels || !spot || !limit || !spot_out) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    int s;
    if ((s = threeb_validate(m, S, F, P, ptr_flags))) return s;
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if ((s = order_streams(ctx, st))) return s;
    ThreeBData d;
    if ((s = threeb_stage(ctx, sample_bg, pixel_intensities, pixels, S, F, P, ptr_flags, st, &d))) return s;
    auto grad = [&](const double* x, double* g) -> int {
        if (x[0] <= 0 || x[1] <= 0) {  // multispot5.cc:618-619
            for (int n = 0; n < 5; ++n) g[n] = std::numeric_limits<double>::quiet_NaN();
            return RFBA_OK;
        }
        return threeb_eval(ctx, m, d, x, g, nullptr, st);
    };
    CgOnly5 cg;
    if ((s = cg.start(spot, limit, grad))) return s;
    cg.max_iterations = max_iterations;
    if ((s = cg.run(grad))) return s;
    for (int n = 0; n < 5; ++n) spot_out[n] = cg.x[n];
    if (iterations) *iterations = cg.iterations;
    if (evaluations) *evaluations = cg.evaluations;
    return RFBA_OK;
}

// The same optimiser on the host with a caller-supplied gradient (no device
// work).
int rfba_cg_only_run(const double start[5], const double limit[5], int max_iterations, rfba_grad5_fn grad,
                     void* user, double x_out[5], int* iterations, int* evaluations) {
    if (!start || !limit || !grad || !x_out) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    auto g = [&](const double* x, double* out) -> int { return grad(x, out, user); };
    CgOnly5 cg;
    int s;
    if ((s = cg.start(start, limit, g))) return s;
    cg.max_iterations = max_iterations;
    if ((s = cg.run(g))) return s;
    for (int n = 0; n < 5; ++n) x_out[n] = cg.x[n];
    if (iterations) *iterations = cg.iterations;
    if (evaluations) *evaluations = cg.evaluations;
    return RFBA_OK;
}

}  // extern "C"

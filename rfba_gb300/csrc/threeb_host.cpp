// Host side of the 3B (Bayesian blinking and bleaching) entry points of
// librfba_srrf.so: the spot gradient and its optimiser, the Gibbs sampler, the
// free energy and the main-loop pass (RFBA Main/multispot5.cc,
// sampled_multispot.h), each staging its data on the context's device scratch
// and driving the kernels of threeb.cu and gibbs.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
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
    const float2* dfd = nullptr;  // the residuals as double-floats, for gradient-only evaluations
    int S = 0, F = 0, P = 0;
};

// Scratch for one evaluation, and the data on the device (copied in once when
// the caller's pointers are host memory). residual_df: also stage the
// residuals as double-floats for an optimiser's gradient-only evaluations.
static int threeb_stage(rfba_ctx* ctx, const double* sample_bg, const double* pixel_intensities, const int* pixels,
                        int S, int F, int P, int ptr_flags, cudaStream_t st, ThreeBData* d, bool residual_df = false) {
    int s;
    const size_t nbg = (size_t)S * F * P, npix = (size_t)F * P;
    if ((s = ctx->tb_val.ensure((size_t)P * 8, "3B spot table")) || (s = ctx->tb_der.ensure((size_t)P * 40, "3B spot table")) ||
        (s = ctx->tb_em.ensure((size_t)S * F * 80, "3B emissions")) || (s = ctx->tb_res.ensure((size_t)S * 48 + 48 + (size_t)(P / 256 + 1) * 48, "3B results")) ||
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
    if (residual_df) {
        if ((s = ctx->tb_dfd.ensure(nbg * 8, "3B residuals")) || (s = ctx->tb_vdf.ensure((size_t)P * 48 + (((size_t)P + 15) & ~(size_t)15) + (size_t)P * 4 + 16,
                                   "3B spot table")))
            return s;
        const int e = launch_threeb_residual(d->bg, d->pix, S, F, P, static_cast<float2*>(ctx->tb_dfd.p), st);
        if (e) return cuda_fail((cudaError_t)e, "3B residual launch");
        ++ctx->launches;
        d->dfd = static_cast<const float2*>(ctx->tb_dfd.p);
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
                          static_cast<double*>(ctx->tb_em.p), static_cast<double*>(ctx->tb_res.p),
                          log_prob ? nullptr : d.dfd, static_cast<float2*>(ctx->tb_vdf.p), st);
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

// Stage one chain in scratch set `set` (the data, the spot intensities, all
// spots off) and fill its kernel parameters; nothing is launched.
static int gibbs_prepare(rfba_ctx* ctx, const rfba_3b_model* m, const double* pix, const int* pixels,
                         const double* spots, const std::vector<int>& hoff, const std::vector<int>& hidx,
                         const GibbsCall& c, int ptr_flags, cudaStream_t st, int set, GibbsParams* gp) {
    int s;
    GibbsScratch& gs = ctx->gb[set];
    const size_t K = (size_t)c.K, F = (size_t)c.F, P = (size_t)c.P, nnz = hidx.size();
    if ((s = gs.moff.ensure((K + 1) * 4, "3B mask offsets")) || (s = gs.midx.ensure(nnz * 4 + 4, "3B masks")) ||
        (s = gs.si.ensure(K * P * 8 + 8, "3B spot intensities")) ||
        (s = gs.state.ensure(K * F + 1, "3B spot states")) || (s = gs.cur.ensure(F * P * 8, "3B sample intensities")) ||
        (s = gs.em.ensure(F * 64, "3B emissions")) || (s = gs.bar.ensure(256, "3B barrier")))
        return s;
    const double* dpix = pix;
    const int* dpixels = pixels;
    const double* dspots = spots;
    if (ptr_flags == RFBA_HOST_PTRS) {
        if ((s = ctx->gb_pix.ensure(F * P * 8, "3B data")) || (s = ctx->gb_pixels.ensure(P * 12, "3B pixels")) ||
            (s = gs.spots.ensure(K * 40 + 8, "3B spots")))
            return s;
        RFBA_CUDA(cudaMemcpyAsync(ctx->gb_pix.p, pix, F * P * 8, cudaMemcpyHostToDevice, st), "data copy");
        RFBA_CUDA(cudaMemcpyAsync(ctx->gb_pixels.p, pixels, P * 12, cudaMemcpyHostToDevice, st), "pixels copy");
        if (K) RFBA_CUDA(cudaMemcpyAsync(gs.spots.p, spots, K * 40, cudaMemcpyHostToDevice, st), "spots copy");
        dpix = static_cast<const double*>(ctx->gb_pix.p);
        dpixels = static_cast<const int*>(ctx->gb_pixels.p);
        dspots = static_cast<const double*>(gs.spots.p);
    }
    RFBA_CUDA(cudaMemcpyAsync(gs.moff.p, hoff.data(), (K + 1) * 4, cudaMemcpyHostToDevice, st), "mask offsets copy");
    if (nnz) RFBA_CUDA(cudaMemcpyAsync(gs.midx.p, hidx.data(), nnz * 4, cudaMemcpyHostToDevice, st), "mask copy");
    if (K) {
        int e = launch_spot_intensity(dpixels, c.P, dspots, c.K, m->z_factor, static_cast<double*>(gs.si.p), st);
        if (e) return cuda_fail((cudaError_t)e, "3B spot intensity launch");
        ++ctx->launches;
    }
    // all spots off (state 2), no spot intensity in the current sample
    RFBA_CUDA(cudaMemsetAsync(gs.state.p, 2, K * F + 1, st), "state init");
    RFBA_CUDA(cudaMemsetAsync(gs.cur.p, 0, F * P * 8, st), "sample init");
    RFBA_CUDA(cudaMemsetAsync(gs.bar.p, 0, 256, st), "barrier init");
    RFBA_CUDA(cudaMemsetAsync(ctx->errw.p, 0, 8, st), "status clear");
    const size_t nd = (size_t)c.n_draws;
    if (c.var_draw) {
        if ((s = gs.var.ensure(nd * 8, "3B variance schedule"))) return s;
        RFBA_CUDA(cudaMemcpyAsync(gs.var.p, c.var_draw, nd * 8, cudaMemcpyHostToDevice, st), "schedule copy");
    }
    if (c.want_state && (s = gs.ostate.ensure(nd * K * F + 1, "3B drawn states"))) return s;
    if (c.want_int && (s = gs.oint.ensure(nd * F * P * 8, "3B drawn intensities"))) return s;
    if (c.want_err && (s = gs.oerr.ensure(nd * F * 8, "3B residual sums"))) return s;
    if (c.trace && ((s = gs.lp.ensure(K * F * 16 + 16, "3B trace")) || (s = gs.filt.ensure(K * F * 24 + 24, "3B trace"))))
        return s;
    GibbsParams& g = *gp;
    std::memset(&g, 0, sizeof g);
    g.pix = dpix;
    g.si = static_cast<const double*>(gs.si.p);
    g.moff = static_cast<const int*>(gs.moff.p);
    g.midx = static_cast<const int*>(gs.midx.p);
    g.K = c.K;
    g.F = c.F;
    g.P = c.P;
    for (int n = 0; n < 9; ++n) g.A[n] = m->A[n];
    for (int n = 0; n < 3; ++n) g.pi[n] = m->pi[n];
    g.variance = m->variance;
    g.var_draw = c.var_draw ? static_cast<const double*>(gs.var.p) : nullptr;
    g.sweeps = c.sweeps;
    g.n_draws = c.n_draws;
    g.seed = c.seed;
    g.draw_base = 0;
    g.state = static_cast<unsigned char*>(gs.state.p);
    g.cur = static_cast<double*>(gs.cur.p);
    g.em = static_cast<double*>(gs.em.p);
    g.bar = static_cast<unsigned int*>(gs.bar.p);
    g.err = static_cast<unsigned long long*>(ctx->errw.p);
    g.out_state = c.want_state ? static_cast<unsigned char*>(gs.ostate.p) : nullptr;
    g.out_int = c.want_int ? static_cast<double*>(gs.oint.p) : nullptr;
    g.exclude_spot = c.exclude;
    g.out_err = c.want_err ? static_cast<double*>(gs.oerr.p) : nullptr;
    g.rec_lp = c.trace ? static_cast<double*>(gs.lp.p) : nullptr;
    g.rec_filt = c.trace ? static_cast<double*>(gs.filt.p) : nullptr;
    return RFBA_OK;
}

// Launch nchains prepared chains side by side in one cooperative kernel, wait
// for it and read its status.
static int gibbs_launch(rfba_ctx* ctx, const GibbsParams* g, int nchains, int F, cudaStream_t st) {
    int s;
    if ((s = ctx->gb_par.ensure(sizeof(GibbsParams) * (size_t)nchains, "3B Gibbs parameters"))) return s;
    RFBA_CUDA(cudaMemcpyAsync(ctx->gb_par.p, g, sizeof(GibbsParams) * (size_t)nchains, cudaMemcpyHostToDevice, st),
              "parameter copy");
    int maxb = 0;
    int e = gibbs_max_blocks(F, &maxb);
    if (e) return cuda_fail((cudaError_t)e, "3B Gibbs occupancy");
    const int grid = std::min(std::min(F, maxb / nchains), ctx->sm_count);
    if (grid < 1) {
        set_error("3B Gibbs kernel does not fit on the GPU");
        return RFBA_ERR_UNSUPPORTED;
    }
    e = launch_gibbs(static_cast<const GibbsParams*>(ctx->gb_par.p), nchains, grid, F, st);
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

// One chain from all spots off in scratch set 0; the outputs stay there.
static int gibbs_run(rfba_ctx* ctx, const rfba_3b_model* m, const double* pix, const int* pixels,
                     const double* spots, const std::vector<int>& hoff, const std::vector<int>& hidx,
                     const GibbsCall& c, int ptr_flags, cudaStream_t st) {
    GibbsParams g;
    int s;
    if ((s = gibbs_prepare(ctx, m, pix, pixels, spots, hoff, hidx, c, ptr_flags, st, 0, &g))) return s;
    return gibbs_launch(ctx, &g, 1, c.F, st);
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

// ---- 3B main loop: passes, sampled-background Hessian, model modification ---

// SplitMix64 (Steele, Lea, Flood, OOPSLA 2014) of a seed mixed with two
// integers: the seeds of the sub-steps of a pass, a modification and a fit.
static unsigned long long mix_seed(unsigned long long seed, long long a, long long b) {
    unsigned long long z = seed ^ ((unsigned long long)a << 32) ^ (unsigned long long)(unsigned)b;
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Seed of spot `s`'s draws in pass `pass` of rfba_3b_optimise_pass.
static unsigned long long pass_seed(unsigned long long seed, int pass, int s) {
    return mix_seed(seed, (unsigned)pass, s);
}

// Uniform doubles in [0, 1) from a SplitMix64 stream: the host's random
// choices of a model modification (the reference's rng()).
struct HostUniform {
    unsigned long long state;
    double next() {
        unsigned long long z = (state += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    }
};

typedef std::array<double, 5> Spot;

// The allowed area of the position prior: the pixels dilated by
// getBall(extra_radius) (dilate_mask, multispot5.cc:1280-1290); off when the
// radius is negative.
struct AllowedArea {
    bool use = false;
    std::set<long long> cells;
    static long long key(int x, int y, int z) {
        return ((long long)(x + (1 << 20)) << 42) | ((long long)(y + (1 << 20)) << 21) | (long long)(z + (1 << 20));
    }
    void build(const int* pixels, int P, double radius) {
        use = radius >= 0;
        cells.clear();
        if (!use) return;
        const std::vector<int> b = ball((float)radius);
        for (int p = 0; p < P; ++p)
            for (size_t j = 0; j < b.size(); j += 3)
                cells.insert(key(pixels[3 * p] + b[j], pixels[3 * p + 1] + b[j + 1], pixels[3 * p + 2] + b[j + 2]));
    }
    // is_zero_prior at the spot's rounded position (ir_rounded3D, multispot5.cc:989-995)
    bool outside(const Spot& s) const {
        return use && !cells.count(key(round_away(s[2]), round_away(s[3]), round_away(s[4])));
    }
};

// get_spot_pixels for one spot (host).
static int spot_mask(const int* pixels, int P, const Spot& s, std::vector<int>* out) {
    int off[2];
    long long n = 0;
    int e;
    if ((e = rfba_3b_spot_masks(pixels, P, s.data(), 1, off, nullptr, 0, &n))) return e;
    out->assign((size_t)n, 0);
    if (n && (e = rfba_3b_spot_masks(pixels, P, s.data(), 1, off, out->data(), n, &n))) return e;
    return RFBA_OK;
}

static void flatten_masks(const std::vector<std::vector<int> >& masks, size_t count, std::vector<int>* off,
                          std::vector<int>* idx) {
    off->assign(count + 1, 0);
    idx->clear();
    for (size_t k = 0; k < count; ++k) {
        idx->insert(idx->end(), masks[k].begin(), masks[k].end());
        (*off)[k + 1] = (int)idx->size();
    }
}

// ln(2^-60): a spot's support is the pixels where its Gaussian factor is at
// least 2^-60 (threeb.cu's double-float gradient uses the same cut).
static constexpr double kSupportS = -41.58883083359672;

// The unmasked sampler's masks (GibbsSampler sums over every pixel): each
// spot's support in pixel order. The terms left out change a frame's on - off
// log probability, the only part of it the filter uses, by less than 2^-60 of
// the terms kept, far under the rounding of the all-pixel sums.
static void support_masks(const int* pixels, int P, const std::vector<Spot>& sp, double zf, std::vector<int>* off,
                          std::vector<int>* idx) {
    off->assign(sp.size() + 1, 0);
    idx->clear();
    for (size_t k = 0; k < sp.size(); ++k) {
        const Spot& s = sp[k];
        for (int q = 0; q < P; ++q) {
            const double d0 = pixels[3 * q] - s[2], d1 = pixels[3 * q + 1] - s[3], d2 = (pixels[3 * q + 2] - s[4]) / zf;
            const double e = -(d0 * d0 + d1 * d1 + d2 * d2) / (2 * s[1] * s[1]);
            if (e >= kSupportS) idx->push_back(q);
        }
        (*off)[k + 1] = (int)idx->size();
    }
}

static int upload_spots(rfba_ctx* ctx, const std::vector<Spot>& sp, cudaStream_t st, int set = 0) {
    int s;
    if ((s = ctx->gb[set].spots.ensure(sp.size() * 40 + 8, "3B spots"))) return s;
    if (!sp.empty())
        RFBA_CUDA(cudaMemcpyAsync(ctx->gb[set].spots.p, sp.data(), sp.size() * 40, cudaMemcpyHostToDevice, st),
                  "spots copy");
    return RFBA_OK;
}

// The block's data on the device (the context's Gibbs data buffers).
static int stage_block(rfba_ctx* ctx, const double* pix, const int* pixels, int F, int P, cudaStream_t st) {
    int s;
    const size_t FP = (size_t)F * P;
    if ((s = ctx->gb_pix.ensure(FP * 8, "3B data")) || (s = ctx->gb_pixels.ensure((size_t)P * 12, "3B pixels"))) return s;
    RFBA_CUDA(cudaMemcpyAsync(ctx->gb_pix.p, pix, FP * 8, cudaMemcpyHostToDevice, st), "data copy");
    RFBA_CUDA(cudaMemcpyAsync(ctx->gb_pixels.p, pixels, (size_t)P * 12, cudaMemcpyHostToDevice, st), "pixels copy");
    return RFBA_OK;
}

// Gibbs draws of the staged block with the spots `sp` (uploaded here) and
// flattened masks; the draws' intensities, spot `exclude` taken off, stay in
// gb_oint.
static int draws_without(rfba_ctx* ctx, const rfba_3b_model* m, int F, int P, const std::vector<Spot>& sp,
                         const std::vector<int>& hoff, const std::vector<int>& hidx, int n_draws, int sweeps,
                         int exclude, unsigned long long seed, cudaStream_t st) {
    int s;
    if ((s = upload_spots(ctx, sp, st))) return s;
    GibbsCall c;
    c.K = (int)sp.size();
    c.F = F;
    c.P = P;
    c.sweeps = sweeps;
    c.n_draws = n_draws;
    c.seed = seed;
    c.exclude = exclude;
    c.want_int = true;
    return gibbs_run(ctx, m, static_cast<const double*>(ctx->gb_pix.p), static_cast<const int*>(ctx->gb_pixels.p),
                     static_cast<const double*>(ctx->gb[0].spots.p), hoff, hidx, c, RFBA_DEVICE_PTRS, st);
}

// The spot optimiser's gradient on staged samples (NaN outside brightness,
// blur > 0, multispot5.cc:618-619).
struct StagedGradient {
    rfba_ctx* ctx;
    const rfba_3b_model* m;
    ThreeBData d;
    cudaStream_t st;
    int operator()(const double* x, double* g) {
        if (x[0] <= 0 || x[1] <= 0) {
            for (int n = 0; n < 5; ++n) g[n] = std::numeric_limits<double>::quiet_NaN();
            return RFBA_OK;
        }
        return threeb_eval(ctx, m, d, x, g, nullptr, st);
    }
};

// One pass of FitSpots::optimize_each_spot_in_turn_for_several_passes
// (multispot5.cc:1511-1690) on the staged block: spots sorted by the sweep
// order of `order_pass`, spot k's draws seeded pass_seed(seed, seed_pass, k).
static int optimise_pass_core(rfba_ctx* ctx, const rfba_3b_model* m, const int* pixels, int F, int P,
                              std::vector<Spot>* spots, int order_pass, int main_samples, int sweeps,
                              int cg_max_iterations, const double* limit, const AllowedArea& area,
                              unsigned long long seed, int seed_pass, int* evaluations, cudaStream_t st) {
    int s;
    std::vector<Spot>& sp = *spots;
    int K = (int)sp.size();
    // masks of every spot (multispot5.cc:1518-1521)
    std::vector<std::vector<int> > masks((size_t)K);
    for (int k = 0; k < K; ++k)
        if ((s = spot_mask(pixels, P, sp[k], &masks[k]))) return s;
    // the sweep order (multispot5.cc:1541-1560): by x or y position, ascending
    // or descending; the reference's third branch repeats `% 4 == 1` and is never
    // taken, so passes 2 and 3 both sort by descending y
    std::vector<int> order((size_t)K);
    for (int k = 0; k < K; ++k) order[k] = k;
    const int mode = order_pass % 4 == 0 ? 0 : order_pass % 4 == 1 ? 1 : 2;
    const int first = mode == 2 ? 3 : 2, second = first == 2 ? 3 : 2;
    std::sort(order.begin(), order.end(), [&](int a, int b) {
        const double fa = sp[a][first], fb = sp[b][first];
        const bool desc = mode != 0;
        if (desc ? fa > fb : fa < fb) return true;
        if (fa == fb) return desc ? sp[a][second] > sp[b][second] : sp[a][second] < sp[b][second];
        return false;
    });
    {
        std::vector<Spot> t((size_t)K);
        for (int k = 0; k < K; ++k) t[k] = sp[order[k]];
        sp.swap(t);
        // masks stay where they were: the reference swaps tmp_spot_pixels[i]
        // with spot_pixels[i], not spot_pixels[index[i]] (multispot5.cc:1570), so
        // a spot's mask is the one at its new position until it is optimised
    }
    int evals = 0;
    for (int k = 0; k < K; ++k) {
        // a fresh sampler for this spot: main_samples draws, the spot taken off
        // them (multispot5.cc:1591-1608)
        std::vector<int> hoff, hidx;
        flatten_masks(masks, (size_t)K, &hoff, &hidx);
        if ((s = draws_without(ctx, m, F, P, sp, hoff, hidx, main_samples, sweeps, k, pass_seed(seed, seed_pass, k),
                               st)))
            return s;
        // optimise the spot on those samples (multispot5.cc:1611-1636)
        StagedGradient grad{ctx, m, ThreeBData(), st};
        if ((s = threeb_stage(ctx, static_cast<const double*>(ctx->gb[0].oint.p), static_cast<const double*>(ctx->gb_pix.p),
                              static_cast<const int*>(ctx->gb_pixels.p), main_samples, F, P, RFBA_DEVICE_PTRS, st,
                              &grad.d, true)))
            return s;
        CgOnly5 cg;
        if ((s = cg.start(sp[k].data(), limit, grad))) return s;
        cg.max_iterations = cg_max_iterations;
        if ((s = cg.run(grad))) return s;
        evals += cg.evaluations;
        for (int n = 0; n < 5; ++n) sp[k][n] = cg.x[n];
        // new mask; eject the spot if it has no pixels or left the allowed area
        // (multispot5.cc:1651-1674)
        if ((s = spot_mask(pixels, P, sp[k], &masks[k]))) return s;
        if (masks[k].empty() || area.outside(sp[k])) {
            sp.erase(sp.begin() + k);
            masks.erase(masks.begin() + k);
            --K;
            --k;
        }
    }
    if (evaluations) *evaluations += evals;
    return RFBA_OK;
}

// The draws' residual sums into NegativeFreeEnergy::compute_with_mask's value
// (multispot5.cc:354-405), host arithmetic in the reference's order; err
// [samples][F]. residuals [samples] may be null.
static double free_energy_value(const rfba_3b_model* m, const std::vector<double>& err, int samples, int F, int P,
                                const double* spots, int K, double* residuals) {
    const double base_sigma = std::sqrt(m->variance);
    const double scale_pow = 100.0;
    const unsigned int npixels = (unsigned int)P, nframes = (unsigned int)F;
    double sum = 0;
    for (int sample = 0; sample < samples; sample++) {
        const double var1 = variance_from_sample(sample - 2, samples, base_sigma, scale_pow);
        const double var2 = variance_from_sample(sample - 1, samples, base_sigma, scale_pow);
        const double var3 = variance_from_sample(sample + 1, samples, base_sigma, scale_pow);
        const double var4 = variance_from_sample(sample + 2, samples, base_sigma, scale_pow);
        double err_sum = 0;
        for (int f = 0; f < F; ++f) err_sum -= err[(size_t)sample * F + f];
        if (residuals) residuals[sample] = -err_sum;
        const double e1 = err_sum / (2 * var1) - npixels * nframes * ::log(2 * M_PI * var1) / 2;
        const double e2 = err_sum / (2 * var2) - npixels * nframes * ::log(2 * M_PI * var2) / 2;
        const double e3 = err_sum / (2 * var3) - npixels * nframes * ::log(2 * M_PI * var3) / 2;
        const double e4 = err_sum / (2 * var4) - npixels * nframes * ::log(2 * M_PI * var4) / 2;
        sum += (-e1 + 8 * e2 - 8 * e3 + e4) / 12;
    }
    const double log_final =
        (::log(variance_from_sample(samples, samples, base_sigma, scale_pow) * 2 * M_PI) / 2) * npixels * nframes;
    double priors = 0;
    for (int i = 0; i < K; i++) {
        priors += log_log_normal(spots[i * 5 + 0], m->mu_brightness, m->sigma_brightness);
        priors += log_log_normal(spots[i * 5 + 1], m->mu_blur, m->sigma_blur);
    }
    return -(sum + priors - log_final);
}

// The free-energy draws: `samples` Gibbs draws from all spots off, draw i at
// the variance of thermodynamic step i - 1; their residual sums per frame.
static int free_energy_draws(rfba_ctx* ctx, const rfba_3b_model* m, const double* pix, const int* pixels,
                             const double* spots, const std::vector<int>& hoff, const std::vector<int>& hidx, int K,
                             int F, int P, int samples, int sweeps, unsigned long long seed, int ptr_flags,
                             cudaStream_t st, std::vector<double>* err) {
    const double base_sigma = std::sqrt(m->variance);
    std::vector<double> var2((size_t)samples);
    for (int i = 0; i < samples; ++i) var2[i] = variance_from_sample(i - 1, samples, base_sigma, 100.0);
    GibbsCall c;
    c.K = K;
    c.F = F;
    c.P = P;
    c.sweeps = sweeps;
    c.n_draws = samples;
    c.seed = seed;
    c.var_draw = var2.data();
    c.want_err = true;
    int s;
    if ((s = gibbs_run(ctx, m, pix, pixels, spots, hoff, hidx, c, ptr_flags, st))) return s;
    err->assign((size_t)samples * F, 0.0);
    RFBA_CUDA(cudaMemcpyAsync(err->data(), ctx->gb[0].oerr.p, err->size() * 8, cudaMemcpyDeviceToHost, st),
              "residual read-back");
    RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    return RFBA_OK;
}

// The negative free energies of n (1 or 2) models of the staged block side by
// side: their chains in one launch, as the reference runs the two of a model
// comparison on two threads (multispot5.cc:2096-2108). Model i uses the first
// sp[i]->size() masks of *masks[i].
static int model_energies(rfba_ctx* ctx, const rfba_3b_model* m, int F, int P, int n, const std::vector<Spot>* sp[],
                          const std::vector<std::vector<int> >* masks[], int samples, int sweeps,
                          const unsigned long long seeds[], cudaStream_t st, double energy[]) {
    int s;
    const double base_sigma = std::sqrt(m->variance);
    std::vector<double> var2((size_t)samples);
    for (int i = 0; i < samples; ++i) var2[i] = variance_from_sample(i - 1, samples, base_sigma, 100.0);
    GibbsParams g[2];
    for (int i = 0; i < n; ++i) {
        std::vector<int> hoff, hidx;
        flatten_masks(*masks[i], sp[i]->size(), &hoff, &hidx);
        if ((s = upload_spots(ctx, *sp[i], st, i))) return s;
        GibbsCall c;
        c.K = (int)sp[i]->size();
        c.F = F;
        c.P = P;
        c.sweeps = sweeps;
        c.n_draws = samples;
        c.seed = seeds[i];
        c.var_draw = var2.data();
        c.want_err = true;
        if ((s = gibbs_prepare(ctx, m, static_cast<const double*>(ctx->gb_pix.p),
                               static_cast<const int*>(ctx->gb_pixels.p), static_cast<const double*>(ctx->gb[i].spots.p),
                               hoff, hidx, c, RFBA_DEVICE_PTRS, st, i, &g[i])))
            return s;
    }
    if ((s = gibbs_launch(ctx, g, n, F, st))) return s;
    for (int i = 0; i < n; ++i) {
        std::vector<double> err((size_t)samples * F);
        RFBA_CUDA(cudaMemcpyAsync(err.data(), ctx->gb[i].oerr.p, err.size() * 8, cudaMemcpyDeviceToHost, st),
                  "residual read-back");
        RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
        energy[i] = -free_energy_value(m, err, samples, F, P, sp[i]->empty() ? nullptr : (*sp[i])[0].data(),
                                       (int)sp[i]->size(), nullptr);
    }
    return RFBA_OK;
}

// hess_log_log_normal (storm.h:446-449)
static double hess_log_log_normal(double x, double mu, double sigma) {
    return (1 + (ref_ln(x) - mu - 1) / (sigma * sigma)) / (x * x);
}

// The device part of sampled_background_spot_hessian_ffbs on device data and
// the reference's normalisation on the host (multispot5.cc:902-985).
static int spot_hessian_dev(rfba_ctx* ctx, const rfba_3b_model* m, const double* bg, const double* pix,
                            const int* pixels, int S, int F, int P, const double spot[5], int bs,
                            unsigned long long seed, double hess[25], cudaStream_t st) {
    int s;
    const int nc = hessian_chunks(S, F, P, ctx->sm_count);
    const size_t nq = (size_t)S * F;
    if ((s = ctx->hs_tab.ensure((size_t)P * 21 * 8, "3B Hessian table")) ||
        (s = ctx->hs_part.ensure((size_t)nc * nq * 22 * 8, "3B Hessian parts")) ||
        (s = ctx->hs_gg.ensure(15 * 8, "3B Hessian outer products")) ||
        (s = ctx->hs_phi.ensure(5 * 8, "3B Hessian spot")) ||
        (s = ctx->hs_frame.ensure(nq * 20 * 8, "3B Hessian frame parts")) ||
        (s = ctx->hs_out.ensure((size_t)S * 20 * 8, "3B Hessian sums")))
        return s;
    RFBA_CUDA(cudaMemcpyAsync(ctx->hs_phi.p, spot, 40, cudaMemcpyHostToDevice, st), "spot upload");
    HessParams h;
    h.bg = bg;
    h.pix = pix;
    h.pixels = pixels;
    h.phi = static_cast<const double*>(ctx->hs_phi.p);
    h.zf = m->z_factor;
    h.variance = m->variance;
    for (int n = 0; n < 9; ++n) h.A[n] = m->A[n];
    for (int n = 0; n < 3; ++n) h.pi[n] = m->pi[n];
    h.S = S;
    h.F = F;
    h.P = P;
    h.nc = nc;
    h.bs = bs;
    h.seed = seed;
    h.tab = static_cast<double*>(ctx->hs_tab.p);
    h.part = static_cast<double*>(ctx->hs_part.p);
    h.gg = static_cast<double*>(ctx->hs_gg.p);
    h.frame = static_cast<double*>(ctx->hs_frame.p);
    h.out = static_cast<double*>(ctx->hs_out.p);
    const int e = launch_spot_hessian(h, st);
    if (e) return cuda_fail((cudaError_t)e, "3B Hessian launch");
    ctx->launches += 4;
    std::vector<double> out((size_t)S * 20);
    RFBA_CUDA(cudaMemcpyAsync(out.data(), ctx->hs_out.p, out.size() * 8, cudaMemcpyDeviceToHost, st),
              "Hessian read-back");
    RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    double sh[15] = {0}, sd[5] = {0};
    for (int i = 0; i < S; ++i) {
        for (int n = 0; n < 15; ++n) sh[n] += out[(size_t)i * 20 + n];
        for (int r = 0; r < 5; ++r) sd[r] += out[(size_t)i * 20 + 15 + r];
    }
    const double norm = (double)((size_t)bs * (size_t)S) * m->variance;
    for (int r = 0, n = 0; r < 5; ++r)
        for (int c = r; c < 5; ++c, ++n) hess[r * 5 + c] = hess[c * 5 + r] = sh[n] / norm;
    for (int r = 0; r < 5; ++r) sd[r] /= norm;
    for (int r = 0; r < 5; ++r)
        for (int c = 0; c < 5; ++c) hess[r * 5 + c] -= sd[r] * sd[c];
    hess[0] += hess_log_log_normal(spot[0], m->mu_brightness, m->sigma_brightness);
    hess[6] += hess_log_log_normal(spot[1], m->mu_blur, m->sigma_blur);
    return RFBA_OK;
}

// diff_log_log_normal (storm.h:431-434)
static double diff_log_log_normal(double x, double mu, double sigma) {
    return -(1 + (ref_ln(x) - mu) / (sigma * sigma)) / x;
}

// FreeEnergyHessian::hessian (multispot5.cc:693-775) on the staged block: the
// unmasked sampler (GibbsSampler) draws `samples` times with every spot in
// the model; per draw, over the frames where spot `which` is on, the spot's
// hess + its priors' second derivatives and deriv + its priors' first
// derivatives; the sums of hess and of deriv deriv^T over the draws, over
// (samples variance), less the outer product of the mean deriv.
static int free_energy_hessian_dev(rfba_ctx* ctx, const rfba_3b_model* m, const int* pixels, int F, int P,
                                   const std::vector<Spot>& sp, int which, int samples, int sweeps,
                                   unsigned long long seed, double hess[25], cudaStream_t st) {
    int s;
    const int K = (int)sp.size();
    std::vector<int> hoff, hidx;
    support_masks(pixels, P, sp, m->z_factor, &hoff, &hidx);
    if ((s = upload_spots(ctx, sp, st))) return s;
    GibbsCall c;
    c.K = K;
    c.F = F;
    c.P = P;
    c.sweeps = sweeps;
    c.n_draws = samples;
    c.seed = seed;
    c.want_state = true;
    c.want_int = true;
    if ((s = gibbs_run(ctx, m, static_cast<const double*>(ctx->gb_pix.p), static_cast<const int*>(ctx->gb_pixels.p),
                       static_cast<const double*>(ctx->gb[0].spots.p), hoff, hidx, c, RFBA_DEVICE_PTRS, st)))
        return s;
    const int nc = hessian_chunks(samples, F, P, ctx->sm_count);
    const size_t nq = (size_t)samples * F;
    if ((s = ctx->hs_tab.ensure((size_t)P * 21 * 8, "3B Hessian table")) ||
        (s = ctx->hs_part.ensure((size_t)nc * nq * 22 * 8, "3B Hessian parts")) ||
        (s = ctx->hs_gg.ensure(15 * 8, "3B Hessian outer products")) || (s = ctx->hs_phi.ensure(5 * 8, "3B Hessian spot")))
        return s;
    RFBA_CUDA(cudaMemcpyAsync(ctx->hs_phi.p, sp[which].data(), 40, cudaMemcpyHostToDevice, st), "spot upload");
    HessParams h;
    std::memset(&h, 0, sizeof h);
    h.bg = static_cast<const double*>(ctx->gb[0].oint.p);
    h.pix = static_cast<const double*>(ctx->gb_pix.p);
    h.pixels = static_cast<const int*>(ctx->gb_pixels.p);
    h.phi = static_cast<const double*>(ctx->hs_phi.p);
    h.zf = m->z_factor;
    h.S = samples;
    h.F = F;
    h.P = P;
    h.nc = nc;
    h.tab = static_cast<double*>(ctx->hs_tab.p);
    h.part = static_cast<double*>(ctx->hs_part.p);
    h.gg = static_cast<double*>(ctx->hs_gg.p);
    const int e = launch_hessian_parts(h, true, st);
    if (e) return cuda_fail((cudaError_t)e, "3B free-energy Hessian launch");
    ctx->launches += 3;
    std::vector<double> part((size_t)nc * nq * 22), gg(15);
    std::vector<unsigned char> states((size_t)samples * K * F);
    RFBA_CUDA(cudaMemcpyAsync(part.data(), ctx->hs_part.p, part.size() * 8, cudaMemcpyDeviceToHost, st), "parts read");
    RFBA_CUDA(cudaMemcpyAsync(gg.data(), ctx->hs_gg.p, 15 * 8, cudaMemcpyDeviceToHost, st), "parts read");
    RFBA_CUDA(cudaMemcpyAsync(states.data(), ctx->gb[0].ostate.p, states.size(), cudaMemcpyDeviceToHost, st),
              "states read");
    RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    const Spot& sw = sp[which];
    double sum1[25] = {0}, sum2[25] = {0}, sumd[5] = {0};
    for (int i = 0; i < samples; ++i) {
        double H[25] = {0}, d[5] = {0};
        for (int f = 0; f < F; ++f) {
            if (states[((size_t)i * K + which) * F + f] != 0) continue;
            const size_t q = (size_t)f * samples + i;
            double v[22] = {0};
            for (int ch = 0; ch < nc; ++ch)
                for (int n = 0; n < 22; ++n) v[n] += part[((size_t)ch * nq + q) * 22 + n];
            for (int r = 0, n = 0; r < 5; ++r)
                for (int cc = r; cc < 5; ++cc, ++n) {
                    const double x = v[2 + n] - gg[n];
                    H[r * 5 + cc] += x;
                    if (cc != r) H[cc * 5 + r] += x;
                }
            for (int r = 0; r < 5; ++r) d[r] += v[17 + r];
        }
        H[0] += hess_log_log_normal(sw[0], m->mu_brightness, m->sigma_brightness);
        H[6] += hess_log_log_normal(sw[1], m->mu_blur, m->sigma_blur);
        d[0] += diff_log_log_normal(sw[0], m->mu_brightness, m->sigma_brightness);
        d[1] += diff_log_log_normal(sw[1], m->mu_blur, m->sigma_blur);
        for (int n = 0; n < 25; ++n) sum1[n] += H[n];
        for (int r = 0; r < 5; ++r)
            for (int cc = 0; cc < 5; ++cc) sum2[r * 5 + cc] += d[r] * d[cc];
        for (int r = 0; r < 5; ++r) sumd[r] += d[r];
    }
    const double norm = (double)samples * m->variance;
    for (int n = 0; n < 25; ++n) {
        sum1[n] /= norm;
        sum2[n] /= norm;
    }
    for (int r = 0; r < 5; ++r) sumd[r] /= norm;
    for (int r = 0; r < 5; ++r)
        for (int cc = 0; cc < 5; ++cc) hess[r * 5 + cc] = sum1[r * 5 + cc] + sum2[r * 5 + cc] - sumd[r] * sumd[cc];
    return RFBA_OK;
}

// Eigen-decomposition of a symmetric 5x5 matrix by cyclic Jacobi rotations
// (Jacobi 1846; Golub and Van Loan, Matrix Computations, sec. 8.5): eigenvalues
// ascending, eigenvectors as rows, each with its largest-magnitude component
// positive.
static void sym_eigen5(const double a_in[25], double evals[5], double evecs[25]) {
    double a[5][5], v[5][5];
    for (int r = 0; r < 5; ++r)
        for (int c = 0; c < 5; ++c) {
            a[r][c] = 0.5 * (a_in[r * 5 + c] + a_in[c * 5 + r]);
            v[r][c] = r == c ? 1.0 : 0.0;
        }
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = 0, diag = 0;
        for (int r = 0; r < 5; ++r) {
            diag += a[r][r] * a[r][r];
            for (int c = r + 1; c < 5; ++c) off += a[r][c] * a[r][c];
        }
        if (off <= 1e-30 * diag || off == 0) break;
        for (int p = 0; p < 4; ++p)
            for (int q = p + 1; q < 5; ++q) {
                if (a[p][q] == 0) continue;
                const double theta = (a[q][q] - a[p][p]) / (2 * a[p][q]);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
                const double c = 1 / std::sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < 5; ++k) {
                    if (k == p || k == q) continue;
                    const double akp = a[k][p], akq = a[k][q];
                    a[k][p] = a[p][k] = c * akp - s * akq;
                    a[k][q] = a[q][k] = s * akp + c * akq;
                }
                const double apq = a[p][q];
                a[p][p] -= t * apq;
                a[q][q] += t * apq;
                a[p][q] = a[q][p] = 0;
                for (int k = 0; k < 5; ++k) {
                    const double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = c * vkp - s * vkq;
                    v[k][q] = s * vkp + c * vkq;
                }
            }
    }
    int idx[5] = {0, 1, 2, 3, 4};
    std::sort(idx, idx + 5, [&](int x, int y) { return a[x][x] < a[y][y]; });
    for (int n = 0; n < 5; ++n) {
        const int j = idx[n];
        evals[n] = a[j][j];
        int big = 0;
        for (int k = 1; k < 5; ++k)
            if (std::fabs(v[k][j]) > std::fabs(v[big][j])) big = k;
        const double sg = v[big][j] < 0 ? -1.0 : 1.0;
        for (int k = 0; k < 5; ++k) evecs[n * 5 + k] = sg * v[k][j];
    }
}

// Determinant of a 5x5 matrix by Gaussian elimination with partial pivoting.
static double det5(const double a_in[25]) {
    double a[5][5];
    for (int r = 0; r < 5; ++r)
        for (int c = 0; c < 5; ++c) a[r][c] = a_in[r * 5 + c];
    double det = 1;
    for (int c = 0; c < 5; ++c) {
        int piv = c;
        for (int r = c + 1; r < 5; ++r)
            if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
        if (a[piv][c] == 0) return 0;
        if (piv != c) {
            for (int k = 0; k < 5; ++k) std::swap(a[c][k], a[piv][k]);
            det = -det;
        }
        det *= a[c][c];
        for (int r = c + 1; r < 5; ++r) {
            const double f = a[r][c] / a[c][c];
            for (int k = c; k < 5; ++k) a[r][k] -= f * a[c][k];
        }
    }
    return det;
}

// log_normal_mode (storm.h:402-405)
static double log_normal_mode(double mu, double sigma) { return std::exp(mu - sigma * sigma); }

// One try of FitSpots::try_modifying_model (multispot5.cc:1840-2160) on the
// staged block.
static int modify_core(rfba_ctx* ctx, const rfba_3b_model* m, const int* pixels, int F, int P,
                       std::vector<Spot>* spots, const rfba_3b_fit_params& prm, const AllowedArea& area,
                       unsigned long long seed, rfba_3b_modify_record* rec, cudaStream_t st) {
    int s;
    HostUniform rng{seed};
    std::vector<Spot>& sp = *spots;
    const int K = (int)sp.size();
    std::memset(rec, 0, sizeof *rec);
    // seconds in: draws, optimiser, Hessians, free energies
    double secs[4] = {0, 0, 0, 0};
    auto clock = [] { return std::chrono::steady_clock::now(); };
    auto since = [](std::chrono::steady_clock::time_point t0) {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    };
    // add with probability 1/2, always with one spot (multispot5.cc:1851) and,
    // here, with none (the reference would index an empty list)
    const bool add = rng.next() > 0.5 || K <= 1;
    std::vector<Spot> model1, model2;
    int original;
    if (add) {
        model1 = sp;
        model2 = sp;
        Spot n;
        n[0] = log_normal_mode(m->mu_brightness, m->sigma_brightness);
        n[1] = log_normal_mode(m->mu_blur, m->sigma_blur);
        if (prm.guide_map) {  // GetPoint (multispot5.cc:2210-2231): a subvoxel drawn by the SRRF map
            float xyz[3];
            if ((s = seed_spots_locked(ctx, prm.guide_map, prm.guide_dims, prm.guide_mag, pixels, P, 1,
                                       mix_seed(seed, 7, 0), xyz, RFBA_HOST_PTRS, st)))
                return s;
            for (int a = 0; a < 3; ++a) n[2 + a] = xyz[a];
        } else {
            const int r = std::min(P - 1, (int)(rng.next() * P));
            for (int a = 0; a < 3; ++a) n[2 + a] = pixels[3 * r + a] + rng.next() - .5;
        }
        model2.push_back(n);
        original = 1;
    } else {
        const int a = std::min(K - 1, (int)(rng.next() * K));
        model1 = sp;
        std::swap(model1[K - 1], model1[a]);
        model2 = model1;
        model1.pop_back();
        original = 2;
    }
    rec->added = add ? 1 : 0;
    const int spot = (int)model2.size() - 1;
    std::vector<std::vector<int> > masks2(model2.size());
    for (size_t k = 0; k < model2.size(); ++k)
        if ((s = spot_mask(pixels, P, model2[k], &masks2[k]))) return s;
    // optimise the mobile spot on GibbsSampler2 draws (multispot5.cc:1935-2010)
    {
        std::vector<int> hoff, hidx;
        flatten_masks(masks2, model2.size(), &hoff, &hidx);
        const int S = prm.opt_samples;
        auto t0 = clock();
        if ((s = draws_without(ctx, m, F, P, model2, hoff, hidx, S, prm.sweeps, spot, mix_seed(seed, 1, 0), st)))
            return s;
        secs[0] += since(t0);
        StagedGradient grad{ctx, m, ThreeBData(), st};
        if ((s = threeb_stage(ctx, static_cast<const double*>(ctx->gb[0].oint.p), static_cast<const double*>(ctx->gb_pix.p),
                              static_cast<const int*>(ctx->gb_pixels.p), S, F, P, RFBA_DEVICE_PTRS, st, &grad.d,
                              true)))
            return s;
        CgOnly5 cg;
        if ((s = cg.start(model2[spot].data(), prm.limit, grad))) return s;
        for (int attempt = 0; attempt < prm.opt_attempts; attempt++) {
            t0 = clock();
            if ((s = cg.run(grad))) return s;
            secs[1] += since(t0);
            if (attempt < prm.opt_attempts - 1) {
                double H[25], ev[5], V[25];
                t0 = clock();
                if ((s = spot_hessian_dev(ctx, m, static_cast<const double*>(ctx->gb[0].oint.p),
                                          static_cast<const double*>(ctx->gb_pix.p),
                                          static_cast<const int*>(ctx->gb_pixels.p), S, F, P, cg.x,
                                          prm.opt_hess_inner_samples, mix_seed(seed, 2, attempt), H, st)))
                    return s;
                secs[2] += since(t0);
                sym_eigen5(H, ev, V);
                if (ev[4] < 0) break;  // negative definite
                // restart along the fourth eigenvector (ascending order)
                double x0[5];
                for (int n = 0; n < 5; ++n) x0[n] = cg.x[n] + 0.1 * V[15 + n];
                cg.restart(x0, V + 15);
            }
        }
        for (int n = 0; n < 5; ++n) model2[spot][n] = cg.x[n];
        rec->evaluations = cg.evaluations;
        if ((s = spot_mask(pixels, P, model2[spot], &masks2[spot]))) return s;
    }
    for (int n = 0; n < 5; ++n) rec->spot[n] = model2[spot][n];
    int keep = original;
    if (area.outside(model2[spot])) {
        keep = 1;  // model 2's spot has zero prior probability
        rec->zero_prior = 1;
    } else {
        const double pos_lp =
            area.use ? (double)(model2.size() - model1.size()) * ref_ln(1.0 / (double)area.cells.size()) : 0.0;
        rec->position_log_prior = pos_lp;
        // the Hessian at model 2's spot on GibbsSampler draws over all pixels
        // (multispot5.cc:2050-2075)
        std::vector<int> hoff, hidx;
        support_masks(pixels, P, model2, m->z_factor, &hoff, &hidx);
        const int S = prm.h_outer_samples;
        auto t0 = clock();
        if ((s = draws_without(ctx, m, F, P, model2, hoff, hidx, S, prm.sweeps, spot, mix_seed(seed, 3, 0), st)))
            return s;
        secs[0] += since(t0);
        double H[25], negH[25], ev[5], V[25];
        t0 = clock();
        if ((s = spot_hessian_dev(ctx, m, static_cast<const double*>(ctx->gb[0].oint.p),
                                  static_cast<const double*>(ctx->gb_pix.p), static_cast<const int*>(ctx->gb_pixels.p), S,
                                  F, P, model2[spot].data(), prm.h_inner_samples, mix_seed(seed, 4, 0), H, st)))
            return s;
        secs[2] += since(t0);
        double scaled[25];
        for (int n = 0; n < 25; ++n) {
            negH[n] = -H[n];
            scaled[n] = -H[n] / (M_PI * 2);
        }
        const double det = det5(scaled);
        sym_eigen5(negH, ev, V);
        if (ev[0] > 1e-6) {
            t0 = clock();
            const std::vector<Spot>* models[2] = {&model2, &model1};
            const std::vector<std::vector<int> >* mk[2] = {&masks2, &masks2};
            const unsigned long long seeds[2] = {mix_seed(seed, 5, 0), mix_seed(seed, 6, 0)};
            double en[2];
            if ((s = model_energies(ctx, m, F, P, 2, models, mk, prm.thermo_samples, prm.sweeps, seeds, st, en)))
                return s;
            const double e2 = en[0], e1 = en[1];
            secs[3] += since(t0);
            const double occam = -0.5 * std::log(det);
            const double p2 = e2 + occam + pos_lp;
            rec->model1_energy = e1;
            rec->model2_energy = e2;
            rec->occam = occam;
            keep = p2 > e1 ? 2 : 1;
        } else {
            rec->bad_hessian = 1;  // a saddle point: keep the original model
        }
    }
    rec->kept = keep;
    sp = keep == 2 ? model2 : model1;
    if (verbose())
        std::fprintf(stderr,
                     "rfba: 3B modification (%s, kept %d): draws %.3f s, optimiser %.3f s (%d evaluations), "
                     "Hessians %.3f s, free energies %.3f s\n",
                     add ? "add" : "remove", keep, secs[0], secs[1], rec->evaluations, secs[2], secs[3]);
    return RFBA_OK;
}

static int fit_check(rfba_ctx* ctx, const rfba_3b_model* m, const double* pix, const int* pixels, int F, int P,
                     const double* spots, const int* nspots, int capacity, const rfba_3b_fit_params* prm) {
    int s;
    if (!pix || !pixels || !spots || !nspots || !prm) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    if ((s = gibbs_check(ctx, m, *nspots, F, P, RFBA_HOST_PTRS))) return s;
    if (capacity < *nspots + 1) {
        set_error("spots capacity must hold one spot more than *nspots");
        return RFBA_ERR_INVALID;
    }
    if (prm->main_samples < 1 || prm->sweeps < 1 || prm->main_cg_max_iterations < 0 || prm->main_passes < 0 ||
        prm->add_remove_tries < 0 || prm->opt_samples < 1 || prm->opt_attempts < 1 ||
        prm->opt_hess_inner_samples < 1 || prm->h_outer_samples < 1 || prm->h_inner_samples < 1 ||
        prm->thermo_samples < 1) {
        set_error("fit settings: sample counts and attempts must be >= 1, passes / tries / iterations >= 0");
        return RFBA_ERR_INVALID;
    }
    if (prm->guide_map && (prm->guide_mag < 1 || prm->guide_dims[0] < 1 || prm->guide_dims[1] < 1 ||
                           prm->guide_dims[2] < 1)) {
        set_error("guide map: magnification and dims must be >= 1");
        return RFBA_ERR_INVALID;
    }
    return RFBA_OK;
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
        const float radius = (float)(sp[1] * 6 + 1);
        const int ox = round_away(sp[2]), oy = round_away(sp[3]), oz = round_away(sp[4]);
        const double r = std::ceil((double)radius + 1);
        if (!(r < 1024) || (2 * r + 1) * (2 * r + 1) * (2 * r + 1) > (double)P) {
            // a ball with more offsets than the block has pixels: test the
            // pixels instead. They are sorted by (z, y, x), and so are their
            // offsets from the centre, which is the ball's order; a blur that is
            // not finite gives an empty mask
            for (int q = 0; q < P; ++q) {
                const long long d[3] = {(long long)pixels[3 * q] - ox, (long long)pixels[3 * q + 1] - oy,
                                        (long long)pixels[3 * q + 2] - oz};
                if (std::fabs((double)d[0]) > r || std::fabs((double)d[1]) > r || std::fabs((double)d[2]) > r) continue;
                const unsigned int m2 = (unsigned int)(d[0] * d[0]) + (unsigned int)(d[1] * d[1]) +
                                        (unsigned int)(d[2] * d[2]);
                if ((float)m2 <= radius * radius) {
                    if (mask_pixels && n < cap) mask_pixels[n] = q;
                    ++n;
                }
            }
        } else {
            const std::vector<int> b = ball(radius);
            for (size_t j = 0; j < b.size(); j += 3) {
                const int t[3] = {b[j] + ox, b[j + 1] + oy, b[j + 2] + oz};
                int lo = 0, hi = P;  // lower_bound
                while (lo < hi) {
                    const int mid = (lo + hi) / 2;
                    const int* q = pixels + 3 * mid;
                    const bool lt = q[2] < t[2] || (q[2] == t[2] && q[1] < t[1]) ||
                                    (q[2] == t[2] && q[1] == t[1] && q[0] < t[0]);
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
    copy_out(states, ctx->gb[0].ostate.p, (size_t)n_draws * K * F, ptr_flags, st, &s);
    copy_out(sample_intensities, ctx->gb[0].oint.p, (size_t)n_draws * F * P * 8, ptr_flags, st, &s);
    if (s) return s;
    RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    return RFBA_OK;
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
    const int K = *nspots;
    if ((s = gibbs_check(ctx, m, K, F, P, RFBA_HOST_PTRS))) return s;
    if (main_samples < 1 || sweeps < 1 || cg_max_iterations < 0) {
        set_error("main_samples and sweeps must be >= 1, cg_max_iterations >= 0");
        return RFBA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    if ((s = order_streams(ctx, st))) return s;
    AllowedArea area;
    area.build(pixels, P, position_extra_radius);
    std::vector<Spot> sp((size_t)K);
    for (int k = 0; k < K; ++k)
        for (int n = 0; n < 5; ++n) sp[k][n] = spots[5 * k + n];
    if ((s = stage_block(ctx, pixel_intensities, pixels, F, P, st))) return s;
    int evals = 0;
    if ((s = optimise_pass_core(ctx, m, pixels, F, P, &sp, pass, main_samples, sweeps, cg_max_iterations, limit, area,
                                seed, pass, &evals, st)))
        return s;
    for (size_t k = 0; k < sp.size(); ++k)
        for (int n = 0; n < 5; ++n) spots[5 * k + n] = sp[k][n];
    *nspots = (int)sp.size();
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
    copy_out(states, ctx->gb[0].ostate.p, (size_t)K * F, ptr_flags, st, &s);
    copy_out(log_prob, ctx->gb[0].lp.p, (size_t)K * F * 16, ptr_flags, st, &s);
    copy_out(filtered, ctx->gb[0].filt.p, (size_t)K * F * 24, ptr_flags, st, &s);
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
    std::vector<double> err;
    if ((s = free_energy_draws(ctx, m, pixel_intensities, pixels, spots, hoff, hidx, K, F, P, samples, sweeps, seed,
                               ptr_flags, st, &err)))
        return s;
    *value = free_energy_value(m, err, samples, F, P, hsp.data(), K, residuals);
    return RFBA_OK;
}

// sampled_background_spot_hessian_ffbs (multispot5.cc:902-985)
int rfba_3b_spot_hessian(rfba_ctx* ctx, const rfba_3b_model* m, const double* sample_bg,
                         const double* pixel_intensities, const int* pixels, int S, int F, int P,
                         const double spot[5], int bs_iterations, unsigned long long seed, double hess[25],
                         int ptr_flags, void* stream) {
    if (!ctx || !m || !sample_bg || !pixel_intensities || !pixels || !spot || !hess) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    int s;
    if ((s = threeb_validate(m, S, F, P, ptr_flags))) return s;
    if (F > 2048 || bs_iterations < 1) {
        set_error("F must be <= 2048 and bs_iterations >= 1");
        return RFBA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if ((s = order_streams(ctx, st))) return s;
    ThreeBData d;
    if ((s = threeb_stage(ctx, sample_bg, pixel_intensities, pixels, S, F, P, ptr_flags, st, &d))) return s;
    return spot_hessian_dev(ctx, m, d.bg, d.pix, d.pixels, S, F, P, spot, bs_iterations, seed, hess, st);
}

// One try of FitSpots::try_modifying_model (multispot5.cc:1840-2160).
int rfba_3b_modify_model(rfba_ctx* ctx, const rfba_3b_model* m, const double* pixel_intensities, const int* pixels,
                         int F, int P, double* spots, int* nspots, int capacity, const rfba_3b_fit_params* prm,
                         unsigned long long seed, rfba_3b_modify_record* record) {
    int s;
    if ((s = fit_check(ctx, m, pixel_intensities, pixels, F, P, spots, nspots, capacity, prm))) return s;
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    if ((s = order_streams(ctx, st))) return s;
    AllowedArea area;
    area.build(pixels, P, prm->position_extra_radius);
    std::vector<Spot> sp((size_t)*nspots);
    for (size_t k = 0; k < sp.size(); ++k)
        for (int n = 0; n < 5; ++n) sp[k][n] = spots[5 * k + n];
    if ((s = stage_block(ctx, pixel_intensities, pixels, F, P, st))) return s;
    rfba_3b_modify_record rec;
    if ((s = modify_core(ctx, m, pixels, F, P, &sp, *prm, area, seed, &rec, st))) return s;
    for (size_t k = 0; k < sp.size(); ++k)
        for (int n = 0; n < 5; ++n) spots[5 * k + n] = sp[k][n];
    *nspots = (int)sp.size();
    if (record) *record = rec;
    return RFBA_OK;
}

// FitSpots::run (multispot5.cc:2234-2278): iterations of the passes and the
// model modifications.
int rfba_3b_fit(rfba_ctx* ctx, const rfba_3b_model* m, const double* pixel_intensities, const int* pixels, int F,
                int P, double* spots, int* nspots, int capacity, const rfba_3b_fit_params* prm, int first_iteration,
                int iterations, unsigned long long seed, rfba_3b_fit_fn progress, void* user) {
    int s;
    if ((s = fit_check(ctx, m, pixel_intensities, pixels, F, P, spots, nspots, capacity, prm))) return s;
    if (first_iteration < 0 || iterations < 0) {
        set_error("first_iteration and iterations must be >= 0");
        return RFBA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    if ((s = order_streams(ctx, st))) return s;
    AllowedArea area;
    area.build(pixels, P, prm->position_extra_radius);
    std::vector<Spot> sp((size_t)*nspots);
    for (size_t k = 0; k < sp.size(); ++k)
        for (int n = 0; n < 5; ++n) sp[k][n] = spots[5 * k + n];
    if ((s = stage_block(ctx, pixel_intensities, pixels, F, P, st))) return s;
    std::vector<double> flat;
    auto report = [&](int it, int step) -> bool {
        if (!progress) return false;
        flat.assign(sp.size() * 5, 0.0);
        for (size_t k = 0; k < sp.size(); ++k)
            for (int n = 0; n < 5; ++n) flat[5 * k + n] = sp[k][n];
        return progress(it, step, flat.data(), (int)sp.size(), user) != 0;
    };
    bool stop = false;
    for (int it = first_iteration; it < first_iteration + iterations && !stop; ++it) {
        const unsigned long long it_seed = mix_seed(seed, it, -1);
        for (int pass = 0; pass < prm->main_passes && !stop; ++pass) {
            int evals = 0;
            if ((s = optimise_pass_core(ctx, m, pixels, F, P, &sp, pass + it, prm->main_samples, prm->sweeps,
                                        prm->main_cg_max_iterations, prm->limit, area, it_seed, pass, &evals, st)))
                return s;
            stop = report(it, pass);
        }
        for (int t = 0; t < prm->add_remove_tries && !stop; ++t) {
            if ((int)sp.size() + 1 > capacity) break;
            rfba_3b_modify_record rec;
            if ((s = modify_core(ctx, m, pixels, F, P, &sp, *prm, area, mix_seed(it_seed, 1 << 20, t), &rec, st)))
                return s;
            stop = report(it, prm->main_passes + t);
        }
    }
    for (size_t k = 0; k < sp.size(); ++k)
        for (int n = 0; n < 5; ++n) spots[5 * k + n] = sp[k][n];
    *nspots = (int)sp.size();
    return RFBA_OK;
}

// FreeEnergyHessian::hessian (multispot5.cc:693-775)
int rfba_3b_free_energy_hessian(rfba_ctx* ctx, const rfba_3b_model* m, const double* pixel_intensities,
                                const int* pixels, const double* spots, int K, int F, int P, int spot, int samples,
                                int sweeps, unsigned long long seed, double hess[25]) {
    int s;
    if (!pixel_intensities || !pixels || !spots || !hess) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    if ((s = gibbs_check(ctx, m, K, F, P, RFBA_HOST_PTRS))) return s;
    if (K < 1 || spot < 0 || spot >= K || samples < 1 || sweeps < 1) {
        set_error("spot outside [0, K), or samples / sweeps < 1");
        return RFBA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    if ((s = order_streams(ctx, st))) return s;
    std::vector<Spot> sp((size_t)K);
    for (int k = 0; k < K; ++k)
        for (int n = 0; n < 5; ++n) sp[k][n] = spots[5 * k + n];
    if ((s = stage_block(ctx, pixel_intensities, pixels, F, P, st))) return s;
    return free_energy_hessian_dev(ctx, m, pixels, F, P, sp, spot, samples, sweeps, seed, hess, st);
}

// NegativeFreeEnergy::compute_with_mask for one or two models side by side
// (the two chains in one launch).
int rfba_3b_free_energy_models(rfba_ctx* ctx, const rfba_3b_model* m, const double* pixel_intensities,
                               const int* pixels, int F, int P, int nmodels, const double* const* spots, const int* K,
                               const int* const* mask_offsets, const int* const* mask_pixels, int samples, int sweeps,
                               const unsigned long long* seeds, double* values) {
    int s;
    if (!pixel_intensities || !pixels || !spots || !K || !mask_offsets || !mask_pixels || !seeds || !values ||
        nmodels < 1 || nmodels > 2 || samples < 1 || sweeps < 1) {
        set_error("null argument, nmodels outside [1, 2], or samples / sweeps < 1");
        return RFBA_ERR_INVALID;
    }
    for (int i = 0; i < nmodels; ++i) {
        if ((s = gibbs_check(ctx, m, K[i], F, P, RFBA_HOST_PTRS))) return s;
        if (K[i] > 0 && (!spots[i] || !mask_pixels[i])) {
            set_error("null spots or masks");
            return RFBA_ERR_INVALID;
        }
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    if ((s = order_streams(ctx, st))) return s;
    std::vector<Spot> sp[2];
    std::vector<std::vector<int> > masks[2];
    for (int i = 0; i < nmodels; ++i) {
        if (!mask_offsets[i]) {
            set_error("null mask offsets");
            return RFBA_ERR_INVALID;
        }
        std::vector<int> hoff, hidx;
        if ((s = gibbs_masks(mask_offsets[i], mask_pixels[i], K[i], P, RFBA_HOST_PTRS, st, &hoff, &hidx))) return s;
        sp[i].resize((size_t)K[i]);
        masks[i].resize((size_t)K[i]);
        for (int k = 0; k < K[i]; ++k) {
            for (int n = 0; n < 5; ++n) sp[i][k][n] = spots[i][5 * k + n];
            masks[i][k].assign(hidx.begin() + hoff[k], hidx.begin() + hoff[k + 1]);
        }
    }
    if ((s = stage_block(ctx, pixel_intensities, pixels, F, P, st))) return s;
    const std::vector<Spot>* models[2] = {&sp[0], &sp[1]};
    const std::vector<std::vector<int> >* mk[2] = {&masks[0], &masks[1]};
    double en[2];
    if ((s = model_energies(ctx, m, F, P, nmodels, models, mk, samples, sweeps, seeds, st, en))) return s;
    for (int i = 0; i < nmodels; ++i) values[i] = -en[i];
    return RFBA_OK;
}

int rfba_3b_support_masks(const int* pixels, int P, const double* spots, int K, double z_factor, int* mask_offsets,
                          int* mask_pixels, long long cap, long long* nnz) {
    if (!pixels || P < 1 || K < 0 || (K > 0 && !spots) || !mask_offsets || !nnz || z_factor == 0) {
        set_error("null argument, bad sizes or z_factor 0");
        return RFBA_ERR_INVALID;
    }
    std::vector<Spot> sp((size_t)K);
    for (int k = 0; k < K; ++k)
        for (int n = 0; n < 5; ++n) sp[k][n] = spots[5 * k + n];
    std::vector<int> off, idx;
    support_masks(pixels, P, sp, z_factor, &off, &idx);
    std::memcpy(mask_offsets, off.data(), off.size() * sizeof(int));
    if (mask_pixels) std::memcpy(mask_pixels, idx.data(), std::min<size_t>(idx.size(), (size_t)std::max(cap, 0LL)) * 4);
    *nnz = (long long)idx.size();
    return RFBA_OK;
}

int rfba_sym_eigen5(const double a[25], double evals[5], double evecs[25]) {
    if (!a || !evals || !evecs) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    sym_eigen5(a, evals, evecs);
    return RFBA_OK;
}

double rfba_det5(const double a[25]) { return a ? det5(a) : 0.0; }


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
    if ((s = threeb_stage(ctx, sample_bg, pixel_intensities, pixels, S, F, P, ptr_flags, st, &d, !log_prob)))
        return s;
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
    if ((s = threeb_stage(ctx, sample_bg, pixel_intensities, pixels, S, F, P, ptr_flags, st, &d, true))) return s;
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

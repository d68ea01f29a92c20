// CPU port of 3B's Gibbs sampler and of one pass of its main loop.
//
// TEST AND MEASUREMENT INFRASTRUCTURE ONLY: built into
// oracle/_build/libthreeb_oracle.so beside threeb_oracle.cpp (whose spot
// gradient it calls), used by tests/ and by bench.py's CPU baseline, never by
// the product library. It restates, in the reference's operation order:
//
//   MT19937::simple_seed / operator()   mt19937.h:47-63 with mersenne.cpp:46-61,
//                                       127-131: Matsumoto and Nishimura's
//                                       generator seeded by init_genrand, 37
//                                       words discarded, 32 bits times 2^-32
//   GibbsSampler2::next                 sampled_multispot.h:658-690 with the
//                                       masked remove_spot / add_spot (:114-130)
//   SpotWithBackgroundMasked            spot_with_background.hh:98-137
//   forward_algorithm_delta2            forward_algorithm.h:385-431
//   backward_sampling                   forward_algorithm.h:500-570
//   get_spot_pixels, getBall,           multispot5.cc:1001-1020, 1259-1290
//   dilate_mask
//   one pass of optimize_each_spot_in_turn_for_several_passes
//                                       multispot5.cc:1511-1690
//   sampled_background_spot_hessian_ffbs multispot5.cc:824-985 with
//                                       spot_shape_hess_position (storm.h:
//                                       87-146), SpotWithBackground over all
//                                       pixels and forward_algorithm_delta
//
// With the same seed its draws are the reference's draws, bit for bit
// (tests/test_gibbs_cpu.py checks that against the reference compiled on the
// host). The pass uses the oracle's spot gradient (threeb_oracle.cpp, OpenMP
// over the samples as the reference's threads are) and the library's
// restatement of ConjugateGradientOnly<5> (rfba_gb300/csrc/cg_only.h, pinned
// to the reference's optimiser bit for bit).
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <limits>
#include <random>
#include <set>
#include <tuple>
#include <vector>

#include "../rfba_gb300/csrc/cg_only.h"

extern "C" int oracle_3b_spot_neg_prob_diff(const double* sample_bg, const double* pix, const int* pixels, int S,
                                            int F, int P, const double* spot, double zFactor, double variance,
                                            const double* A, const double* pi, double mu_brightness,
                                            double sigma_brightness, double mu_blur, double sigma_blur, int nthreads,
                                            double* out, double* logp);

namespace {

struct RefRng {
    std::mt19937 g;
    explicit RefRng(int seed) : g((uint32_t)seed) { g.discard(37); }
    double operator()() { return (double)g() * (1. / (65536. * 65536.)); }
};

double ln_(double x) { return x == 0 ? -1e100 : std::log(x); }
double sq(double x) { return x * x; }

int select_random_element(const std::array<double, 3>& v, double scale, RefRng& rng) {
    double total = 0, choice = rng() * scale;
    for (int i = 0; i < 3; i++) {
        total += v[i];
        if (choice <= total) return i;
    }
    return 2;
}

int sample_unscaled_log(std::array<double, 3> a, RefRng& rng) {
    const double hi = *std::max_element(a.begin(), a.end());
    double sum = 0;
    for (int i = 0; i < 3; i++) {
        a[i] = std::exp(a[i] - hi);
        sum += a[i];
    }
    return select_random_element(a, sum, rng);
}

struct Sampler {
    const double* pix;  // [F][P]
    const double* si;   // [K][P]
    std::vector<std::vector<int> > masks;
    double A[9], pi[3];
    double variance;
    int sweeps, K, F, P;
    std::vector<unsigned char> state;  // [K][F]
    std::vector<double> cur;           // [F][P]
    std::vector<std::array<double, 3> > delta;

    void reset() {
        state.assign((size_t)K * F, 2);
        cur.assign((size_t)F * P, 0.0);
    }

    void update(int k, RefRng& rng) {
        const std::vector<int>& mask = masks[k];
        const double* v = si + (size_t)k * P;
        unsigned char* st = state.data() + (size_t)k * F;
        for (int f = 0; f < F; f++)  // remove_spot over the mask
            if (st[f] == 0)
                for (size_t p = 0; p < mask.size(); p++) cur[(size_t)f * P + mask[p]] -= v[mask[p]];
        // SpotWithBackgroundMasked
        const unsigned int n_pix = (unsigned int)mask.size();
        std::vector<std::pair<double, double> > lp((size_t)F);
        for (int f = 0; f < F; f++) {
            double log_prob_off = 0, log_prob_on = 0;
            const double* d = pix + (size_t)f * P;
            const double* c = cur.data() + (size_t)f * P;
            for (unsigned int p = 0; p < n_pix; p++) {
                const int m = mask[p];
                const double e = d[m] - (c[m] + v[m]);
                log_prob_off -= sq(d[m] - c[m]);
                log_prob_on -= sq(e);
            }
            log_prob_on = log_prob_on / (2 * variance) - n_pix * ::log(2 * M_PI * variance) / 2;
            log_prob_off = log_prob_off / (2 * variance) - n_pix * ::log(2 * M_PI * variance) / 2;
            lp[f] = std::make_pair(log_prob_on, log_prob_off);
        }
        auto B = [&](int s, int t) { return s == 0 ? lp[t].first : lp[t].second; };
        // forward_algorithm_delta2
        delta.resize((size_t)F);
        for (int i = 0; i < 3; i++) delta[0][i] = ln_(pi[i]) + B(i, 0);
        double lA[9];
        for (int i = 0; i < 9; i++) lA[i] = ln_(A[i]);
        for (int t = 1; t < F; t++)
            for (int j = 0; j < 3; j++) {
                double Ztj = -HUGE_VAL;
                for (int i = 0; i < 3; i++) Ztj = std::max(Ztj, delta[t - 1][i] + lA[i * 3 + j]);
                double sum = 0;
                for (int i = 0; i < 3; i++) sum += std::exp(delta[t - 1][i] + lA[i * 3 + j] - Ztj);
                delta[t][j] = B(j, t) + Ztj + ln_(sum);
            }
        // backward_sampling
        st[F - 1] = (unsigned char)sample_unscaled_log(delta[F - 1], rng);
        for (int i = F - 2; i >= 0; i--) {
            std::array<double, 3> r = delta[i];
            for (int j = 0; j < 3; j++) r[j] += lA[j * 3 + st[i + 1]];
            st[i] = (unsigned char)sample_unscaled_log(r, rng);
        }
        for (int f = 0; f < F; f++)  // add_spot over the mask
            if (st[f] == 0)
                for (size_t p = 0; p < mask.size(); p++) cur[(size_t)f * P + mask[p]] += v[mask[p]];
    }

    void next(RefRng& rng) {
        for (int j = 0; j < sweeps; j++)
            for (int k = 0; k < K; k++) update(k, rng);
    }
};

std::vector<std::array<int, 3> > ball(float radius) {
    std::vector<std::array<int, 3> > pts;
    const int r = (int)std::ceil(radius + 1);
    for (int z = -r; z <= r; z++)
        for (int y = -r; y <= r; y++)
            for (int x = -r; x <= r; x++)
                if ((float)((unsigned)(x * x) + (unsigned)(y * y) + (unsigned)(z * z)) <= radius * radius)
                    pts.push_back({x, y, z});
    return pts;
}

int round_away(double v) { return static_cast<int>(v > 0.0 ? v + 0.5 : v - 0.5); }

// get_spot_pixels; pixels sorted by (z, y, x)
std::vector<int> spot_pixels(const int* pixels, int P, const double* spot) {
    std::vector<int> out;
    const int o[3] = {round_away(spot[2]), round_away(spot[3]), round_away(spot[4])};
    for (const auto& b : ball((float)(spot[1] * 6 + 1))) {
        const int t[3] = {b[0] + o[0], b[1] + o[1], b[2] + o[2]};
        int lo = 0, hi = P;
        while (lo < hi) {
            const int mid = (lo + hi) / 2;
            const int* q = pixels + 3 * mid;
            if (q[2] < t[2] || (q[2] == t[2] && q[1] < t[1]) || (q[2] == t[2] && q[1] == t[1] && q[0] < t[0]))
                lo = mid + 1;
            else
                hi = mid;
        }
        if (lo < P && pixels[3 * lo] == t[0] && pixels[3 * lo + 1] == t[1] && pixels[3 * lo + 2] == t[2])
            out.push_back(lo);
    }
    return out;
}

double spot_shape(const int* x, const double* phi, double zf) {
    double d[3] = {x[0] - phi[2], x[1] - phi[3], x[2] - phi[4]};
    d[2] = d[2] / zf;
    const double s = -(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) / (2 * phi[1] * phi[1]);
    const double r_2_pi = std::sqrt(2 * M_PI);
    return std::exp(s) * phi[0] / (phi[1] * r_2_pi);
}

// spot_shape_hess_position (storm.h:87-146): value, gradient and Hessian
// (symmetric) of a spot at a pixel.
void spot_shape_hess(const int* x, const double* phi, double zf, double* val, double g[5], double H[5][5]) {
    const double d0 = x[0] - phi[2], d1 = x[1] - phi[3], d2 = x[2] - phi[4];
    const double d2s = d2 / zf;
    const double s = -(d0 * d0 + d1 * d1 + d2s * d2s) / (2 * phi[1] * phi[1]);
    const double r = std::sqrt(2 * M_PI), es = std::exp(s), p0 = phi[0], p1 = phi[1];
    *val = es * p0 / (p1 * r);
    const double c = es / (p1 * r);
    const double dv[3] = {d0, d1, d2};
    g[0] = c;
    g[1] = c * (-p0 * (1 + 2 * s) / p1);
    for (int a = 0; a < 3; ++a) g[2 + a] = c * (dv[a] * (p0 / sq(p1)));
    H[0][0] = 0;
    H[0][1] = H[1][0] = -es * (1 + 2 * s) / (p1 * p1 * r);
    H[1][1] = 2 * p0 * es * (1 + 5 * s + 2 * s * s) / (std::pow(p1, 3) * r);
    for (int a = 0; a < 3; ++a) {
        H[0][2 + a] = H[2 + a][0] = es * dv[a] / (std::pow(p1, 3) * r);
        H[1][2 + a] = H[2 + a][1] = -p0 * es * (3 + 2 * s) * dv[a] / (std::pow(p1, 4) * r);
        for (int b = a; b < 3; ++b)
            H[2 + a][2 + b] = H[2 + b][2 + a] =
                a == b ? p0 * es * (sq(dv[a]) - sq(p1)) / (r * std::pow(p1, 5))
                       : p0 * es * dv[a] * dv[b] / (r * std::pow(p1, 5));
    }
}

}  // namespace

extern "C" {

// sampled_background_spot_hessian_ffbs (multispot5.cc:824-985): the samples
// split over nthreads threads as the reference's threads take them (sample i
// on thread i % nthreads), each thread with its own MT19937 (simple_seed(seed
// + thread)). bg [S][F][P]; hess [25].
int port_spot_hessian(const double* bg, const double* pix, const int* pixels, int S, int F, int P, const double* spot,
                      double zFactor, double variance, const double* A, const double* pi, double mu_b,
                      double sigma_b, double mu_blur, double sigma_blur, int bs_iterations, int seed, int nthreads,
                      double* hess) {
    std::vector<double> val((size_t)P), g((size_t)P * 5), H((size_t)P * 25);
    for (int p = 0; p < P; ++p) {
        double h[5][5];
        spot_shape_hess(pixels + 3 * p, spot, zFactor, &val[p], &g[(size_t)p * 5], h);
        for (int a = 0; a < 5; ++a)
            for (int b = 0; b < 5; ++b) H[(size_t)p * 25 + a * 5 + b] = h[a][b];
    }
    if (nthreads < 1) nthreads = 1;
    if (nthreads > S) nthreads = S;
    std::vector<double> th_hess((size_t)nthreads * 25, 0.0), th_deriv((size_t)nthreads * 5, 0.0);
    double lA[9];
    for (int i = 0; i < 9; i++) lA[i] = ln_(A[i]);
#pragma omp parallel for num_threads(nthreads) schedule(static, 1)
    for (int t = 0; t < nthreads; ++t) {
        RefRng rng(seed + t);
        std::vector<double> part((size_t)F * 30);  // per frame: Hessian [25], derivative [5]
        std::vector<std::array<double, 3> > delta((size_t)F);
        std::vector<unsigned char> st((size_t)F);
        double* sh = th_hess.data() + (size_t)t * 25;
        double* sd = th_deriv.data() + (size_t)t * 5;
        for (int i = t; i < S; i += nthreads) {
            const double* b = bg + (size_t)i * F * P;
            std::vector<std::pair<double, double> > lp((size_t)F);
            for (int f = 0; f < F; ++f) {
                double* hp = part.data() + (size_t)f * 30;
                std::fill(hp, hp + 30, 0.0);
                double log_prob_off = 0, log_prob_on = 0;
                for (int p = 0; p < P; ++p) {
                    const double d = pix[(size_t)f * P + p], c = b[(size_t)f * P + p];
                    const double e = d - (c + val[p]);
                    log_prob_off -= sq(d - c);
                    log_prob_on -= sq(e);
                    const double* gp = &g[(size_t)p * 5];
                    const double* Hp = &H[(size_t)p * 25];
                    for (int a = 0; a < 5; ++a)
                        for (int c2 = 0; c2 < 5; ++c2) hp[a * 5 + c2] += e * Hp[a * 5 + c2] - gp[a] * gp[c2];
                    for (int a = 0; a < 5; ++a) hp[25 + a] += e * gp[a];
                }
                lp[f] = std::make_pair(log_prob_on / (2 * variance) - P * ::log(2 * M_PI * variance) / 2,
                                       log_prob_off / (2 * variance) - P * ::log(2 * M_PI * variance) / 2);
            }
            auto B = [&](int s2, int f) { return s2 == 0 ? lp[f].first : lp[f].second; };
            for (int k = 0; k < 3; k++) delta[0][k] = ln_(pi[k]) + B(k, 0);
            for (int f = 1; f < F; f++)
                for (int j = 0; j < 3; j++) {
                    double Z = -HUGE_VAL;
                    for (int k = 0; k < 3; k++) Z = std::max(Z, delta[f - 1][k] + lA[k * 3 + j]);
                    double sum = 0;
                    for (int k = 0; k < 3; k++) sum += std::exp(delta[f - 1][k] + lA[k * 3 + j] - Z);
                    delta[f][j] = B(j, f) + Z + ln_(sum);
                }
            for (int it = 0; it < bs_iterations; ++it) {
                st[F - 1] = (unsigned char)sample_unscaled_log(delta[F - 1], rng);
                for (int f = F - 2; f >= 0; f--) {
                    std::array<double, 3> r = delta[f];
                    for (int j = 0; j < 3; j++) r[j] += lA[j * 3 + st[f + 1]];
                    st[f] = (unsigned char)sample_unscaled_log(r, rng);
                }
                double h[25] = {0}, d[5] = {0};
                for (int f = 0; f < F; ++f)
                    if (st[f] == 0) {
                        const double* hp = part.data() + (size_t)f * 30;
                        for (int a = 0; a < 25; ++a) h[a] += hp[a];
                        for (int a = 0; a < 5; ++a) d[a] += hp[25 + a];
                    }
                for (int a = 0; a < 5; ++a)
                    for (int c2 = 0; c2 < 5; ++c2) sh[a * 5 + c2] += h[a * 5 + c2] + d[a] * d[c2];
                for (int a = 0; a < 5; ++a) sd[a] += d[a];
            }
        }
    }
    double sum_hess[25] = {0}, sum_deriv[5] = {0};
    for (int t = 0; t < nthreads; ++t) {
        for (int a = 0; a < 25; ++a) sum_hess[a] += th_hess[(size_t)t * 25 + a];
        for (int a = 0; a < 5; ++a) sum_deriv[a] += th_deriv[(size_t)t * 5 + a];
    }
    const double norm = (double)bs_iterations * S * variance;
    for (int a = 0; a < 25; ++a) sum_hess[a] /= norm;
    for (int a = 0; a < 5; ++a) sum_deriv[a] /= norm;
    for (int a = 0; a < 5; ++a)
        for (int c2 = 0; c2 < 5; ++c2) hess[a * 5 + c2] = sum_hess[a * 5 + c2] - sum_deriv[a] * sum_deriv[c2];
    hess[0] += (1 + (ln_(spot[0]) - mu_b - 1) / sq(sigma_b)) / sq(spot[0]);
    hess[6] += (1 + (ln_(spot[1]) - mu_blur - 1) / sq(sigma_blur)) / sq(spot[1]);
    return 0;
}

// GibbsSampler2: n_draws calls of next() from all spots off, MT19937 seeded by
// simple_seed(seed). si [K][P] spot intensities, masks as offsets / indices.
int port_gibbs_run(const double* pix, const double* si, const int* moff, const int* midx, int K, int F, int P,
                   const double* A, const double* pi, double variance, int sweeps, int n_draws, int seed,
                   unsigned char* states, double* intensities) {
    Sampler s;
    s.pix = pix;
    s.si = si;
    s.masks.resize((size_t)K);
    for (int k = 0; k < K; ++k) s.masks[k].assign(midx + moff[k], midx + moff[k + 1]);
    for (int i = 0; i < 9; ++i) s.A[i] = A[i];
    for (int i = 0; i < 3; ++i) s.pi[i] = pi[i];
    s.variance = variance;
    s.sweeps = sweeps;
    s.K = K;
    s.F = F;
    s.P = P;
    s.reset();
    RefRng rng(seed);
    for (int d = 0; d < n_draws; ++d) {
        s.next(rng);
        std::copy(s.state.begin(), s.state.end(), states + (size_t)d * K * F);
        if (intensities) std::copy(s.cur.begin(), s.cur.end(), intensities + (size_t)d * F * P);
    }
    return 0;
}

// One pass of optimize_each_spot_in_turn_for_several_passes (multispot5.cc:
// 1511-1690) with one MT19937 for the pass. spots [*nspots][5] in place.
// max_spots >= 0 optimises only the first max_spots spots of the pass's order
// (a bounded timing sample); seconds[0..1] receive the time in the sampler and
// in the optimiser.
int port_optimise_pass(const double* pix, const int* pixels, int F, int P, double* spots, int* nspots, int pass,
                       int main_samples, int sweeps, int cg_max_iterations, const double* limit,
                       double position_extra_radius, const double* A, const double* pi, double variance,
                       double zFactor, double mu_b, double sigma_b, double mu_blur, double sigma_blur, int seed,
                       int nthreads, int max_spots, double* seconds) {
    using clk = std::chrono::steady_clock;
    int K = *nspots;
    std::vector<std::array<double, 5> > sp((size_t)K);
    for (int k = 0; k < K; ++k)
        for (int n = 0; n < 5; ++n) sp[k][n] = spots[5 * k + n];
    std::vector<std::vector<int> > masks((size_t)K);
    for (int k = 0; k < K; ++k) masks[k] = spot_pixels(pixels, P, sp[k].data());
    std::set<std::tuple<int, int, int> > allowed;
    const bool use_prior = position_extra_radius >= 0;
    if (use_prior) {
        const auto b = ball((float)position_extra_radius);
        for (int p = 0; p < P; ++p)
            for (const auto& o : b)
                allowed.insert(std::make_tuple(pixels[3 * p] + o[0], pixels[3 * p + 1] + o[1], pixels[3 * p + 2] + o[2]));
    }
    std::vector<int> order((size_t)K);
    for (int k = 0; k < K; ++k) order[k] = k;
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
        sp.swap(t);  // masks stay in place (multispot5.cc:1570)
    }
    RefRng rng(seed);
    double t_gibbs = 0, t_cg = 0;
    const int limit_k = max_spots >= 0 ? std::min(max_spots, K) : K;
    for (int k = 0; k < K && k < limit_k; ++k) {
        const auto t0 = clk::now();
        std::vector<double> si((size_t)K * P);
        for (int j = 0; j < K; ++j)
            for (int p = 0; p < P; ++p) si[(size_t)j * P + p] = spot_shape(pixels + 3 * p, sp[j].data(), zFactor);
        Sampler s;
        s.pix = pix;
        s.si = si.data();
        s.masks = masks;
        for (int i = 0; i < 9; ++i) s.A[i] = A[i];
        for (int i = 0; i < 3; ++i) s.pi[i] = pi[i];
        s.variance = variance;
        s.sweeps = sweeps;
        s.K = K;
        s.F = F;
        s.P = P;
        s.reset();
        std::vector<double> bg((size_t)main_samples * F * P);
        for (int d = 0; d < main_samples; ++d) {
            s.next(rng);
            double* o = bg.data() + (size_t)d * F * P;
            std::copy(s.cur.begin(), s.cur.end(), o);
            const unsigned char* stk = s.state.data() + (size_t)k * F;
            for (int f = 0; f < F; ++f)  // remove_spot over all pixels
                if (stk[f] == 0)
                    for (int p = 0; p < P; ++p) o[(size_t)f * P + p] -= si[(size_t)k * P + p];
        }
        const auto t1 = clk::now();
        auto grad = [&](const double* x, double* g) -> int {
            if (x[0] <= 0 || x[1] <= 0) {
                for (int n = 0; n < 5; ++n) g[n] = std::numeric_limits<double>::quiet_NaN();
                return 0;
            }
            return oracle_3b_spot_neg_prob_diff(bg.data(), pix, pixels, main_samples, F, P, x, zFactor, variance, A, pi,
                                                mu_b, sigma_b, mu_blur, sigma_blur, nthreads, g, nullptr);
        };
        rfba::CgOnly5 cg;
        if (cg.start(sp[k].data(), limit, grad)) return -1;
        cg.max_iterations = cg_max_iterations;
        if (cg.run(grad)) return -1;
        for (int n = 0; n < 5; ++n) sp[k][n] = cg.x[n];
        masks[k] = spot_pixels(pixels, P, sp[k].data());
        const bool zero_prior =
            use_prior &&
            !allowed.count(std::make_tuple(round_away(sp[k][2]), round_away(sp[k][3]), round_away(sp[k][4])));
        const auto t2 = clk::now();
        t_gibbs += std::chrono::duration<double>(t1 - t0).count();
        t_cg += std::chrono::duration<double>(t2 - t1).count();
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
    if (seconds) {
        seconds[0] = t_gibbs;
        seconds[1] = t_cg;
    }
    return 0;
}

}  // extern "C"

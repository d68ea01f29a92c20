// CPU oracle (FP64) of the 3B spot-gradient evaluation — TEST INFRASTRUCTURE
// ONLY: used by tests/ and by bench.py's CPU-baseline leg, never by the product.
//
// A restatement, in the reference's operation order, of the derivative of the
// negative log probability of one spot given sampled backgrounds, which 3B's
// conjugate-gradient spot optimiser evaluates (RFBA Main):
//   SpotNegProbabilityDiffWithSampledBackground::operator()  multispot5.cc:616-664
//   compute_spot_intensity_derivatives                      sampled_multispot.h:195-202
//   spot_shape_s / spot_shape_diff_position                 storm.h:51-84
//   SpotWithBackground (emission log probabilities)         spot_with_background.hh:55-135
//   forward_algorithm_hessian (derivative part), ln         forward_algorithm.h:34-40, 157-259
//   diff_log_log_normal                                     storm.h:431-434
// The reference splits the samples over threads (thread k sums samples k,
// k + nthreads, ...; the partial sums are then added in thread order,
// multispot5.cc:625-655); `nthreads` reproduces that summation order.
// Pinned bit for bit to the reference's own headers compiled on the host
// (oracle/refshim/ref3b_harness.cpp, tests/test_threeb_cpu.py).
#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

namespace {

constexpr int kM = 5;  // spot parameters: brightness, blur, x, y, z

// forward_algorithm.h:34-40
inline double ln(double x) { return x == 0 ? -1e100 : std::log(x); }
inline double sq(double x) { return x * x; }

// storm.h:51-84: spot shape at voxel x and its derivative with respect to the
// parameters phi = (brightness, blur, x, y, z)
void spot_shape_diff_position(const double x[3], const double phi[5], double zf, double* prob, double deriv[5]) {
    double d0 = x[0] - phi[2], d1 = x[1] - phi[3], d2 = x[2] - phi[4];
    d2 = d2 / zf;
    double n2 = 0;
    n2 += d0 * d0;
    n2 += d1 * d1;
    n2 += d2 * d2;
    const double s = -n2 / (2 * phi[1] * phi[1]);
    const double r_2_pi = std::sqrt(2 * M_PI);
    *prob = std::exp(s) * phi[0] / (phi[1] * r_2_pi);
    const double k = std::exp(s) / (phi[1] * r_2_pi);
    const double v[5] = {1, -phi[0] * (1 + 2 * s) / phi[1], (x[0] - phi[2]) * (phi[0] / sq(phi[1])),
                         (x[1] - phi[3]) * (phi[0] / sq(phi[1])), (x[2] - phi[4]) * (phi[0] / sq(phi[1]))};
    for (int i = 0; i < 5; ++i) deriv[i] = k * v[i];
}

// storm.h:431-434
inline double diff_log_log_normal(double x, double mu, double sigma) { return -(1 + (ln(x) - mu) / sq(sigma)) / x; }

// One sample: emission log probabilities of every frame
// (spot_with_background.hh:98-133) and the forward algorithm's derivative
// (forward_algorithm.h:157-259 with compute_hessian = 0). States: 0 spot on
// (log_prob.first, diff), 1 off, 2 bleached (log_prob.second, no diff).
void sample_gradient(const double* bg, const double* pix, int F, int P, const std::vector<double>& val,
                     const std::vector<double>& der, double variance, const double A[9], const double pi[3],
                     double grad[5], double* logp) {
    std::vector<double> lon(F), loff(F), dif((size_t)F * kM);
    for (int f = 0; f < F; ++f) {
        double log_prob_off = 0, log_prob_on = 0;
        double diff[kM] = {0, 0, 0, 0, 0};
        const double* I = pix + (size_t)f * P;
        const double* G = bg + (size_t)f * P;
        for (int p = 0; p < P; ++p) {
            const double e = I[p] - (G[p] + val[p]);
            log_prob_off -= sq(I[p] - G[p]);
            log_prob_on -= sq(e);
            for (int i = 0; i < kM; ++i) diff[i] += der[(size_t)p * kM + i] * e;
        }
        const unsigned int n_pix = (unsigned int)P;
        log_prob_on = log_prob_on / (2 * variance) - n_pix * ::log(2 * M_PI * variance) / 2;
        log_prob_off = log_prob_off / (2 * variance) - n_pix * ::log(2 * M_PI * variance) / 2;
        for (int i = 0; i < kM; ++i) diff[i] /= variance;
        lon[f] = log_prob_on;
        loff[f] = log_prob_off;
        for (int i = 0; i < kM; ++i) dif[(size_t)f * kM + i] = diff[i];
    }
    auto blog = [&](int j, int f) { return j == 0 ? lon[f] : loff[f]; };
    double delta[3], ndelta[3], dd[3][kM], ndd[3][kM];
    for (int i = 0; i < 3; ++i) {
        delta[i] = ln(pi[i]) + blog(i, 0);
        for (int n = 0; n < kM; ++n) dd[i][n] = i == 0 ? dif[n] : 0.0;
    }
    for (int t = 1; t < F; ++t) {
        for (int j = 0; j < 3; ++j) {
            double Ztj = -HUGE_VAL;
            for (int i = 0; i < 3; ++i) Ztj = std::max(Ztj, delta[i] + ln(A[i * 3 + j]));
            double sum = 0;
            for (int i = 0; i < 3; ++i) sum += std::exp(delta[i] + ln(A[i * 3 + j]) - Ztj);
            ndelta[j] = blog(j, t) + Ztj + ln(sum);
            double top[kM] = {0, 0, 0, 0, 0};
            for (int i = 0; i < 3; ++i) {
                const double w = std::exp(delta[i] + ln(A[i * 3 + j]) - Ztj);
                for (int n = 0; n < kM; ++n) top[n] += dd[i][n] * w;
            }
            for (int n = 0; n < kM; ++n) ndd[j][n] = (j == 0 ? dif[(size_t)t * kM + n] : 0.0) + top[n] / sum;
        }
        for (int j = 0; j < 3; ++j) {
            delta[j] = ndelta[j];
            for (int n = 0; n < kM; ++n) dd[j][n] = ndd[j][n];
        }
    }
    double Z = -HUGE_VAL;
    for (int i = 0; i < 3; ++i) Z = std::max(Z, delta[i]);
    double sum = 0;
    for (int i = 0; i < 3; ++i) sum += std::exp(delta[i] - Z);
    const double log_prob = Z + ln(sum);
    for (int n = 0; n < kM; ++n) grad[n] = 0;
    for (int i = 0; i < 3; ++i) {
        const double w = std::exp(delta[i] - log_prob);
        for (int n = 0; n < kM; ++n) grad[n] += w * dd[i][n];
    }
    *logp = log_prob;
}

}  // namespace

extern "C" {

// multispot5.cc:616-664. sample_bg [S][F][P], pix [F][P], pixels [P][3] (x, y,
// z), spot (brightness, blur, x, y, z), A row-major 3 x 3, out[5]; logp[S]
// (may be null) receives each sample's log probability.
int oracle_3b_spot_neg_prob_diff(const double* sample_bg, const double* pix, const int* pixels, int S, int F, int P,
                                 const double* spot, double zFactor, double variance, const double* A,
                                 const double* pi, double mu_brightness, double sigma_brightness, double mu_blur,
                                 double sigma_blur, int nthreads, double* out, double* logp) {
    if (S < 1 || F < 1 || P < 1 || nthreads < 1) return -1;
    if (spot[0] <= 0 || spot[1] <= 0) {
        for (int i = 0; i < kM; ++i) out[i] = 1 * std::numeric_limits<double>::quiet_NaN();
        return 0;
    }
    std::vector<double> val(P), der((size_t)P * kM);
    for (int p = 0; p < P; ++p) {
        const double x[3] = {(double)pixels[3 * p], (double)pixels[3 * p + 1], (double)pixels[3 * p + 2]};
        spot_shape_diff_position(x, spot, zFactor, &val[p], &der[(size_t)p * kM]);
    }
    const int nt = std::min(S, nthreads);
    std::vector<double> res((size_t)nt * kM, 0.0);
#pragma omp parallel for schedule(static, 1)
    for (int k = 0; k < nt; ++k) {
        for (int s = k; s < S; s += nt) {
            double g[kM], lp;
            sample_gradient(sample_bg + (size_t)s * F * P, pix, F, P, val, der, variance, A, pi, g, &lp);
            for (int n = 0; n < kM; ++n) res[(size_t)k * kM + n] += g[n];
            if (logp) logp[s] = lp;
        }
    }
    double sum_diff_log[kM] = {0, 0, 0, 0, 0};
    for (int k = 0; k < nt; ++k)
        for (int n = 0; n < kM; ++n) sum_diff_log[n] += res[(size_t)k * kM + n];
    double diff_log[kM];
    for (int n = 0; n < kM; ++n) diff_log[n] = sum_diff_log[n] / (double)S;
    const double prior[kM] = {diff_log_log_normal(spot[0], mu_brightness, sigma_brightness),
                              diff_log_log_normal(spot[1], mu_blur, sigma_blur), 0, 0, 0};
    for (int n = 0; n < kM; ++n) out[n] = -(diff_log[n] + prior[n]);
    return 0;
}

}  // extern "C"

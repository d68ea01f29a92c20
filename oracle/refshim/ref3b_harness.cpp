// Host harness around the reference's own 3B headers (built by
// oracle/build_ref.sh from the reference tree; never committed as a binary).
// It runs the reference's spot_shape_diff_position (storm.h:64-84),
// SpotWithBackground (spot_with_background.hh) and forward_algorithm_deriv
// (forward_algorithm.h:325-331) exactly as compiled from their sources. Only
// the composition of SpotNegProbabilityDiffWithSampledBackground::operator()
// (multispot5.cc:616-664, in a file that cannot be compiled on its own) and of
// compute_spot_intensity_derivatives (sampled_multispot.h:195-202) is written
// out here, with the reference's per-thread partial sums done in sequence, and
// the spot optimisation loop of multispot5.cc:1624-1636 around the reference's
// own ConjugateGradientOnly<5> (conjugate_gradient_only.h).
// The three std::tr1 names the headers use are aliases of their std
// counterparts, so the reference's `using namespace std; using namespace
// std::tr1;` resolves without ambiguity in C++11.
#include <array>
#include <cmath>
#include <cstdio>
#include <limits>
#include <tuple>
#include <utility>
#include <vector>
namespace std {
namespace tr1 {
using std::array;
using std::get;
using std::ignore;
using std::make_tuple;
using std::tie;
using std::tuple;
}  // namespace tr1
}  // namespace std
#include <TooN/TooN.h>
using namespace TooN;
using namespace std;
#include "debug.h"
#include "utility.h"
#include "forward_algorithm.h"
#include "storm.h"
#define SWBG_NAME SpotWithBackground
#include "spot_with_background.hh"

extern "C" int ref3b_spot_neg_prob_diff(const double* sample_bg, const double* pix, const int* pixels, int S, int F,
                                        int P, const double* spot_in, double zFactor, double variance,
                                        const double* A_in, const double* pi_in, double mu_brightness,
                                        double sigma_brightness, double mu_blur, double sigma_blur, int nthreads,
                                        double* out) {
    Vector<5> spot = makeVector(spot_in[0], spot_in[1], spot_in[2], spot_in[3], spot_in[4]);
    if (spot[0] <= 0 || spot[1] <= 0) {
        Vector<5> r = Ones * std::numeric_limits<double>::quiet_NaN();
        for (int i = 0; i < 5; ++i) out[i] = r[i];
        return 0;
    }
    Matrix<3> A;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) A[i][j] = A_in[i * 3 + j];
    Vector<3> pi = makeVector(pi_in[0], pi_in[1], pi_in[2]);
    vector<vector<vector<double> > > samples(S, vector<vector<double> >(F, vector<double>(P)));
    vector<vector<double> > pixel_intensities(F, vector<double>(P));
    for (int s = 0; s < S; ++s)
        for (int f = 0; f < F; ++f)
            for (int p = 0; p < P; ++p) samples[s][f][p] = sample_bg[((size_t)s * F + f) * P + p];
    for (int f = 0; f < F; ++f)
        for (int p = 0; p < P; ++p) pixel_intensities[f][p] = pix[(size_t)f * P + p];
    // compute_spot_intensity_derivatives
    vector<pair<double, Vector<5> > > spot_intensities(P);
    for (int p = 0; p < P; ++p) {
        Vector<3> x;
        x[0] = pixels[3 * p];
        x[1] = pixels[3 * p + 1];
        x[2] = pixels[3 * p + 2];
        spot_intensities[p] = spot_shape_diff_position(x, spot, zFactor);
    }
    vector<int> O(F);
    for (int f = 0; f < F; ++f) O[f] = f;
    int thread_num = S;
    if (thread_num > nthreads) thread_num = nthreads;
    Vector<5> sum_diff_log = Zeros;
    for (int k = 0; k < thread_num; ++k) {
        Vector<5> res = Zeros;
        for (int i = k; i < S; i = i + thread_num) {
            SpotWithBackground B(samples[i], spot_intensities, pixel_intensities, variance);
            pair<double, Vector<5> > r = forward_algorithm_deriv(A, pi, B, O);
            res += r.second;
        }
        sum_diff_log += res;
    }
    Vector<5> diff_log = sum_diff_log / samples.size();
    Vector<5> logprior_deriv = makeVector(diff_log_log_normal(spot[0], mu_brightness, sigma_brightness),
                                          diff_log_log_normal(spot[1], mu_blur, sigma_blur), 0, 0, 0);
    Vector<5> r = -(diff_log + logprior_deriv);
    for (int i = 0; i < 5; ++i) out[i] = r[i];
    return 0;
}

// The reference's own ConjugateGradientOnly<5> (conjugate_gradient_only.h),
// driven as multispot5.cc:1624-1636 drives it, with the gradient above.
#include "conjugate_gradient_only.h"

namespace {
struct RefSpotDeriv {
    const double *sample_bg, *pix;
    const int* pixels;
    int S, F, P;
    double zFactor, variance;
    const double *A, *pi;
    double mu_b, sigma_b, mu_r, sigma_r;
    int nthreads;
    Vector<5> operator()(const Vector<5>& x) const {
        double s[5], out[5];
        for (int i = 0; i < 5; ++i) s[i] = x[i];
        ref3b_spot_neg_prob_diff(sample_bg, pix, pixels, S, F, P, s, zFactor, variance, A, pi, mu_b, sigma_b, mu_r,
                                 sigma_r, nthreads, out);
        return makeVector(out[0], out[1], out[2], out[3], out[4]);
    }
};
}  // namespace

extern "C" int ref3b_cg_optimise(const double* sample_bg, const double* pix, const int* pixels, int S, int F, int P,
                                 const double* spot_in, double zFactor, double variance, const double* A_in,
                                 const double* pi_in, double mu_brightness, double sigma_brightness, double mu_blur,
                                 double sigma_blur, int nthreads, const double* limit_in, int max_iterations,
                                 double* x_out, int* iterations) {
    RefSpotDeriv d{sample_bg, pix, pixels, S, F, P, zFactor, variance, A_in, pi_in,
                   mu_brightness, sigma_brightness, mu_blur, sigma_blur, nthreads};
    Vector<5> start = makeVector(spot_in[0], spot_in[1], spot_in[2], spot_in[3], spot_in[4]);
    Vector<5> limit = makeVector(limit_in[0], limit_in[1], limit_in[2], limit_in[3], limit_in[4]);
    ConjugateGradientOnly<5> cg(start, d, limit);
    cg.max_iterations = max_iterations;
    while (cg.iterate(d)) {
    }
    for (int i = 0; i < 5; ++i) x_out[i] = cg.x[i];
    *iterations = cg.iterations;
    return 0;
}

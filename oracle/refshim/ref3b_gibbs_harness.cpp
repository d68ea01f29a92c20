// Host harness around the reference's own 3B Gibbs sampler (built by
// oracle/build_ref.sh from the reference tree with its mersenne.cpp; never
// committed as a binary). What runs is the reference's code as compiled from
// its headers: GibbsSampler2 (sampled_multispot.h:360-690) with its masked
// add_spot / remove_spot, SpotWithBackgroundMasked (spot_with_background.hh),
// forward_algorithm_delta2 and forward_backward_algorithm
// (forward_algorithm.h:385-484), backward_sampling, MT19937 and
// compute_spot_intensity. Written out here, because it lives in a file that
// cannot be compiled on its own, is the body of
// NegativeFreeEnergy::compute_with_mask (multispot5.cc:335-405) around that
// sampler; and ref_gibbs_trace replays one sweep with given drawn states to
// expose the quantities each draw was made from.
// sampled_multispot.h's image3d.h declares Ref3D's members with a redundant
// class qualification, so this unit compiles with -fpermissive.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
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
int MAXTHREAD = 1;
#include "debug.h"
#include "utility.h"
#include "forward_algorithm.h"
#include "storm.h"
#include "sampled_multispot.h"

namespace {

vector<vector<double> > frames_of(const double* a, int F, int P) {
    vector<vector<double> > v(F, vector<double>(P));
    for (int f = 0; f < F; ++f)
        for (int p = 0; p < P; ++p) v[f][p] = a[(size_t)f * P + p];
    return v;
}

vector<vector<int> > masks_of(const int* moff, const int* midx, int K) {
    vector<vector<int> > m(K);
    for (int k = 0; k < K; ++k) m[k].assign(midx + moff[k], midx + moff[k + 1]);
    return m;
}

vector<Ref3D> refs_of(const int* pixels, int P) {
    vector<Ref3D> r(P);
    for (int p = 0; p < P; ++p) r[p] = Ref3D(pixels[3 * p], pixels[3 * p + 1], pixels[3 * p + 2]);
    return r;
}

Matrix<3> A_of(const double* a) {
    Matrix<3> A;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) A[i][j] = a[i * 3 + j];
    return A;
}

}  // namespace

extern "C" {

// compute_spot_intensity (sampled_multispot.h:182-191) for K spots: out [K][P].
int ref_spot_intensity(const int* pixels, int P, const double* spots, int K, double zFactor, double* out) {
    const vector<Ref3D> px = refs_of(pixels, P);
    for (int k = 0; k < K; ++k) {
        const double* s = spots + 5 * (size_t)k;
        const vector<double> v = SampledMultispot::compute_spot_intensity(px, makeVector(s[0], s[1], s[2], s[3], s[4]),
                                                                          zFactor);
        std::copy(v.begin(), v.end(), out + (size_t)k * P);
    }
    return 0;
}

// One sweep from all spots off with the states `states` [K][F] the sweep
// drew: for each spot, SpotWithBackgroundMasked over its mask (lp [K][F][2]:
// on, off), the forward filter normalised (filt [K][F][3]) and the
// forward-backward posterior (post [K][F][3]); then the spot is added back
// with its drawn states, as GibbsSampler2::next does.
int ref_gibbs_trace(const double* pix, const double* si, const int* moff, const int* midx, int K, int F, int P,
                    const double* A_in, const double* pi_in, double variance, const unsigned char* states, double* lp,
                    double* filt, double* post) {
    const vector<vector<double> > pixel_intensities = frames_of(pix, F, P);
    const vector<vector<double> > spot_intensities = frames_of(si, K, P);
    const vector<vector<int> > masks = masks_of(moff, midx, K);
    const Matrix<3> A = A_of(A_in);
    const Vector<3> pi = makeVector(pi_in[0], pi_in[1], pi_in[2]);
    vector<vector<double> > cur(F, vector<double>(P, 0.0));
    const vector<int> O = SampledMultispot::sequence(F);
    for (int k = 0; k < K; ++k) {
        SampledMultispot::SpotWithBackgroundMasked B3(cur, spot_intensities[k], pixel_intensities, variance, masks[k]);
        std::vector<array<double, 3> > delta;
        forward_algorithm_delta2<3>(A, pi, B3, O, delta);
        const auto fb = forward_backward_algorithm<3>(A, pi, B3, O);
        for (int f = 0; f < F; ++f) {
            lp[((size_t)k * F + f) * 2] = B3.log(0, f);
            lp[((size_t)k * F + f) * 2 + 1] = B3.log(1, f);
            double hi = -HUGE_VAL, tot = 0;
            for (int j = 0; j < 3; ++j) hi = std::max(hi, delta[f][j]);
            for (int j = 0; j < 3; ++j) tot += exp(delta[f][j] - hi);
            for (int j = 0; j < 3; ++j) filt[((size_t)k * F + f) * 3 + j] = exp(delta[f][j] - hi) / tot;
            double a[3];
            hi = -HUGE_VAL;
            tot = 0;
            for (int j = 0; j < 3; ++j) {
                a[j] = fb.first[f][j] + fb.second[f][j];
                hi = std::max(hi, a[j]);
            }
            for (int j = 0; j < 3; ++j) tot += exp(a[j] - hi);
            for (int j = 0; j < 3; ++j) post[((size_t)k * F + f) * 3 + j] = exp(a[j] - hi) / tot;
        }
        vector<State> st(F);
        for (int f = 0; f < F; ++f) st[f] = (State)states[(size_t)k * F + f];
        SampledMultispot::add_spot(cur, spot_intensities[k], st, masks[k]);
    }
    return 0;
}

// GibbsSampler2 with MT19937 seeded by simple_seed(seed): n_draws calls of
// next(); states [n][K][F], intensities [n][F][P] (may be NULL).
int ref_gibbs_run(const double* pix, const double* si, const int* moff, const int* midx, int K, int F, int P,
                  const double* A_in, const double* pi_in, double variance, int sweeps, int n_draws, int seed,
                  unsigned char* states, double* intensities) {
    const vector<vector<double> > pixel_intensities = frames_of(pix, F, P);
    const vector<vector<double> > spot_intensities = frames_of(si, K, P);
    const vector<vector<int> > masks = masks_of(moff, midx, K);
    vector<Vector<5> > spots(K, Zeros);  // only their count is used by the sampler
    GibbsSampler2 sampler(pixel_intensities, spot_intensities, spots, masks, A_of(A_in),
                          makeVector(pi_in[0], pi_in[1], pi_in[2]), variance, sweeps);
    MT19937 rng;
    rng.simple_seed(seed);
    for (int d = 0; d < n_draws; ++d) {
        sampler.next(rng);
        for (int k = 0; k < K; ++k)
            for (int f = 0; f < F; ++f) states[((size_t)d * K + k) * F + f] = (unsigned char)sampler.sample()[k][f];
        if (intensities)
            for (int f = 0; f < F; ++f)
                for (int p = 0; p < P; ++p)
                    intensities[((size_t)d * F + f) * P + p] = sampler.sample_intensities()[f][p];
    }
    return 0;
}

// sampled_background_spot_hessian_ffbs (multispot5.cc:824-985) for one thread
// (MAXTHREAD = 1: one MT19937, simple_seed(seed), draws every backward sample):
// the reference's compute_spot_intensity_hessian, compute_spot_intensity,
// SpotWithBackground over all pixels, forward_algorithm_delta and
// backward_sampling, the per-frame parts and sums written out as hess_handler
// has them. bg [S][F][P]; hess [25] row-major. The reference never writes
// entry [4][3] of its per-pixel Hessian (storm.h:143), so hess[4 * 5 + 3] is
// indeterminate; the upper triangle is what is defined.
int ref_spot_hessian(const double* bg, const double* pix, const int* pixels, int S, int F, int P, const double* spot,
                     const double* A_in, const double* pi_in, double variance, double zFactor, double mu_brightness,
                     double sigma_brightness, double mu_blur, double sigma_blur, int bs_iterations, int seed,
                     double* hess) {
    const vector<vector<double> > pixel_intensities = frames_of(pix, F, P);
    const vector<Ref3D> px = refs_of(pixels, P);
    const Vector<5> sp = makeVector(spot[0], spot[1], spot[2], spot[3], spot[4]);
    const vector<tuple<double, Vector<5>, Matrix<5> > > spot_hess_etc =
        SampledMultispot::compute_spot_intensity_hessian(px, sp, zFactor);
    const vector<double> spot_intensities = SampledMultispot::compute_spot_intensity(px, sp, zFactor);
    const Matrix<3> A = A_of(A_in);
    const Vector<3> pi = makeVector(pi_in[0], pi_in[1], pi_in[2]);
    const vector<int> O = SampledMultispot::sequence(F);
    MT19937 rng;
    rng.simple_seed(seed);
    Matrix<5> sum_hess = Zeros;
    Vector<5> sum_deriv = Zeros;
    vector<pair<Matrix<5>, Vector<5> > > hess_and_deriv_part(F);
    for (int i = 0; i < S; i++) {
        const vector<vector<double> > bgi = frames_of(bg + (size_t)i * F * P, F, P);
        SpotWithBackground B(bgi, spot_intensities, pixel_intensities, variance);
        for (int frame = 0; frame < F; frame++) {
            Matrix<5> h = Zeros;
            Vector<5> d = Zeros;
            for (int pixel = 0; pixel < P; pixel++) {
                double e = pixel_intensities[frame][pixel] - (bgi[frame][pixel] + spot_intensities[pixel]);
                h += e * get<2>(spot_hess_etc[pixel]) -
                     get<1>(spot_hess_etc[pixel]).as_col() * get<1>(spot_hess_etc[pixel]).as_row();
                d += e * get<1>(spot_hess_etc[pixel]);
            }
            hess_and_deriv_part[frame] = make_pair(h, d);
        }
        std::vector<array<double, 3> > delta = forward_algorithm_delta(A, pi, B, O);
        for (int b = 0; b < bs_iterations; b++) {
            vector<State> current_sample = backward_sampling<3, State>(A, delta, rng);
            Matrix<5> h = Zeros;
            Vector<5> d = Zeros;
            for (int frame = 0; frame < F; frame++)
                if (current_sample[frame] == 0) {
                    h += hess_and_deriv_part[frame].first;
                    d += hess_and_deriv_part[frame].second;
                }
            sum_hess += h + d.as_col() * d.as_row();
            sum_deriv += d;
        }
    }
    sum_hess /= (bs_iterations * S * variance);
    sum_deriv /= (bs_iterations * S * variance);
    sum_hess -= sum_deriv.as_col() * sum_deriv.as_row();
    sum_hess[0][0] += hess_log_log_normal(sp[0], mu_brightness, sigma_brightness);
    sum_hess[1][1] += hess_log_log_normal(sp[1], mu_blur, sigma_blur);
    for (int r = 0; r < 5; ++r)
        for (int c = 0; c < 5; ++c) hess[r * 5 + c] = sum_hess[r][c];
    return 0;
}

// FreeEnergyHessian::hessian (multispot5.cc:693-775) given the sampler's
// draws (states [S][K][F], intensities [S][F][P], which hold every spot): the
// loop after sampler.next written out around the reference's
// compute_spot_intensity_hessian and log-normal prior derivatives. hess [25];
// entry [4][3] is indeterminate as in ref_spot_hessian.
int ref_free_energy_hessian_draws(const double* pix, const int* pixels, const double* spots_in, int K, int F, int P,
                                  int spot, int samples, const unsigned char* states, const double* ints,
                                  double variance, double zFactor, double mu_brightness, double sigma_brightness,
                                  double mu_blur, double sigma_blur, double* hess) {
    const vector<vector<double> > pixel_intensities = frames_of(pix, F, P);
    const vector<Ref3D> px = refs_of(pixels, P);
    const double* sp = spots_in + 5 * (size_t)spot;
    const Vector<5> s5 = makeVector(sp[0], sp[1], sp[2], sp[3], sp[4]);
    const vector<tuple<double, Vector<5>, Matrix<5> > > spot_hess_etc =
        SampledMultispot::compute_spot_intensity_hessian(px, s5, zFactor);
    Matrix<5> sum_hess1 = Zeros;
    Matrix<5> sum_hess2 = Zeros;
    Vector<5> sum_deriv = Zeros;
    for (int sample = 0; sample < samples; sample++) {
        const double* si = ints + (size_t)sample * F * P;
        Matrix<5> h = Zeros;
        Vector<5> deriv = Zeros;
        for (int frame = 0; frame < F; frame++)
            for (int pixel = 0; pixel < P; pixel++) {
                double e = pixel_intensities[frame][pixel] - si[(size_t)frame * P + pixel];
                if (states[((size_t)sample * K + spot) * F + frame] == 0) {
                    h += e * get<2>(spot_hess_etc[pixel]) -
                         get<1>(spot_hess_etc[pixel]).as_col() * get<1>(spot_hess_etc[pixel]).as_row();
                    deriv += e * get<1>(spot_hess_etc[pixel]);
                }
            }
        h[0][0] += hess_log_log_normal(s5[0], mu_brightness, sigma_brightness);
        h[1][1] += hess_log_log_normal(s5[1], mu_blur, sigma_blur);
        sum_hess1 += h;
        deriv[0] += diff_log_log_normal(s5[0], mu_brightness, sigma_brightness);
        deriv[1] += diff_log_log_normal(s5[1], mu_blur, sigma_blur);
        sum_hess2 += deriv.as_col() * deriv.as_row();
        sum_deriv = sum_deriv + deriv;
    }
    sum_hess1 /= (samples * variance);
    sum_hess2 /= (samples * variance);
    sum_deriv /= (samples * variance);
    const Matrix<5> out = sum_hess1 + sum_hess2 - sum_deriv.as_col() * sum_deriv.as_row();
    for (int r = 0; r < 5; ++r)
        for (int c = 0; c < 5; ++c) hess[r * 5 + c] = out[r][c];
    return 0;
}

// NegativeFreeEnergy::compute_with_mask (multispot5.cc:335-405), its steps in
// order, on the reference's GibbsSampler2 and MT19937 (simple_seed(seed)).
// residuals [samples] receives each draw's -err_sum (may be NULL).
double ref_free_energy(const double* pix, const int* pixels, const double* spots_in, const int* moff, const int* midx,
                       int K, int F, int P, const double* A_in, const double* pi_in, double variance, double zFactor,
                       double mu_brightness, double sigma_brightness, double mu_blur, double sigma_blur,
                       int samples, int sample_iterations, int seed, double* residuals) {
    const vector<vector<double> > pixel_intensities = frames_of(pix, F, P);
    const vector<vector<int> > spot_pixels = masks_of(moff, midx, K);
    const vector<Ref3D> px = refs_of(pixels, P);
    Vector<> spots(5 * K);
    for (int i = 0; i < 5 * K; ++i) spots[i] = spots_in[i];
    MT19937 rng;
    rng.simple_seed(seed);
    auto variance_from_sample = [](double sample, double samples, double base_sigma, double scale_pow) {
        double scale = pow(1.25, sample * 1. / samples * scale_pow);
        double sigma = base_sigma * scale;
        double new_variance = sq(sigma);
        return new_variance;
    };
    double base_sigma = sqrt(variance);
    double scale_pow = 100.0;
    const unsigned int nspots = spots.size() / 5;
    const unsigned int nframes = pixel_intensities.size();
    const unsigned int npixels = px.size();
    vector<vector<double> > spot_intensity;
    vector<Vector<5> > spot_vec;
    for (unsigned int i = 0; i < nspots; i++) {
        spot_intensity.push_back(SampledMultispot::compute_spot_intensity(px, spots.slice(i * 5, 5), zFactor));
        spot_vec.push_back(spots.slice(i * 5, 5));
    }
    GibbsSampler2 sampler(pixel_intensities, spot_intensity, spot_vec, spot_pixels, A_of(A_in),
                          makeVector(pi_in[0], pi_in[1], pi_in[2]), variance, sample_iterations);
    double sum = 0;
    for (int sample = 0; sample < samples; sample++) {
        double var1 = variance_from_sample(sample - 2, samples, base_sigma, scale_pow);
        double var2 = variance_from_sample(sample - 1, samples, base_sigma, scale_pow);
        double var3 = variance_from_sample(sample + 1, samples, base_sigma, scale_pow);
        double var4 = variance_from_sample(sample + 2, samples, base_sigma, scale_pow);
        sampler.set_variance(var2);
        sampler.next(rng);
        double err_sum = 0;
        for (unsigned int frame = 0; frame < nframes; frame++)
            for (unsigned int pixel = 0; pixel < npixels; pixel++)
                err_sum -= sq(pixel_intensities[frame][pixel] - sampler.sample_intensities()[frame][pixel]);
        if (residuals) residuals[sample] = -err_sum;
        double e1 = err_sum / (2 * var1) - npixels * nframes * ::log(2 * M_PI * var1) / 2;
        double e2 = err_sum / (2 * var2) - npixels * nframes * ::log(2 * M_PI * var2) / 2;
        double e3 = err_sum / (2 * var3) - npixels * nframes * ::log(2 * M_PI * var3) / 2;
        double e4 = err_sum / (2 * var4) - npixels * nframes * ::log(2 * M_PI * var4) / 2;
        sum += (-e1 + 8 * e2 - 8 * e3 + e4) / 12;
    }
    double log_final = (log(variance_from_sample(samples, samples, base_sigma, scale_pow) * 2 * M_PI) / 2) * npixels *
                       nframes;
    double priors = 0;
    for (unsigned int i = 0; i < nspots; i++) {
        priors += log_log_normal(spots[i * 5 + 0], mu_brightness, sigma_brightness);
        priors += log_log_normal(spots[i * 5 + 1], mu_blur, sigma_blur);
    }
    return -(sum + priors - log_final);
}

}  // extern "C"

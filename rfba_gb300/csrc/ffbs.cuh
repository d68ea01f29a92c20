// Forward filtering and backward-sampling tables of 3B's three-state spot
// chain (on / off / bleached), shared by the Gibbs sampler and the
// sampled-background Hessian.
//
// The filter (forward_algorithm_delta / _delta2, RFBA Main/forward_algorithm.h:
// 385-431) is the reference's log-space recursion held in other coordinates:
// each state's forward value is a mantissa in [0.5, 1) with its own
// power-of-two exponent, so the sequential chain needs neither exp nor log.
// The mantissas are double-float numbers (an unevaluated sum hi + lo of two
// floats, |lo| <= ulp(hi) / 2; Dekker, "A floating-point technique for
// extending the available precision", Numer. Math. 18, 1971, with the
// products' error terms from fused multiply-adds), about 2^-46 relative per
// step: on this GPU a dependent FP64 operation costs on the order of a hundred
// cycles and the FP32 pipe 64 times the FP64 one, and the chain is strictly
// sequential over frames. Terms more than 2^100 below the largest term of a
// step are dropped (far below the format's precision).
//
// Backward sampling (backward_sampling, forward_algorithm.h:546-570) draws
// the last frame from the filter and every earlier frame from the filter
// weighted by the transition into the next frame's state. For every frame and
// each state the next frame may hold (index 3: none, for the last frame) the
// two cumulative thresholds of states 0 and 1 are formed in FP32 and compared
// with the frame's 53-bit uniform exactly, as integers (u <= p exactly when
// u * 2^53 <= floor(p * 2^53)).
#pragma once
#include <cstdint>

#include "dfloat.cuh"

namespace rfba {
namespace ffbs {

using namespace dfloat;

constexpr int kZeroExp = -(1 << 29);  // exponent of a zero forward value
constexpr int kDropBits = 100;

// exp(x) = mant 2^k for x <= 0 (mant in [1, 2)): x = k ln2 + r with r by one
// fused multiply-add. Relative probabilities below 2^-(2^24) are 0. exp(0) is
// (1, 0) without a call.
__device__ __forceinline__ void exp_split(double x, double* mant, int* k) {
    if (x == 0.0) {
        *mant = 1.0;
        *k = 0;
        return;
    }
    const double kd = floor(x * 1.4426950408889634);
    if (kd < -16777216.0) {
        *mant = 0.0;
        *k = kZeroExp;
        return;
    }
    *mant = exp(fma(-kd, 0.6931471805599453, x));
    *k = (int)kd;
}

// A frame's emission terms (p(on), p(off) relative to their larger one) in
// filter form: double-float mantissas emf[2t + s] and exponents emk[2t + s],
// s = 0 on, 1 off (the bleached state emits as off).
__device__ __forceinline__ void emission_terms(double lon, double loff, float2* emf, int* emk) {
    const double m = lon > loff ? lon : loff;
    double mo, mf;
    int ko, kf;
    exp_split(lon - m, &mo, &ko);
    exp_split(loff - m, &mf, &kf);
    emf[0] = df_from(mo);
    emk[0] = ko;
    emf[1] = df_from(mf);
    emk[1] = kf;
}

// The forward filter over F frames, run by one warp (lanes 0-2 carry the
// states; the step is branch-free, so the three lanes never diverge).
// xs[3t + j], es[3t + j]: frame t's forward value of state j.
__device__ __forceinline__ void forward_filter(int lane, int F, const double* A, const double* pi, const float2* emf,
                                               const int* emk, float2* xs, int* es) {
    if (lane >= 3) return;
    const unsigned m3 = 0x7u;
    const int j = lane;
    float2 Aj[3];
    bool nz[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        Aj[i] = df_from(A[i * 3 + j]);
        nz[i] = A[i * 3 + j] != 0.0;
    }
    const int es_sel = j == 0 ? 0 : 1;
    float2 x;
    int E;
    // y * 2^base as a mantissa in [0.5, 1) and an exponent; zero when y is not
    // a positive normal float or base is the zero exponent
    auto normalise = [&](float2 y, int base) {
        const int ex = (__float_as_int(y.x) >> 23) & 0xff;
        const bool zero = !(y.x > 0.f) || ex == 0 || base == kZeroExp;
        const int sh = ex - 126;
        const float sc = pow2f(zero ? 0 : -sh);
        x = zero ? make_float2(0.f, 0.f) : make_float2(y.x * sc, y.y * sc);
        E = zero ? kZeroExp : base + sh;
    };
    {
        const int ke = emk[es_sel];
        normalise(df_mul(df_from(pi[j]), emf[es_sel]), (pi[j] == 0.0 || ke == kZeroExp) ? kZeroExp : ke);
    }
    xs[j] = x;
    es[j] = E;
    for (int t = 1; t < F; ++t) {
        const float2 mant = emf[2 * t + es_sel];
        const int ke = emk[2 * t + es_sel];
        int Ev[3];
        float2 xv[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            Ev[i] = __shfl_sync(m3, E, i);
            xv[i].x = __shfl_sync(m3, x.x, i);
            xv[i].y = __shfl_sync(m3, x.y, i);
        }
        int Em = kZeroExp;
#pragma unroll
        for (int i = 0; i < 3; ++i) Em = (nz[i] && Ev[i] > Em) ? Ev[i] : Em;
        float2 tm[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const int dd = Ev[i] - Em;
            const bool use = nz[i] && Ev[i] != kZeroExp && dd >= -kDropBits;
            const float sc = use ? pow2f(dd < -126 ? -126 : dd) : 0.f;
            tm[i] = df_mul(Aj[i], xv[i]);
            tm[i].x *= sc;
            tm[i].y *= sc;
        }
        const float2 y = df_add(df_add(tm[0], tm[1]), tm[2]);
        normalise(df_mul(y, mant), (Em == kZeroExp || ke == kZeroExp) ? kZeroExp : Em + ke);
        xs[3 * t + j] = x;
        es[3 * t + j] = E;
    }
}

// floor(p * 2^53) for a float p in [0, 1], by integer arithmetic
__device__ __forceinline__ unsigned long long threshold53(float p) {
    const int b = __float_as_int(p);
    const int e = (b >> 23) & 0xff;
    if (p <= 0.f || e == 0) return 0ull;
    const unsigned long long m = (unsigned long long)((b & 0x7fffff) | 0x800000);  // p = m 2^(e - 150)
    const int s = e - 97;                                                          // p 2^53 = m 2^s
    return s >= 0 ? (m << s) : (s > -64 ? (m >> -s) : 0ull);
}

// Cumulative thresholds (p0, p1) of states 0 and 1 for frame t when the next
// frame holds state nx (3: no next frame): the filter's values weighted by the
// transition into nx, as fractions of their total, in FP32; no weight at all
// gives (1, 1), state 0, as a zero total does in the reference. Af: A as
// floats; nzA: bit 3i + n set where A[i][n] != 0.
__device__ __forceinline__ float2 frame_thresholds(int t, int nx, const float2* xs, const int* es, const float* Af,
                                                   unsigned nzA) {
    int Em = kZeroExp;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const bool use = (nx == 3 || ((nzA >> (3 * i + nx)) & 1u)) && es[3 * t + i] != kZeroExp;
        Em = (use && es[3 * t + i] > Em) ? es[3 * t + i] : Em;
    }
    float a[3], tot = 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const bool use = (nx == 3 || ((nzA >> (3 * i + nx)) & 1u)) && es[3 * t + i] != kZeroExp;
        const int dd = es[3 * t + i] - Em;
        const float tr = nx == 3 ? 1.f : Af[3 * i + nx];
        a[i] = (use && dd >= -126) ? xs[3 * t + i].x * pow2f(dd < -126 ? -126 : dd) * tr : 0.f;
        tot += a[i];
    }
    return tot > 0.f ? make_float2(a[0] / tot, (a[0] + a[1]) / tot) : make_float2(1.f, 1.f);
}

// The state drawn by a uniform U (53-bit integer) against thresholds (p0, p1).
__device__ __forceinline__ int draw_state(unsigned long long U, float2 th) {
    return U <= threshold53(th.x) ? 0 : (U <= threshold53(th.y) ? 1 : 2);
}

// The draws of frame t from its uniform U for each state the next frame may
// hold (index 3: no next frame).
__device__ __forceinline__ void frame_draws(int t, unsigned long long U, const float2* xs, const int* es,
                                            const float* Af, unsigned nzA, unsigned char out[4]) {
#pragma unroll
    for (int nx = 0; nx < 4; ++nx) out[nx] = (unsigned char)draw_state(U, frame_thresholds(t, nx, xs, es, Af, nzA));
}

// A as floats and its non-zero pattern, for frame_thresholds.
__device__ __forceinline__ void transition_floats(const double* A, float Af[9], unsigned* nzA) {
    unsigned m = 0;
#pragma unroll
    for (int n = 0; n < 9; ++n) {
        Af[n] = (float)A[n];
        m |= A[n] != 0.0 ? 1u << n : 0u;
    }
    *nzA = m;
}

// The backward walk through a decision table, by one warp: sel[4t + n] is the
// state frame t takes when frame t + 1 holds n (n = 3: no next frame), so
// frame t's decisions are a map from {0..3} to {0..2}, packed here as four
// 2-bit fields. The walk s_t = f_t(s_{t+1}), s_F = 3, is a suffix composition
// of those maps: each lane composes the maps of its chunk of frames, a
// Kogge-Stone scan over the lanes composes the chunks that follow, and each
// lane then walks its own chunk from the state its successors hand it.
__device__ __forceinline__ unsigned map_compose(unsigned g, unsigned h) {  // g after h: n -> g(h(n))
    unsigned r = 0;
#pragma unroll
    for (int n = 0; n < 4; ++n) r |= ((g >> (2 * ((h >> (2 * n)) & 3u))) & 3u) << (2 * n);
    return r;
}
__device__ __forceinline__ void walk_decisions(int lane, int F, const unsigned char* sel, unsigned char* sts) {
    const unsigned full = 0xffffffffu;
    const int per = (F + 31) / 32;
    const int a = min(F, lane * per), b = min(F, a + per);
    auto code = [&](int t) {
        const unsigned w = *reinterpret_cast<const unsigned*>(sel + 4 * t);  // four decision bytes
        return (w & 3u) | ((w >> 6) & 0xCu) | ((w >> 12) & 0x30u) | ((w >> 18) & 0xC0u);
    };
    // this chunk's map: s_a from s_b
    unsigned h = 0xE4u;  // identity
    for (int t = b - 1; t >= a; --t) h = map_compose(code(t), h);
    // suffix scan: H_l = h_l after h_(l+1) after ... (lanes past the last frame hold the identity)
    unsigned H = h;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned nxt = __shfl_down_sync(full, H, o);
        if (lane + o < 32) H = map_compose(H, nxt);
    }
    // the state of frame b (the chunk after this one's first frame) is H_(l+1)(3)
    const unsigned after = __shfl_down_sync(full, H, 1);
    int s = lane + 1 < 32 ? (int)((after >> 6) & 3u) : 3;
    for (int t = b - 1; t >= a; --t) {
        s = sel[4 * t + s];
        sts[t] = (unsigned char)s;
    }
}

// 53-bit integer uniform of Philox outputs a, b (u53 = U 2^-53)
__device__ __forceinline__ unsigned long long uniform53(uint32_t a, uint32_t b) {
    return ((unsigned long long)(a >> 5) << 26) | (unsigned long long)(b >> 6);
}

// The filtering distribution of frame t (trace output).
__device__ __forceinline__ void filter_probs(int t, const float2* xs, const int* es, double out[3]) {
    int Em = kZeroExp;
    for (int i = 0; i < 3; ++i) Em = max(Em, es[3 * t + i]);
    double w[3], tot = 0.0;
    for (int i = 0; i < 3; ++i) {
        const int dd = es[3 * t + i] - Em;
        w[i] = (es[3 * t + i] != kZeroExp && dd >= -1022) ? df_to(xs[3 * t + i]) * ldexp(1.0, dd) : 0.0;
        tot += w[i];
    }
    for (int i = 0; i < 3; ++i) out[i] = w[i] / tot;
}

}  // namespace ffbs
}  // namespace rfba

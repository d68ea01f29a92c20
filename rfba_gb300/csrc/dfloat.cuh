// Double-float arithmetic: a value as the unevaluated sum hi + lo of two
// floats, |lo| <= ulp(hi) / 2 (Dekker, "A floating-point technique for
// extending the available precision", Numer. Math. 18, 1971; the products'
// error terms by fused multiply-add), about 2^-46 relative per operation, on
// the FP32 pipe. On this GPU the FP32 pipe has 64 times the FP64 pipe's
// throughput and a dependent FP64 operation costs on the order of a hundred
// cycles, so sequential chains and dot products that need more than FP32 but
// not all of FP64 run here. The helpers follow the published algorithms
// (two-sum, fast-two-sum, two-product by FMA) and are exact for any signs.
#pragma once

namespace rfba {
namespace dfloat {

__device__ __forceinline__ float2 df_from(double v) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - (double)h));
}
__device__ __forceinline__ double df_to(float2 a) { return (double)a.x + (double)a.y; }
// s + e with |s| >= |e| as a normalised pair
__device__ __forceinline__ float2 df_fast_two_sum(float s, float e) {
    const float r = s + e;
    return make_float2(r, e - (r - s));
}
// s + e as a normalised pair, any magnitudes (two-sum)
__device__ __forceinline__ float2 df_two_sum(float s, float e) {
    const float r = s + e;
    const float v = r - s;
    return make_float2(r, (s - (r - v)) + (e - v));
}
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    return df_fast_two_sum(p, e);
}
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    const float s = a.x + b.x;
    const float v = s - a.x;
    float e = (a.x - (s - v)) + (b.x - v);
    e += a.y + b.y;
    return df_fast_two_sum(s, e);
}
// acc += a * b for a running sum kept unnormalised: the product's high part
// joins acc.x by two-sum (Knuth), its error terms and the two-sum's rounding
// join acc.y, which holds many ulps of acc.x; df_two_sum(acc.x, acc.y)
// normalises the sum once at the end.
__device__ __forceinline__ void df_acc_mul(float2& acc, float2 a, float2 b) {
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    const float s = acc.x + p;
    const float bp = s - acc.x;
    const float err = (acc.x - (s - bp)) + (p - bp);
    acc.y += err + e;
    acc.x = s;
}
// 2^d as a float, -126 <= d <= 127
__device__ __forceinline__ float pow2f(int d) { return __int_as_float((d + 127) << 23); }

}  // namespace dfloat
}  // namespace rfba

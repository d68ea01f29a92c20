// Temporal reduction carried across time batches (sm_103a).
//
// A series too long for its radiality and intensity stacks to sit in HBM whole
// is run in batches of volumes: the radiality kernel fills the stacks of one
// batch, then this kernel folds that batch into a per-subvoxel state and, after
// the last batch, writes the map. One thread per subvoxel; the state is
// structure-of-arrays (field f of subvoxel g at state[f * stride + g]), so
// every load and store is coalesced.
//
// The methods and their state (same semantics as temporal.cu, which reduces a
// whole series at once):
//   TRM   kernel.cu:332-366  running max from 0                    1 field
//   TRA   kernel.cu:291-327  Kahan sum of rad (rad*I with IW)     2 fields
//   TRPPM kernel.cu:372-419  Kahan sums of r+, r+^2 and I          6 fields
// TRM, TRA and TRPPM add the values in the same order as the one-pass kernel,
// so the streamed map is bit-identical to it.
//   TRAC, ITC 0, order k (kernel.cu:423-500): the cumulant sums run over
//   the window t = 0 .. T-k-1 of the deviations d_t = r_t - mean, with the mean
//   over the whole series, which is known only after the last batch. The state
//   keeps sums of products of y_t = r_t - K instead, K being the subvoxel's mean
//   over the first batch (so y stays centred and the expansion below is well
//   conditioned), the last k-1 values of y, and Kahan sums of y and of r*I. With
//   c = mean - K every window sum of deviation products is a polynomial in c
//   over the sums of y products (for k = 2:
//   sum d_t d_{t+1} = P01 - c (S0 + S1) + N c^2), evaluated in double after the
//   last batch. The sums are Kahan-compensated FP32 like the one-pass kernel's;
//   the result agrees with it to rounding, not bit for bit.
// TRAC with ITC 1 bins the whole series level by level and is not carried; a
// forward that needs it slices space instead.
#include <cuda_runtime.h>

#include "srrf_internal.h"

namespace rfba {
namespace {

struct KahanRef {
    float* s;
    float* c;
    __device__ __forceinline__ void add(float x) {
        const float y = x - *c;
        const float t = *s + y;
        *c = (t - *s) - y;
        *s = t;
    }
    __device__ __forceinline__ double value() const { return (double)*s - (double)*c; }
};

// number of window sums of y products for order k: all non-empty subsets of
// the k window positions of size <= k (size 1: S_j, 2: P_ij, ...)
__host__ __device__ constexpr int trac_sums(int k) { return k == 2 ? 3 : (k == 3 ? 7 : 15); }

}  // namespace

int temporal_stream_fields(int method, int order) {
    switch (method) {
        case 0: return 1;
        case 1: return 2;
        case 2: return 6;
        default: {
            const int k = order < 2 ? 2 : (order > 4 ? 4 : order);
            // K, sum y (2), sum r*I (2), last k-1 values, the window sums (2 each)
            return 5 + (k - 1) + 2 * trac_sums(k);
        }
    }
}

namespace {

// Each thread's values of the batch are staged in shared memory by cp.async
// (no register staging, a chunk's copies all in flight at once), double
// buffered in chunks of kChunk volumes; the sums then read shared memory.
// Only the thread that copied a value reads it back.
constexpr int kStreamThreads = 256;
constexpr int kChunk = 8;
using Stage = float[2][kChunk][kStreamThreads];

__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// f(i, r, I) for the batch's values i = 0 .. nb - 1 in order (I is 0 when the
// intensity stack is not needed).
template <class F>
__device__ __forceinline__ void for_each_value(const float* rad, const float* inten, long long V, int nb,
                                               bool need_int, Stage& sr, Stage& si, F&& f) {
    const int tx = threadIdx.x;
    auto issue = [&](int buf, int c0) {
        const int n = min(kChunk, nb - c0);
        for (int j = 0; j < n; ++j) {
            cp_async4(&sr[buf][j][tx], rad + (long long)(c0 + j) * V);
            if (need_int) cp_async4(&si[buf][j][tx], inten + (long long)(c0 + j) * V);
        }
        cp_async_commit();
    };
    issue(0, 0);
    int buf = 0;
    for (int c0 = 0; c0 < nb; c0 += kChunk) {
        if (c0 + kChunk < nb) {
            issue(buf ^ 1, c0 + kChunk);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        const int n = min(kChunk, nb - c0);
        for (int j = 0; j < n; ++j) f(c0 + j, sr[buf][j][tx], need_int ? si[buf][j][tx] : 0.f);
        buf ^= 1;
    }
}

template <int K>
__device__ __forceinline__ void trac_carry(const StreamParams& p, long long g, const float* rad, const float* inten,
                                           long long V, Stage& sr, Stage& si, float* out_val) {
    constexpr int NS = trac_sums(K);
    constexpr int NF = 5 + (K - 1) + 2 * NS;
    float* st = p.state + g;
    const long long S = p.state_stride;
    float reg[NF];
    const int nb = p.t_hi - p.t_lo;
    const bool iw = p.iw == 1;
    if (p.t_lo == 0) {
        // K: the mean of the first batch, in the order the values arrive
        float m = 0.f;
        for_each_value(rad, inten, V, nb, false, sr, si, [&](int, float r, float) { m += r; });
        reg[0] = m / (float)nb;
#pragma unroll
        for (int f = 1; f < NF; ++f) reg[f] = 0.f;
    } else {
#pragma unroll
        for (int f = 0; f < NF; ++f) reg[f] = st[f * S];
    }
    const float shift = reg[0];
    KahanRef ysum{&reg[1], &reg[2]};
    KahanRef iws{&reg[3], &reg[4]};
    float* prev = &reg[5];  // prev[0] = y_{t-1}, prev[1] = y_{t-2}, prev[2] = y_{t-3}
    float* sums = &reg[5 + (K - 1)];
    auto sum = [&](int i) { return KahanRef{&sums[2 * i], &sums[2 * i + 1]}; };
    const int N = p.T - K;  // window length
    for_each_value(rad, inten, V, nb, iw, sr, si, [&](int i, float r, float I) {
        const int t = p.t_lo + i;
        const float y = r - shift;
        ysum.add(y);
        if (iw) iws.add(r * I);
        const int w = t - (K - 1);
        if (w >= 0 && w < N) {
            if (K == 2) {
                const float a = prev[0], b = y;
                sum(0).add(a);
                sum(1).add(b);
                sum(2).add(a * b);
            } else if (K == 3) {
                const float a = prev[1], b = prev[0], c = y;
                sum(0).add(a);
                sum(1).add(b);
                sum(2).add(c);
                sum(3).add(a * b);
                sum(4).add(a * c);
                sum(5).add(b * c);
                sum(6).add(a * b * c);
            } else {
                const float a = prev[2], b = prev[1], c = prev[0], d = y;
                sum(0).add(a);
                sum(1).add(b);
                sum(2).add(c);
                sum(3).add(d);
                sum(4).add(a * b);
                sum(5).add(a * c);
                sum(6).add(a * d);
                sum(7).add(b * c);
                sum(8).add(b * d);
                sum(9).add(c * d);
                sum(10).add(a * b * c);
                sum(11).add(a * b * d);
                sum(12).add(a * c * d);
                sum(13).add(b * c * d);
                sum(14).add(a * b * c * d);
            }
        }
#pragma unroll
        for (int j = K - 2; j > 0; --j) prev[j] = prev[j - 1];
        prev[0] = y;
    });
    if (!p.last) {
#pragma unroll
        for (int f = 0; f < NF; ++f) st[f * S] = reg[f];
        return;
    }
    double out = 0.0;
    if (N > 0) {
        const double c = ysum.value() / (double)p.T;
        const double n = (double)N;
        auto v = [&](int i) { return sum(i).value(); };
        if (K == 2) {
            out = fabs(v(2) - c * (v(0) + v(1)) + n * c * c);
        } else if (K == 3) {
            out = fabs(v(6) - c * (v(3) + v(4) + v(5)) + c * c * (v(0) + v(1) + v(2)) - n * c * c * c);
        } else {
            auto pair = [&](int pij, int si_, int sj) { return v(pij) - c * (v(si_) + v(sj)) + n * c * c; };
            const double ab = pair(4, 0, 1), ac = pair(5, 0, 2), ad = pair(6, 0, 3);
            const double bc = pair(7, 1, 2), bd = pair(8, 1, 3), cd = pair(9, 2, 3);
            const double abcd = v(14) - c * (v(10) + v(11) + v(12) + v(13)) +
                                c * c * (v(4) + v(5) + v(6) + v(7) + v(8) + v(9)) -
                                c * c * c * (v(0) + v(1) + v(2) + v(3)) + n * c * c * c * c;
            out = fabs(abcd - ab * cd - ac * bd - ad * bc);
        }
        out /= (double)p.T;
    }
    float res = (float)out;
    if (iw) res = (float)(iws.value() / (double)p.T) * res;
    *out_val = res;
}

__global__ void __launch_bounds__(kStreamThreads) temporal_stream_kernel(const StreamParams p) {
    __shared__ Stage sr, si;
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= p.total_vox) return;
    int lo = 0, hi = p.nblocks - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (p.vox_prefix[mid] <= gid) lo = mid;
        else hi = mid - 1;
    }
    const BlockDev& B = p.blocks[lo];
    const long long v = gid - p.vox_prefix[lo];
    const long long V = B.vox;
    const float* rad = p.rad_stack + B.stack_off + v;
    const float* inten = p.int_stack + B.stack_off + v;
    const long long S = p.state_stride;
    float* st = p.state + gid;
    const int nb = p.t_hi - p.t_lo;
    const bool first = p.t_lo == 0;
    const bool iw = p.iw == 1;
    float result = 0.f;

    if (p.method == 1) {  // TRA
        float s = first ? 0.f : st[0], c = first ? 0.f : st[S];
        KahanRef k{&s, &c};
        for_each_value(rad, inten, V, nb, iw, sr, si, [&](int, float r, float I) { k.add(iw ? r * I : r); });
        if (!p.last) {
            st[0] = s;
            st[S] = c;
            return;
        }
        result = s / (float)p.T;
    } else if (p.method == 0) {  // TRM
        float mip = first ? 0.f : st[0];
        for_each_value(rad, inten, V, nb, iw, sr, si,
                       [&](int, float r, float I) { mip = fmaxf(iw ? r * I : r, mip); });
        if (!p.last) {
            st[0] = mip;
            return;
        }
        result = mip;
    } else if (p.method == 2) {  // TRPPM
        float r6[6];
        for (int f = 0; f < 6; ++f) r6[f] = first ? 0.f : st[f * S];
        KahanRef s1{&r6[0], &r6[1]}, s2{&r6[2], &r6[3]}, s3{&r6[4], &r6[5]};
        for_each_value(rad, inten, V, nb, iw, sr, si, [&](int, float rv, float I) {
            const float r = fmaxf(rv, 0.f);
            s1.add(r);
            s2.add(r * r);
            if (iw) s3.add(I);
        });
        if (!p.last) {
            for (int f = 0; f < 6; ++f) st[f * S] = r6[f];
            return;
        }
        const float count = fmaxf(0.5f * (float)p.T * (float)(p.T + 1), 1.f);
        float pps = (0.5f * (r6[0] * r6[0] + r6[2])) / count;
        if (iw) pps *= r6[4] / (float)p.T;
        result = pps;
    } else {  // TRAC, ITC 0
        if (p.order == 3) trac_carry<3>(p, gid, rad, inten, V, sr, si, &result);
        else if (p.order == 4) trac_carry<4>(p, gid, rad, inten, V, sr, si, &result);
        else trac_carry<2>(p, gid, rad, inten, V, sr, si, &result);
        if (!p.last) return;
    }

    const long long nx = B.nreg[0], ny = B.nreg[1];
    long long x, y, z;
    if (v < 0x7fffffffLL) {
        const unsigned vv = (unsigned)v, ux = (unsigned)nx, uy = (unsigned)ny;
        const unsigned q = vv / ux;
        x = vv - q * ux;
        y = q % uy;
        z = q / uy;
    } else {
        x = v % nx;
        y = (v / nx) % ny;
        z = v / (nx * ny);
    }
    p.out[B.out_offset + x * B.out_stride[0] + y * B.out_stride[1] + z * B.out_stride[2]] = result;
}

}  // namespace

int launch_temporal_stream(const StreamParams& p, void* stream) {
    if (p.total_vox == 0 || p.t_hi <= p.t_lo) return 0;
    const long long grid = (p.total_vox + kStreamThreads - 1) / kStreamThreads;
    temporal_stream_kernel<<<(unsigned)grid, kStreamThreads, 0, static_cast<cudaStream_t>(stream)>>>(p);
    return (int)cudaGetLastError();
}

}  // namespace rfba

// Differentiable SRRF path (sm_103a): drift resampling, and the adjoint of a
// scalar objective on the map with respect to the input voxels and the
// per-volume drift shifts. The reference has no derivatives; the forward it
// differentiates is the reference's radiality (kernel.cu:44-287) and temporal
// reduction (TRA kernel.cu:291-327, TRAC with ITC 0 kernel.cu:469-507) on
// volumes resampled by the drift operator
//     I'_t(x) = sum_{i,j,k} c(x + d_x - i) c(y + d_y - j) c(z + d_z - k) I_t[clamp(i, j, k)],
// c = the reference's Catmull-Rom kernel (kernel.cu:128-138), applied one axis
// at a time (x, then y, then z).
//
// Backward, per call:
//   1. temporal adjoint, one thread per subvoxel: dL/drad_t and dL/dI_t from
//      dL/dmap and the stored radiality/intensity stacks;
//   2. radiality adjoint, persistent over (tile, time) like the forward: the
//      interpolated gradient at every ring sample is recomputed (not stored),
//      the derivative of the radiality term is pushed back through the z pass
//      (registers), the frame rotation, the y pass (shared-memory atomics), the
//      x pass (shared-memory atomics) and the gradient stencil (gather), and the
//      tile's contribution to dL/dI' is added to global memory;
//   3. the drift operator's transpose gives dL/dI, and dL/dd_t is the sum over
//      the volume of dL/dI'_t times the resampling with derivative weights on
//      one axis.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>

#include "srrf_internal.h"

namespace rfba {
namespace {

__device__ __forceinline__ float rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float sign_weight(float w, float d) {
    return __int_as_float(__float_as_int(w) | (~__float_as_int(d) & 0x80000000));
}
__device__ __forceinline__ float2 dup(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
__device__ __forceinline__ int floordiv(int a, int b) {
    int q = a / b;
    return (a % b != 0 && a < 0) ? q - 1 : q;
}
template <int V>
struct IntC {
    static constexpr int value = V;
};

// Bounds check of a computed global index: out of range records the first
// offence (site in the top byte, index below) and the access is skipped.
__device__ __forceinline__ bool in_range(long long i, long long n, unsigned long long* err, int site) {
    if (i >= 0 && i < n) return true;
    if (err) atomicCAS(err, 0ull, ((unsigned long long)site << 56) | ((unsigned long long)i & 0x00ffffffffffffffull));
    return false;
}

// Catmull-Rom kernel and its derivative (a = 0.5), kernel.cu:128-138.
__device__ __forceinline__ float cr(float xx) {
    const float a = 0.5f;
    const float x = fabsf(xx);
    if (x < 1.f) return x * x * (x * (2.f - a) + (a - 3.f)) + 1.f;
    if (x < 2.f) return ((-a * x + 5.f * a) * x - 8.f * a) * x + 4.f * a;
    return 0.f;
}
__device__ __forceinline__ float dcr(float xx) {
    const float a = 0.5f;
    const float x = fabsf(xx), s = xx < 0.f ? -1.f : 1.f;
    if (x < 1.f) return s * (3.f * (2.f - a) * x * x + 2.f * (a - 3.f) * x);
    if (x < 2.f) return s * ((-3.f * a * x + 10.f * a) * x - 8.f * a);
    return 0.f;
}

// ---------------------------------------------------------------------------
// Drift operator, one axis: mode 0 resamples, mode 1 resamples with derivative
// weights, mode 2 applies the transpose (gather over the outputs whose clamped
// taps hit each input position).
__global__ void shift_axis_kernel(const float* __restrict__ src, float* __restrict__ dst, int W, int H, int D, int T,
                                  int axis, const float* __restrict__ shifts, int mode, unsigned long long* err) {
    const long long n = (long long)W * H * D * T;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % W);
        const int y = (int)((i / W) % H);
        const int z = (int)((i / ((long long)W * H)) % D);
        const int t = (int)(i / ((long long)W * H * D));
        const int len = axis == 0 ? W : (axis == 1 ? H : D);
        const long long stride = axis == 0 ? 1 : (axis == 1 ? W : (long long)W * H);
        const int c = axis == 0 ? x : (axis == 1 ? y : z);
        const long long line = i - (long long)c * stride;
        const float d = shifts[3 * t + axis];
        float acc = 0.f;
        if (mode != 2) {
            const float pos = (float)c + d;
            const int base = (int)floorf(pos);
#pragma unroll
            for (int k = -1; k <= 2; ++k) {
                const int ii = clampi(base + k, 0, len - 1);
                const float u = pos - (float)(base + k);
                const long long si = line + ii * stride;
                if (in_range(si, n, err, 1)) acc = fmaf(mode == 1 ? dcr(u) : cr(u), src[si], acc);
            }
        } else {
            // outputs x whose taps floor(x + d) - 1 .. + 2, clamped, include c
            int lo = (int)floorf((float)c - d) - 3, hi = (int)ceilf((float)c - d) + 3;
            if (c == 0) lo = -1000000;
            if (c == len - 1) hi = 1000000;
            lo = max(lo, 0);
            hi = min(hi, len - 1);
            for (int xo = lo; xo <= hi; ++xo) {
                const float pos = (float)xo + d;
                const int base = (int)floorf(pos);
                float w = 0.f;
#pragma unroll
                for (int k = -1; k <= 2; ++k)
                    if (clampi(base + k, 0, len - 1) == c) w += cr(pos - (float)(base + k));
                const long long si = line + xo * stride;
                if (w != 0.f && in_range(si, n, err, 2)) acc = fmaf(w, src[si], acc);
            }
        }
        dst[i] = acc;
    }
}

// dL/dd[t][axis] = sum over volume t of g[t] * dv[t] (double accumulation).
__global__ void drift_dot_kernel(const float* __restrict__ g, const float* __restrict__ dv, long long nv, int axis,
                                 double* __restrict__ out, unsigned long long* err) {
    const int t = blockIdx.y;
    const float* gt = g + (long long)t * nv;
    const float* dt = dv + (long long)t * nv;
    double acc = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (long long)gridDim.x * blockDim.x)
        acc += (double)gt[i] * (double)dt[i];
    __shared__ double red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(out + 3 * t + axis, red[0]);
}

// Drift operator on all three axes at once: the x-, y- and z-passes with
// per-axis index clamping compose to one 4 x 4 x 4 tensor-product stencil with
// clamped indices. mode 0 writes I'_t; mode 1 adds, per volume, the sums over
// voxels of g * dI'/dd_a (a = x, y, z: derivative weights on axis a) into
// out[3 t + a] (FP64, one atomic per block and axis).
template <int MODE>
__global__ void drift3d_kernel(const float* __restrict__ src, float* __restrict__ dst, const float* __restrict__ g,
                               int W, int H, int D, const float* __restrict__ shifts, double* __restrict__ out) {
    const int t = blockIdx.y;
    const long long nv = (long long)W * H * D;
    const float* st = src + (long long)t * nv;
    const float dx = shifts[3 * t], dy = shifts[3 * t + 1], dz = shifts[3 * t + 2];
    double acc[3] = {0.0, 0.0, 0.0};
    // one (z, y) output row per block iteration, x across the threads; every
    // index is clamped into the volume, so no tap can leave it
    for (int row = blockIdx.x; row < D * H; row += gridDim.x) {
        const int z = row / H, y = row - z * H;
        const float py = (float)y + dy, pz = (float)z + dz;
        const int by = (int)floorf(py), bz = (int)floorf(pz);
        float wy[4], wz[4], ey[4], ez[4];
        const float* rows[4][4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            wy[k] = cr(py - (float)(by + k - 1));
            wz[k] = cr(pz - (float)(bz + k - 1));
            if (MODE == 1) {
                ey[k] = dcr(py - (float)(by + k - 1));
                ez[k] = dcr(pz - (float)(bz + k - 1));
            }
        }
#pragma unroll
        for (int kz = 0; kz < 4; ++kz)
#pragma unroll
            for (int ky = 0; ky < 4; ++ky)
                rows[kz][ky] = st + ((long long)clampi(bz + kz - 1, 0, D - 1) * H + clampi(by + ky - 1, 0, H - 1)) * W;
        for (int x = threadIdx.x; x < W; x += blockDim.x) {
            const float px = (float)x + dx;
            const int bx = (int)floorf(px);
            float wx[4], ex[4];
            int ix[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                ix[k] = clampi(bx + k - 1, 0, W - 1);
                wx[k] = cr(px - (float)(bx + k - 1));
                if (MODE == 1) ex[k] = dcr(px - (float)(bx + k - 1));
            }
            // x pass per (z, y) row, then y, then z, as the per-axis passes compose
            float v = 0.f, gx_ = 0.f, gy_ = 0.f, gz_ = 0.f;
#pragma unroll
            for (int kz = 0; kz < 4; ++kz) {
                float sy = 0.f, sy_dx = 0.f, sy_dy = 0.f;
#pragma unroll
                for (int ky = 0; ky < 4; ++ky) {
                    const float* rp = rows[kz][ky];
                    float sx = 0.f, sx_d = 0.f;
#pragma unroll
                    for (int kx = 0; kx < 4; ++kx) {
                        const float val = __ldg(rp + ix[kx]);
                        sx = fmaf(wx[kx], val, sx);
                        if (MODE == 1) sx_d = fmaf(ex[kx], val, sx_d);
                    }
                    sy = fmaf(wy[ky], sx, sy);
                    if (MODE == 1) {
                        sy_dx = fmaf(wy[ky], sx_d, sy_dx);
                        sy_dy = fmaf(ey[ky], sx, sy_dy);
                    }
                }
                v = fmaf(wz[kz], sy, v);
                if (MODE == 1) {
                    gx_ = fmaf(wz[kz], sy_dx, gx_);
                    gy_ = fmaf(wz[kz], sy_dy, gy_);
                    gz_ = fmaf(ez[kz], sy, gz_);
                }
            }
            const long long o = (long long)t * nv + (long long)row * W + x;
            if (MODE == 0) {
                dst[o] = v;
            } else {
                const double gg = g[o];
                acc[0] += gg * gx_;
                acc[1] += gg * gy_;
                acc[2] += gg * gz_;
            }
        }
    }
    if (MODE == 1) {
        __shared__ double red[3][256];
#pragma unroll
        for (int a = 0; a < 3; ++a) red[a][threadIdx.x] = acc[a];
        __syncthreads();
        for (int s2 = blockDim.x / 2; s2 > 0; s2 >>= 1) {
            if (threadIdx.x < s2)
#pragma unroll
                for (int a = 0; a < 3; ++a) red[a][threadIdx.x] += red[a][threadIdx.x + s2];
            __syncthreads();
        }
        if (threadIdx.x < 3) atomicAdd(out + 3 * t + threadIdx.x, red[threadIdx.x][0]);
    }
}

// ---------------------------------------------------------------------------
// Temporal adjoint, one thread per subvoxel of the single block. FP32 with
// compensated (Kahan) sums over t: FP64 arithmetic runs at a small fraction of
// the FP32 rate on this GPU and would make this HBM-sized pass compute-bound.
struct KSum {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

// Adjoint of TRAC with ITC 1 (kernel.cu:437-555) for one subvoxel; r, I its
// radiality and intensity series (stride V), m and IW the level-0 mean and
// intensity weight. The forward bins the series in place level after level
// (entry t < nB - k becomes the mean of entries tk .. tk + k - 1, entry 0
// reading itself as 0, entries past the series reading 0; the rest keep their
// values) and sums per level AB (reset) and ABC / ABCD, CD, AC, BD, AD, BC (not
// reset) around m; out = sum_l |C_l| / nB_l. Reverse mode over the levels with
// O(T) memory per subvoxel: one forward sweep gives each level's sums, hence
// d out / d(each level's partial sums) as suffix sums over the levels; then,
// from the deepest level up, the level's array state is replayed from r into
// S (the dL/dI buffer, free until the end) and the gradient with respect to
// that state is formed in place in Gd (the dL/dS buffer): the level's own
// sums' derivatives plus its transposed binning of the next level's gradient,
// walking the entries downwards so that every entry a later bin reads is still
// the next level's. The level-0 mean takes minus the sum of all direct terms
// over T. FP32 with compensated sums in the forward sweep.
constexpr int kMaxLevels = 32;

__device__ void trac_itc1_adjoint(const float* r, const float* I, long long V, int T, int k, int iw, int renorm,
                                  int poscon, float g, float m, float IW, float* Gd, float* S) {
    float Cl[kMaxLevels], ABl[kMaxLevels], CDa[kMaxLevels], ACa[kMaxLevels], BDa[kMaxLevels], ADa[kMaxLevels],
        BCa[kMaxLevels];
    int nbl[kMaxLevels];
    const float invk = 1.f / (float)k;
    // binning of one level in place (the forward's order)
    auto bin_level = [&](int nb) {
        for (int t = 0; t < nb - k; ++t) {
            float nv = 0.f;
            if (t * k < nb)
                for (int j = 0; j < k; ++j) {
                    const int src = t * k + j;
                    const float rv = (src == t || src >= T) ? 0.f : S[(long long)src * V];
                    nv += rv / (float)k;
                }
            S[(long long)t * V] = nv;
        }
    };
    for (int t = 0; t < T; ++t) S[(long long)t * V] = r[(long long)t * V];
    KSum ABC, ABCD, CD, AC, BD, AD, BC;
    float out_raw = 0.f;
    int L = 0, nB = T;
    while (nB > k && L < kMaxLevels) {
        KSum AB;
        for (int t = 0; t < nB - k; ++t) {
            const float A = S[(long long)t * V] - m, B = S[(long long)(t + 1) * V] - m;
            AB.add(A * B);
            if (k >= 3) {
                const float C = S[(long long)(t + 2) * V] - m;
                if (k == 3) ABC.add(A * B * C);
                if (k == 4) {
                    const float D = S[(long long)(t + 3) * V] - m;
                    ABCD.add(A * B * C * D);
                    CD.add(C * D);
                    AC.add(A * C);
                    BD.add(B * D);
                    AD.add(A * D);
                    BC.add(B * C);
                }
            }
        }
        bin_level(nB);
        const float C = k == 2 ? AB.s : (k == 3 ? ABC.s : ABCD.s - AB.s * CD.s - AC.s * BD.s - AD.s * BC.s);
        Cl[L] = C;
        ABl[L] = AB.s;
        CDa[L] = CD.s;
        ACa[L] = AC.s;
        BDa[L] = BD.s;
        ADa[L] = AD.s;
        BCa[L] = BC.s;
        nbl[L] = nB;
        out_raw += fabsf(C) / (float)nB;
        ++L;
        nB = nB / k;
    }
    // d out / d(partial sums of each level): suffix sums over the levels
    float wM[kMaxLevels], wAB[kMaxLevels], wCD[kMaxLevels], wAC[kMaxLevels], wBD[kMaxLevels], wAD[kMaxLevels],
        wBC[kMaxLevels];
    {
        float ss = 0.f, scd = 0.f, sac = 0.f, sbd = 0.f, sad = 0.f, sbc = 0.f;
        for (int l = L - 1; l >= 0; --l) {
            const float sl = (Cl[l] > 0.f ? 1.f : (Cl[l] < 0.f ? -1.f : 0.f)) / (float)nbl[l];
            ss += sl;
            scd -= sl * ABl[l];
            sac -= sl * BDa[l];
            sbd -= sl * ACa[l];
            sad -= sl * BCa[l];
            sbc -= sl * ADa[l];
            wM[l] = k == 2 ? sl : ss;
            wAB[l] = -sl * CDa[l];
            wCD[l] = scd;
            wAC[l] = sac;
            wBD[l] = sbd;
            wAD[l] = sad;
            wBC[l] = sbc;
        }
    }
    for (int t = 0; t < T; ++t) Gd[(long long)t * V] = 0.f;
    float dm = 0.f;
    for (int l = L - 1; l >= 0; --l) {
        // replay level l's state
        for (int t = 0; t < T; ++t) S[(long long)t * V] = r[(long long)t * V];
        int nb = T;
        for (int j = 0; j < l; ++j) {
            bin_level(nb);
            nb /= k;
        }
        const int N = nb - k;
        auto sv = [&](int t) { return S[(long long)t * V] - m; };
        for (int p = T - 1; p >= 0; --p) {
            // transposed binning: entries at or past N keep their value, entry
            // p feeds bin p / k
            float gp = p >= N ? Gd[(long long)p * V] : 0.f;
            const int tb = p / k;
            if (tb < N && tb * k < nb && p != tb) gp += Gd[(long long)tb * V] * invk;
            // this level's sums: the products starting at t = p - q hold entry p
            float dp = 0.f;
            for (int q = 0; q < k; ++q) {
                const int t = p - q;
                if (t < 0 || t >= N) continue;
                const float A = sv(t), B = sv(t + 1);
                if (k == 2) {
                    dp += wM[l] * (q == 0 ? B : A);
                } else if (k == 3) {
                    const float C = sv(t + 2);
                    dp += wM[l] * (q == 0 ? B * C : (q == 1 ? A * C : A * B));
                } else {
                    const float C = sv(t + 2), D = sv(t + 3);
                    if (q == 0) dp += wM[l] * B * C * D + wAB[l] * B + wAC[l] * C + wAD[l] * D;
                    if (q == 1) dp += wM[l] * A * C * D + wAB[l] * A + wBD[l] * D + wBC[l] * C;
                    if (q == 2) dp += wM[l] * A * B * D + wCD[l] * D + wAC[l] * A + wBC[l] * B;
                    if (q == 3) dp += wM[l] * A * B * C + wCD[l] * C + wBD[l] * B + wAD[l] * A;
                }
            }
            Gd[(long long)p * V] = gp + dp;
            dm += dp;
        }
    }
    const float invT = 1.f / (float)T;
    const float scale = iw ? IW : 1.f;
    for (int t = 0; t < T; ++t) {
        const float rv = r[(long long)t * V], Iv = I[(long long)t * V];
        float gr = g * (scale * (Gd[(long long)t * V] - dm * invT) + (iw ? out_raw * Iv * invT : 0.f));
        const float gi = iw ? g * out_raw * rv * invT : 0.f;
        if (renorm) gr *= 0.5f;
        if (poscon && !(rv > 0.f)) gr = 0.f;
        Gd[(long long)t * V] = gr;
        S[(long long)t * V] = Iv > 0.f ? gi : 0.f;
    }
}

__global__ void temporal_adjoint_kernel(const BlockDev* __restrict__ blocks, const float* __restrict__ rad,
                                        const float* __restrict__ inten, const float* __restrict__ gmap, int T,
                                        int method, int itc, int order, int iw, int renorm, int poscon,
                                        float* __restrict__ gS, float* __restrict__ gI, long long nmap,
                                        unsigned long long* err) {
    const BlockDev& B = blocks[0];
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= B.vox) return;
    const long long V = B.vox;
    const long long nx = B.nreg[0], ny = B.nreg[1];
    const long long x = v % nx, y = (v / nx) % ny, z = v / (nx * ny);
    const long long gidx = B.out_offset + x * B.out_stride[0] + y * B.out_stride[1] + z * B.out_stride[2];
    if (!in_range(gidx, nmap, err, 5)) return;
    const float g = gmap[gidx];
    const float* r = rad + v;
    const float* I = inten + v;
    // first pass: sums
    KSum ms, iws;
    bool finite = isfinite(g);
    for (int t = 0; t < T; ++t) {
        const float rv = r[t * V];
        finite = finite && isfinite(rv);
        ms.add(rv);
        iws.add(rv * I[t * V]);
    }
    if (!finite) {
        for (int t = 0; t < T; ++t) {
            gS[t * V + v] = 0.f;
            gI[t * V + v] = 0.f;
        }
        return;
    }
    const float invT = 1.f / (float)T;
    if (method == 0 || method == 2) {
        // TRM (kernel.cu:332-366): the first argmax of the seeded maximum carries
        // the derivative. TRPPM (kernel.cu:372-419): d/dr_t of ((sum r+)^2 +
        // sum r+^2) / 2 / count is (sum r+ + r_t) / count where r_t > 0.
        int arg = -1;
        float mip = 0.f;
        KSum s1, s2, si;
        for (int t = 0; t < T; ++t) {
            const float rv = r[t * V], Iv = I[t * V];
            if (method == 0) {
                const float val = iw ? rv * Iv : rv;
                if (val > mip) {
                    mip = val;
                    arg = t;
                }
            } else {
                const float rp = fmaxf(rv, 0.f);
                s1.add(rp);
                s2.add(rp * rp);
                si.add(Iv);
            }
        }
        const float count = fmaxf(0.5f * (float)T * (float)(T + 1), 1.f);
        const float scale = iw ? si.s * invT : 1.f;
        const float pps = 0.5f * (s1.s * s1.s + s2.s) / count;
        for (int t = 0; t < T; ++t) {
            const float rv = r[t * V], Iv = I[t * V];
            float gr = 0.f, gi = 0.f;
            if (method == 0) {
                if (t == arg) {
                    gr = g * (iw ? Iv : 1.f);
                    gi = iw ? g * rv : 0.f;
                }
            } else {
                gr = rv > 0.f ? g * (s1.s + rv) / count * scale : 0.f;
                gi = iw ? g * pps * invT : 0.f;
            }
            if (renorm) gr *= 0.5f;
            if (poscon && !(rv > 0.f)) gr = 0.f;
            gS[t * V + v] = gr;
            gI[t * V + v] = Iv > 0.f ? gi : 0.f;
        }
        return;
    }
    if (method == 3 && itc == 1) {
        trac_itc1_adjoint(r, I, V, T, order, iw, renorm, poscon, g, ms.s * invT, iws.s * invT, gS + v, gI + v);
        return;
    }
    const float m = ms.s * invT;
    const float IW = iws.s * invT;
    const float scale_iw = iw ? IW : 1.f;
    float C = 0.f, AB = 0.f, CD = 0.f, AC = 0.f, BD = 0.f, AD = 0.f, BC = 0.f;
    // sum over s of dC/da_s, in closed form from window sums of the same pass:
    // order 2: S0 + S1; order 3: P12 + P02 + P01; order 4: the four triple sums
    // minus each lag's three single-sum x pair-sum terms
    float sumd = 0.f;
    const int N = T - order;
    if (method == 3) {
        KSum c1, s4, ab, cd, ac, bd, ad, bc, s0, s1, s2, s3, p012, p013, p023, p123;
        for (int t = 0; t < N; ++t) {
            const float A = r[t * V] - m, Bv = r[(t + 1) * V] - m;
            s0.add(A);
            s1.add(Bv);
            if (order == 2) c1.add(A * Bv);
            if (order >= 3) {
                const float Cv = r[(t + 2) * V] - m;
                s2.add(Cv);
                if (order == 3) {
                    c1.add(A * Bv * Cv);
                    ab.add(A * Bv);
                    ac.add(A * Cv);
                    bc.add(Bv * Cv);
                }
                if (order == 4) {
                    const float Dv = r[(t + 3) * V] - m;
                    s3.add(Dv);
                    s4.add(A * Bv * Cv * Dv);
                    ab.add(A * Bv);
                    cd.add(Cv * Dv);
                    ac.add(A * Cv);
                    bd.add(Bv * Dv);
                    ad.add(A * Dv);
                    bc.add(Bv * Cv);
                    p012.add(A * Bv * Cv);
                    p013.add(A * Bv * Dv);
                    p023.add(A * Cv * Dv);
                    p123.add(Bv * Cv * Dv);
                }
            }
        }
        C = c1.s;
        AB = ab.s, CD = cd.s, AC = ac.s, BD = bd.s, AD = ad.s, BC = bc.s;
        if (order == 4) C = s4.s - AB * CD - AC * BD - AD * BC;
        if (order == 2) {
            sumd = s0.s + s1.s;
        } else if (order == 3) {
            sumd = BC + AC + AB;
        } else {
            sumd = (p123.s + p023.s + p013.s + p012.s) - (s1.s * CD + s2.s * BD + s3.s * BC) -
                   (s0.s * CD + s3.s * AC + s2.s * AD) - (s3.s * AB + s0.s * BD + s1.s * AD) -
                   (s2.s * AB + s1.s * AC + s0.s * BC);
        }
    }
    // dC/da_s for every s, then centring (dC/dr_t = dC/da_t - mean_s dC/da_s)
    auto dCda = [&](int s) -> float {
        float d = 0.f;
        auto a = [&](int t) -> float { return (t >= 0 && t < T) ? r[t * V] - m : 0.f; };
        for (int l = 0; l < order; ++l) {
            const int t0 = s - l;  // the product starting at t0 contains a_s at lag l
            if (t0 < 0 || t0 >= N) continue;
            if (order == 2) d += a(t0 + 1 - l);
            else if (order == 3) {
                float p = 1.f;
                for (int q = 0; q < 3; ++q)
                    if (q != l) p *= a(t0 + q);
                d += p;
            } else {
                const float A = a(t0), Bv = a(t0 + 1), Cv = a(t0 + 2), Dv = a(t0 + 3);
                if (l == 0) d += Bv * Cv * Dv - Bv * CD - Cv * BD - Dv * BC;
                if (l == 1) d += A * Cv * Dv - A * CD - Dv * AC - Cv * AD;
                if (l == 2) d += A * Bv * Dv - Dv * AB - A * BD - Bv * AD;
                if (l == 3) d += A * Bv * Cv - Cv * AB - Bv * AC - A * BC;
            }
        }
        return d;
    };
    const float mean_d = sumd * invT;
    const float sgn = C > 0.f ? 1.f : (C < 0.f ? -1.f : 0.f);
    const float aC = fabsf(C);
    for (int t = 0; t < T; ++t) {
        const float rv = r[t * V], Iv = I[t * V];
        float gr, gi;
        if (method == 1) {
            gr = g * (iw ? Iv : 1.f) * invT;
            gi = iw ? g * rv * invT : 0.f;
        } else {
            gr = g * (sgn * invT * scale_iw * (dCda(t) - mean_d) + (iw ? aC * invT * Iv * invT : 0.f));
            gi = iw ? g * aC * invT * rv * invT : 0.f;
        }
        if (renorm) gr *= 0.5f;
        if (poscon && !(rv > 0.f)) gr = 0.f;
        gS[t * V + v] = gr;
        gI[t * V + v] = Iv > 0.f ? gi : 0.f;
    }
}

// ---------------------------------------------------------------------------
// Radiality adjoint.
template <int MR, int XR, int YR, int ZR>
__device__ __forceinline__ float4 gradient_fixed(const float* base, int NIX, int NIY) {
    auto I = [&](int dx, int dy, int dz) { return base[(dz * NIY + dy) * NIX + dx]; };
    float gx = 0.f, gy = 0.f, gz = 0.f;
#pragma unroll
    for (int i = 1; i <= MR; ++i)
#pragma unroll
        for (int j = -YR; j <= YR; ++j)
#pragma unroll
            for (int k = -ZR; k <= ZR; ++k) gx += I(i, j, k) - I(-i, j, k);
#pragma unroll
    for (int j = 1; j <= MR; ++j)
#pragma unroll
        for (int i = -XR; i <= XR; ++i)
#pragma unroll
            for (int k = -ZR; k <= ZR; ++k) gy += I(i, j, k) - I(i, -j, k);
#pragma unroll
    for (int k = 1; k <= MR; ++k)
#pragma unroll
        for (int i = -XR; i <= XR; ++i)
#pragma unroll
            for (int j = -YR; j <= YR; ++j) gz += I(i, j, k) - I(i, j, -k);
    return make_float4(gx, gy, gz, I(0, 0, 0));
}

__device__ __forceinline__ float4 gradient_generic(const float* base, int NIX, int NIY, const int gr[4]) {
    auto I = [&](int dx, int dy, int dz) { return base[(dz * NIY + dy) * NIX + dx]; };
    const int mR = gr[0], xR = gr[1], yR = gr[2], zR = gr[3];
    float gx = 0.f, gy = 0.f, gz = 0.f;
    for (int i = 1; i <= mR; ++i)
        for (int j = -yR; j <= yR; ++j)
            for (int k = -zR; k <= zR; ++k) gx += I(i, j, k) - I(-i, j, k);
    for (int j = 1; j <= mR; ++j)
        for (int i = -xR; i <= xR; ++i)
            for (int k = -zR; k <= zR; ++k) gy += I(i, j, k) - I(i, -j, k);
    for (int k = 1; k <= mR; ++k)
        for (int i = -xR; i <= xR; ++i)
            for (int j = -yR; j <= yR; ++j) gz += I(i, j, k) - I(i, j, -k);
    return make_float4(gx, gy, gz, I(0, 0, 0));
}

// Adjoint tile: 16 fine x columns x kAdjRows fine y rows x FZ fine z rows,
// kAdjThreads threads. Warp k owns x columns 4k..4k+3; lane l of a warp takes
// column 4k + (l >> 3) and the fine rows 2 (l & 7), 2 (l & 7) + 1. All
// threads that touch an x column's U-stage entries sit in one warp, so the
// y-pass transpose needs no shared-memory atomics: the lanes of one column
// whose 5-row windows start on the same row (possible when my > 2) add in
// separate phases, and __syncwarp orders the row updates of lanes whose
// windows overlap. The x pass and its transpose run one (z, y) row of cells
// per thread with a sliding 4-cell window, so every cell has one writer.
//
// Shared-memory row strides are odd in float4 units (17 for the U stage, NU
// rounded up to odd for the cell grid). A 16-byte access is served a quarter
// warp (8 lanes) at a time; 8 lanes walking 8 consecutive rows at one column
// (the row windows of one x column, or one cell row per thread) then hit 8
// different bank groups.
constexpr int kURow = kTileX + 1;

__host__ __device__ __forceinline__ int adj_nup(int NU) { return NU | 1; }
__host__ __device__ __forceinline__ int adj_u_region_f4(int NV, int NW, int NIX, int NIY, int NIZ) {
    const int ustage = 2 * kURow * (NV + 1) * NW;
    const int inp = (NIX * NIY * NIZ + 3) / 4;
    return ustage > inp ? ustage : inp;
}

// Division of 0 <= c < 65536 by d >= 2 with one multiply-high.
struct FastDiv {
    unsigned m;
    __device__ explicit FastDiv(int d) : m(0xffffffffu / (unsigned)d + 1u) {}
    __device__ int operator()(int c) const { return (int)__umulhi((unsigned)c, m); }
};

__device__ __forceinline__ float4 f4fma(float s, float4 a, float4 c) {
    return make_float4(fmaf(s, a.x, c.x), fmaf(s, a.y, c.y), fmaf(s, a.z, c.z), fmaf(s, a.w, c.w));
}
__device__ __forceinline__ float4 f4add(float4 a, float4 b) {
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}

template <int MZ, int CZ>
__global__ void __launch_bounds__(kAdjThreads, 2) radiality_adjoint_kernel(const RadParams p, const AdjParams a) {
    constexpr int FZ = MZ * CZ;
    constexpr int NW = CZ + 4;
    extern __shared__ float4 smem4[];
    const int NU = p.NU, NV = p.NV, NVA = p.NV + 1, NUP = adj_nup(p.NU);
    const int ncell = NUP * NV * NW;
    const int nut = kURow * NVA * NW;
    float4* gt = smem4;                    // forward G + I   [NW][NV][NUP]
    float4* ggt = gt + ncell;              // dL/d(G, I)      [NW][NV][NUP]
    float4* ut = ggt + ncell;              // forward U       [NW][NVA][kURow]; row NV is zero
    float4* gut = ut + nut;                // dL/dU           [NW][NVA][kURow]
    float* inp = reinterpret_cast<float*>(ut);  // input tile, dead once gt is built
    float4* xw4 = ut + adj_u_region_f4(NV, NW, p.NIX, p.NIY, p.NIZ);  // x weights of the group [16]
    int* xub = reinterpret_cast<int*>(xw4 + kTileX);                 // first tap cell of each x column [16]
    float* tab = reinterpret_cast<float*>(xub + kTileX);
    __shared__ unsigned int s_item;

    const int nthr = blockDim.x;
    const int tid = threadIdx.x;
    const int mx = p.mag[0], my = p.mag[1];
    const int lane = tid & 31;
    const int xf = (tid >> 5) * 4 + (lane >> 3);
    const int tr = lane & 7;
    // lanes tr, tr' of one column with tr = tr' mod nph have rows >= my apart,
    // hence different window starts
    const int nph = (my + 1) >> 1;
    const int myph = tr % nph;
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);

    for (int i = tid; i < p.smem_table_words; i += nthr) tab[i] = p.tables[i];
    const float* wx = tab + p.tl.wx;
    const int* offx = reinterpret_cast<const int*>(tab + p.tl.offx);
    const float* wy = tab + p.tl.wy;
    const int* offy = reinterpret_cast<const int*>(tab + p.tl.offy);
    const float* wz = tab + p.tl.wz;
    const int* offz = reinterpret_cast<const int*>(tab + p.tl.offz);
    const float* wzi = tab + p.tl.wzi;
    const int* grp_xval = reinterpret_cast<const int*>(tab + p.tl.grp_xval);
    const int* grp = reinterpret_cast<const int*>(tab + p.tl.grp);
    const int* pair_yval = reinterpret_cast<const int*>(tab + p.tl.pair_yval);
    const int* pair_pt = reinterpret_cast<const int*>(tab + p.tl.pair_pt);
    const int* pt_zval = reinterpret_cast<const int*>(tab + p.tl.pt_zval);
    const float4* pt_vec = reinterpret_cast<const float4*>(tab + p.tl.pt_vec);
    const float2* pair_rot = reinterpret_cast<const float2*>(tab + p.tl.pair_rot);

    const float* in = static_cast<const float*>(p.in);
    const int NIX = p.NIX, NIY = p.NIY, NIZ = p.NIZ, R = p.R;
    const int nin = NIX * NIY * NIZ;
    const FastDiv div_nup(NUP), div_nv(NV), div_nva(NVA), div_nix(NIX), div_niy(NIY), div_nixy(NIX * NIY);

    for (;;) {
        __syncthreads();
        if (tid == 0) s_item = atomicAdd(p.work_counter, 1u);
        __syncthreads();
        const long long item = s_item;
        if (item >= p.nitems) break;
        const int tile_i = (int)(item % p.ntiles);
        const int chunk = (int)(item / p.ntiles);
        const TileDesc td = p.tiles[tile_i];
        const BlockDev& B = p.blocks[td.block];
        const int bw = B.size[0], bh = B.size[1], bd = B.size[2];
        const int X0 = B.lo[0] + td.tx * kTileX;
        const int Y0 = B.lo[1] + td.ty * kAdjRows;
        const int Z0 = B.zbase + td.tz * FZ;
        const int cx0 = floordiv(X0, mx) - 2;
        const int cy0 = floordiv(Y0, my) - 2;
        const int cz0 = Z0 / MZ - 2;
        const int X = X0 + xf;
        const int Ya = Y0 + 2 * tr, Yb = Ya + 1;
        const int yia = floordiv(Ya, my), yra = Ya - yia * my;
        const int yib = floordiv(Yb, my), yrb = Yb - yib * my;
        const bool xin = X < B.hi[0];
        const bool ina = xin && Ya < B.hi[1];
        const bool inb = xin && Yb < B.hi[1];
        const long long V = B.vox;
        const long long va = ((long long)(Ya - B.lo[1])) * B.nreg[0] + (X - B.lo[0]);
        const long long vb = va + B.nreg[0];
        const long long zstride = (long long)B.nreg[0] * B.nreg[1];
        // volumes [t_lo, t_hi) of this launch (t_hi 0: up to T); dL/dS and dL/dI
        // hold rows from volume stack_t0 on
        const int t0 = p.t_lo + chunk * p.t_chunk;
        const int t1 = min(p.t_hi > 0 ? p.t_hi : p.T, t0 + p.t_chunk);
        for (int t = t0; t < t1; ++t) {
            const long long sbase = B.stack_off + (long long)(t - p.stack_t0) * V;
            const long long tbase = (long long)t * p.D * p.H * p.W;
            // forward: input tile, gradient cells; clear the adjoint cells
            for (int r = tid / kTileX; r < NIY * NIZ; r += nthr / kTileX) {
                const int iz = div_niy(r), iy = r - iz * NIY;
                const int by = clampi(cy0 - R + iy, 0, bh - 1);
                const int bz = clampi(cz0 - R + iz, 0, bd - 1);
                const long long rowg = tbase + ((long long)(B.origin[2] + bz) * p.H + (B.origin[1] + by)) * p.W +
                                       B.origin[0];
                for (int ix = tid % kTileX; ix < NIX; ix += kTileX) {
                    const long long gi = rowg + clampi(cx0 - R + ix, 0, bw - 1);
                    inp[r * NIX + ix] = in_range(gi, a.n_in, a.err, 8) ? __ldg(in + gi) : 0.f;
                }
            }
            __syncthreads();
            for (int c = tid; c < ncell; c += nthr) {
                const int row = div_nup(c);
                const int u = c - row * NUP;
                const int w = div_nv(row), v = row - w * NV;
                const int cu = cx0 + u, cv = cy0 + v, cw = cz0 + w;
                float4 g4 = zero4;
                if (u < NU && cu >= 0 && cu < bw && cv >= 0 && cv < bh && cw >= 0 && cw < bd) {
                    const float* base = inp + ((w + R) * NIY + (v + R)) * NIX + (u + R);
                    if (p.grad_mode == 1)
                        g4 = gradient_fixed<1, 1, 1, 1>(base, NIX, NIY);
                    else if (p.grad_mode == 2)
                        g4 = gradient_fixed<1, 0, 0, 0>(base, NIX, NIY);
                    else
                        g4 = gradient_generic(base, NIX, NIY, p.gr);
                }
                gt[c] = g4;
                ggt[c] = zero4;
            }
            // dL/dS of this thread's subvoxels (dL/dI is read in the (0, 0) pair)
            float2 gS[FZ];
#pragma unroll
            for (int z = 0; z < FZ; ++z) {
                const int Z = Z0 + z;
                const bool zin = Z >= B.lo[2] && Z < B.hi[2];
                const long long zo = sbase + (long long)(Z - B.lo[2]) * zstride;
                const bool oka = zin && ina && in_range(zo + va, a.n_stack, a.err, 9);
                const bool okb = zin && inb && in_range(zo + vb, a.n_stack, a.err, 9);
                gS[z].x = oka ? a.gS[zo + va] : 0.f;
                gS[z].y = okb ? a.gS[zo + vb] : 0.f;
            }

            for (int gi_ = 0; gi_ < p.ngroups; ++gi_) {
                __syncthreads();  // gt built / previous group's x transpose done with gut and the x tables
                const int av = grp_xval[gi_];
                if (tid < kTileX) {
                    const int Xc = X0 + tid;
                    const int xic = floordiv(Xc, mx), xrc = Xc - xic * mx;
                    xub[tid] = xic - cx0 - 2 + offx[av * mx + xrc];
                    xw4[tid] = *reinterpret_cast<const float4*>(wx + (av * mx + xrc) * 4);
                }
                for (int e = tid; e < nut; e += nthr) gut[e] = zero4;
                __syncthreads();
                // x pass, one (w, v) row per thread: U[xf] = sum_k wx_xf[k] G[ub(xf) + k];
                // ub steps by 0 or 1 from one column to the next
                for (int row = tid; row < NVA * NW; row += nthr) {
                    const int w = div_nva(row), v = row - w * NVA;
                    float4* dst = ut + row * kURow;
                    if (v >= NV) {
#pragma unroll
                        for (int x = 0; x < kTileX; ++x) dst[x] = zero4;
                        continue;
                    }
                    const float4* src = gt + (w * NV + v) * NUP;
                    int ub = xub[0];
                    float4 c0 = src[ub], c1 = src[ub + 1], c2 = src[ub + 2], c3 = src[ub + 3];
#pragma unroll
                    for (int x = 0; x < kTileX; ++x) {
                        if (x > 0) {
                            const int nb = xub[x];
                            if (nb != ub) {
                                ub = nb;
                                c0 = c1;
                                c1 = c2;
                                c2 = c3;
                                c3 = src[ub + 3];
                            }
                        }
                        const float4 wk = xw4[x];
                        float4 r;
                        r.x = fmaf(wk.w, c3.x, fmaf(wk.z, c2.x, fmaf(wk.y, c1.x, wk.x * c0.x)));
                        r.y = fmaf(wk.w, c3.y, fmaf(wk.z, c2.y, fmaf(wk.y, c1.y, wk.x * c0.y)));
                        r.z = fmaf(wk.w, c3.z, fmaf(wk.z, c2.z, fmaf(wk.y, c1.z, wk.x * c0.z)));
                        r.w = 0.f;
                        dst[x] = r;
                    }
                }
                __syncthreads();
                for (int pi = grp[gi_]; pi < grp[gi_ + 1]; ++pi) {
                    const int b = pair_yval[pi];
                    const int sa = yia - cy0 - 2 + offy[b * my + yra];
                    const int sb = yib - cy0 - 2 + offy[b * my + yrb];
                    const bool sh = sb != sa;  // column b's taps start one row later
                    const float4 wa = *reinterpret_cast<const float4*>(wy + (b * my + yra) * 4);
                    const float4 wb = *reinterpret_cast<const float4*>(wy + (b * my + yrb) * 4);
                    // (column a, column b) weights of rows sa .. sa + 4
                    float2 w2[5];
                    w2[0] = make_float2(wa.x, sh ? 0.f : wb.x);
                    w2[1] = make_float2(wa.y, sh ? wb.x : wb.y);
                    w2[2] = make_float2(wa.z, sh ? wb.y : wb.z);
                    w2[3] = make_float2(wa.w, sh ? wb.z : wb.w);
                    w2[4] = make_float2(0.f, sh ? wb.w : 0.f);
                    const int r0 = sa * kURow + xf;
                    float2 Tx[NW], Ty[NW], Tz[NW];
#pragma unroll
                    for (int w = 0; w < NW; ++w) {
                        const float4* src = ut + w * NVA * kURow + r0;
                        const float4 u0 = src[0], u1 = src[kURow], u2 = src[2 * kURow], u3 = src[3 * kURow],
                                     u4 = src[4 * kURow];
                        Tx[w].x = fmaf(wa.w, u3.x, fmaf(wa.z, u2.x, fmaf(wa.y, u1.x, wa.x * u0.x)));
                        Ty[w].x = fmaf(wa.w, u3.y, fmaf(wa.z, u2.y, fmaf(wa.y, u1.y, wa.x * u0.y)));
                        Tz[w].x = fmaf(wa.w, u3.z, fmaf(wa.z, u2.z, fmaf(wa.y, u1.z, wa.x * u0.z)));
                        Tx[w].y = fmaf(w2[4].y, u4.x, fmaf(w2[3].y, u3.x, fmaf(w2[2].y, u2.x, fmaf(w2[1].y, u1.x, w2[0].y * u0.x))));
                        Ty[w].y = fmaf(w2[4].y, u4.y, fmaf(w2[3].y, u3.y, fmaf(w2[2].y, u2.y, fmaf(w2[1].y, u1.y, w2[0].y * u0.y))));
                        Tz[w].y = fmaf(w2[4].y, u4.z, fmaf(w2[3].y, u3.z, fmaf(w2[2].y, u2.z, fmaf(w2[1].y, u1.z, w2[0].y * u0.z))));
                    }
                    const float2 rot = pair_rot[pi];
                    const float2 ca = dup(rot.x), sb2 = dup(rot.y), nsb = dup(-rot.y);
#pragma unroll
                    for (int w = 0; w < NW; ++w) {
                        const float2 gx = Tx[w], gy = Ty[w];
                        Tx[w] = fma2(gy, sb2, mul2(gx, ca));   // P
                        Ty[w] = fma2(gy, ca, mul2(gx, nsb));   // E
                    }
                    float2 gP[NW], gE[NW], gZ[NW];
#pragma unroll
                    for (int w = 0; w < NW; ++w) gP[w] = gE[w] = gZ[w] = make_float2(0.f, 0.f);
                    for (int qi = pair_pt[pi]; qi < pair_pt[pi + 1]; ++qi) {
                        const float4 pv = pt_vec[qi];
                        const float2 hh = dup(pv.x), cc = dup(pv.y), ncc = dup(-pv.y), nhh = dup(-pv.x);
                        const float wgt2 = pv.z * (-2.0f * pv.w);  // multiplicity / n times 2|u|
                        const float2 nun = dup(pv.w);              // -|u|
                        const int zc = pt_zval[qi];
                        const float* wzc = wz + zc * (MZ * 4);
                        const int offmask = offz[zc];
                        auto zpass = [&](auto OFF, int zr, const float2 (&w4)[4]) {
                            constexpr int o = decltype(OFF)::value;
#pragma unroll
                            for (int zi = 0; zi < CZ; ++zi) {
                                const int z = zi * MZ + zr;
                                float2 gx = mul2(w4[0], Tx[zi + o]);
                                float2 gy = mul2(w4[0], Ty[zi + o]);
                                float2 gz = mul2(w4[0], Tz[zi + o]);
#pragma unroll
                                for (int m = 1; m < 4; ++m) {
                                    gx = fma2(w4[m], Tx[zi + o + m], gx);
                                    gy = fma2(w4[m], Ty[zi + o + m], gy);
                                    gz = fma2(w4[m], Tz[zi + o + m], gz);
                                }
                                // forward quantities (P = gx, E = gy, Z = gz)
                                const float2 dot = fma2(cc, gz, mul2(hh, gx));
                                const float2 cp = fma2(hh, gz, mul2(ncc, gx));
                                const float2 c2 = fma2(cp, cp, mul2(gy, gy));
                                const float2 g2 = fma2(dot, dot, c2);
                                const float2 xx = mul2(c2, g2);
                                // inv = 1/(|g| |g_perp|); where g is parallel to u (c2 = 0) every
                                // product below carries a factor c2, cp or E and vanishes
                                const float2 inv = make_float2(rsqrt_approx(fmaxf(xx.x, 1e-30f)),
                                                               rsqrt_approx(fmaxf(xx.y, 1e-30f)));
                                const float2 sn = mul2(c2, inv);                          // sin
                                const float2 om = fma2(sn, nun, dup(1.0f));               // 1 - Dk/r
                                // -dL/dsin = (dL/dS) (+-w) 2 om |u| (signed weight and 2|u|
                                // folded into one table value)
                                const float2 sw = make_float2(sign_weight(wgt2, dot.x), sign_weight(wgt2, dot.y));
                                const float2 coef = mul2(mul2(sw, om), gS[z]);
                                // d sin / d(P, E, Z) = g_perp/(|g||g_perp|) - sin g/|g|^2 with
                                // g_perp = (-c cp, E, h cp) and 1/(|g||g_perp|) = inv, sin/|g|^2
                                // = sin^2 inv; times dL/dsin = -coef:
                                //   dP = k (sin^2 P + c cp), dZ = k (sin^2 Z - h cp),
                                //   dE = k (sin^2 - 1) E,   k = coef inv
                                const float2 k = mul2(coef, inv);
                                const float2 s2 = mul2(sn, sn);
                                const float2 dP = mul2(k, fma2(s2, gx, mul2(cc, cp)));
                                const float2 dZ = mul2(k, fma2(s2, gz, mul2(nhh, cp)));
                                const float2 dE = mul2(fma2(s2, k, make_float2(-k.x, -k.y)), gy);
#pragma unroll
                                for (int m = 0; m < 4; ++m) {
                                    gP[zi + o + m] = fma2(w4[m], dP, gP[zi + o + m]);
                                    gE[zi + o + m] = fma2(w4[m], dE, gE[zi + o + m]);
                                    gZ[zi + o + m] = fma2(w4[m], dZ, gZ[zi + o + m]);
                                }
                            }
                        };
#pragma unroll
                        for (int zr = 0; zr < MZ; ++zr) {
                            float2 w4[4];
#pragma unroll
                            for (int m = 0; m < 4; ++m) w4[m] = dup(wzc[zr * 4 + m]);
                            if ((offmask >> zr) & 1)
                                zpass(IntC<1>{}, zr, w4);
                            else
                                zpass(IntC<0>{}, zr, w4);
                        }
                    }
                    // back to (x, y): X = ca P - sb E, Y = sb P + ca E
#pragma unroll
                    for (int w = 0; w < NW; ++w) {
                        const float2 P = gP[w], E = gE[w];
                        gP[w] = fma2(E, nsb, mul2(P, ca));
                        gE[w] = fma2(E, ca, mul2(P, sb2));
                    }
                    // intensity at the subvoxel centre rides on the (0, 0) pair: z pass
                    // transpose with rho_z = 0 (5 taps) of dL/dI
                    float2 gW[NW];
#pragma unroll
                    for (int w = 0; w < NW; ++w) gW[w] = make_float2(0.f, 0.f);
                    if (pi == p.zero_pair) {
#pragma unroll
                        for (int z = 0; z < FZ; ++z) {
                            const int Z = Z0 + z;
                            const bool zin = Z >= B.lo[2] && Z < B.hi[2];
                            const long long zo = sbase + (long long)(Z - B.lo[2]) * zstride;
                            const bool oka = zin && ina && in_range(zo + va, a.n_stack, a.err, 9);
                            const bool okb = zin && inb && in_range(zo + vb, a.n_stack, a.err, 9);
                            const float2 gi = make_float2(oka ? a.gI[zo + va] : 0.f, okb ? a.gI[zo + vb] : 0.f);
                            const int zr = z % MZ, zi = z / MZ;
                            const float* qz = wzi + zr * 5;
#pragma unroll
                            for (int m = 0; m < 5; ++m)
                                if (zi + m < NW) gW[zi + m] = fma2(dup(qz[m]), gi, gW[zi + m]);
                        }
                    }
                    // y pass transpose: row sa + m of every z cell gets w2[m] . (column a, column b)
                    for (int ph = 0; ph < nph; ++ph) {
                        const bool act = myph == ph;
#pragma unroll
                        for (int w = 0; w < NW; ++w) {
                            float4* dst = gut + w * NVA * kURow + r0;
                            const float2 xya = make_float2(gP[w].x, gE[w].x), xyb = make_float2(gP[w].y, gE[w].y);
                            const float2 zwa = make_float2(gZ[w].x, gW[w].x), zwb = make_float2(gZ[w].y, gW[w].y);
#pragma unroll
                            for (int m = 0; m < 5; ++m) {
                                if (act) {
                                    float4* d = dst + m * kURow;
                                    const float4 o4 = *d;
                                    float2 xy = make_float2(o4.x, o4.y), zw = make_float2(o4.z, o4.w);
                                    xy = fma2(dup(w2[m].x), xya, xy);
                                    xy = fma2(dup(w2[m].y), xyb, xy);
                                    zw = fma2(dup(w2[m].x), zwa, zw);
                                    zw = fma2(dup(w2[m].y), zwb, zw);
                                    *d = make_float4(xy.x, xy.y, zw.x, zw.y);
                                }
                                if (m < 4) __syncwarp();
                            }
                        }
                        if (nph > 1) __syncwarp();
                    }
                }
                __syncthreads();
                // x pass transpose, one (w, v) row of cells per thread: a 4-cell window
                // slides with ub; a cell leaving the window is final for this group
                for (int row = tid; row < NV * NW; row += nthr) {
                    const int w = div_nv(row), v = row - w * NV;
                    const float4* src = gut + (w * NVA + v) * kURow;
                    float4* dst = ggt + row * NUP;
                    int ub = xub[0];
                    float4 a0 = zero4, a1 = zero4, a2 = zero4, a3 = zero4;
#pragma unroll
                    for (int x = 0; x < kTileX; ++x) {
                        if (x > 0) {
                            const int nb = xub[x];
                            if (nb != ub) {
                                dst[ub] = f4add(dst[ub], a0);
                                a0 = a1;
                                a1 = a2;
                                a2 = a3;
                                a3 = zero4;
                                ub = nb;
                            }
                        }
                        const float4 g = src[x];
                        const float4 wk = xw4[x];
                        a0 = f4fma(wk.x, g, a0);
                        a1 = f4fma(wk.y, g, a1);
                        a2 = f4fma(wk.z, g, a2);
                        a3 = f4fma(wk.w, g, a3);
                    }
                    dst[ub] = f4add(dst[ub], a0);
                    dst[ub + 1] = f4add(dst[ub + 1], a1);
                    dst[ub + 2] = f4add(dst[ub + 2], a2);
                    dst[ub + 3] = f4add(dst[ub + 3], a3);
                }
            }
            __syncthreads();
            // stencil transpose onto the input tile positions, then into dL/dI'. Cells
            // outside the tile grid or the block do not depend on the input.
            for (int i = tid; i < nin; i += nthr) {
                const int iz = div_nixy(i);
                const int rem = i - iz * (NIX * NIY);
                const int iy = div_nix(rem), ix = rem - iy * NIX;
                const int u = ix - R, v = iy - R, w = iz - R;  // cell with the same position
                float acc = 0.f;
                if (p.grad_mode == 1 || p.grad_mode == 2) {
                    // 3 x 3 x 3 neighbourhood with clamped indices and 0/1 masks
                    int cu[3], cv[3], cw[3];
                    float mu[3], mv[3], mw[3];
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        const int uu = u + d - 1, vv = v + d - 1, ww = w + d - 1;
                        mu[d] = (uu >= 0 && uu < NU && cx0 + uu >= 0 && cx0 + uu < bw) ? 1.f : 0.f;
                        mv[d] = (vv >= 0 && vv < NV && cy0 + vv >= 0 && cy0 + vv < bh) ? 1.f : 0.f;
                        mw[d] = (ww >= 0 && ww < NW && cz0 + ww >= 0 && cz0 + ww < bd) ? 1.f : 0.f;
                        cu[d] = clampi(uu, 0, NU - 1);
                        cv[d] = clampi(vv, 0, NV - 1) * NUP;
                        cw[d] = clampi(ww, 0, NW - 1) * (NV * NUP);
                    }
                    auto G = [&](int dx, int dy, int dz) -> float4 { return ggt[cw[dz + 1] + cv[dy + 1] + cu[dx + 1]]; };
                    if (p.grad_mode == 1) {
                        // neighbour d adds -(dx Gx + dy Gy + dz Gz) (ranges 1, 1, 1, 1)
#pragma unroll
                        for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
                            for (int dy = -1; dy <= 1; ++dy) {
                                const float myz = mv[dy + 1] * mw[dz + 1];
#pragma unroll
                                for (int dx = -1; dx <= 1; ++dx) {
                                    const float4 g = G(dx, dy, dz);
                                    float s = 0.f;
                                    if (dx) s = dx < 0 ? s + g.x : s - g.x;
                                    if (dy) s = dy < 0 ? s + g.y : s - g.y;
                                    if (dz) s = dz < 0 ? s + g.z : s - g.z;
                                    if (!dx && !dy && !dz) s = g.w;
                                    acc = fmaf(myz * mu[dx + 1], s, acc);
                                }
                            }
                    } else {
                        // ranges 1, 0, 0, 0: axis neighbours only
                        acc = mu[1] * mv[1] * mw[1] * G(0, 0, 0).w;
                        acc = fmaf(mu[0] * mv[1] * mw[1], G(-1, 0, 0).x, acc);
                        acc = fmaf(-mu[2] * mv[1] * mw[1], G(1, 0, 0).x, acc);
                        acc = fmaf(mu[1] * mv[0] * mw[1], G(0, -1, 0).y, acc);
                        acc = fmaf(-mu[1] * mv[2] * mw[1], G(0, 1, 0).y, acc);
                        acc = fmaf(mu[1] * mv[1] * mw[0], G(0, 0, -1).z, acc);
                        acc = fmaf(-mu[1] * mv[1] * mw[2], G(0, 0, 1).z, acc);
                    }
                } else {
                    const int mR = p.gr[0], xR = p.gr[1], yR = p.gr[2], zR = p.gr[3];
                    auto G = [&](int du, int dv, int dw) -> float4 {
                        const int uu = u + du, vv = v + dv, ww = w + dw;
                        if (uu < 0 || uu >= NU || vv < 0 || vv >= NV || ww < 0 || ww >= NW) return zero4;
                        if (cx0 + uu < 0 || cx0 + uu >= bw || cy0 + vv < 0 || cy0 + vv >= bh || cz0 + ww < 0 ||
                            cz0 + ww >= bd)
                            return zero4;
                        return ggt[(ww * NV + vv) * NUP + uu];
                    };
                    acc = G(0, 0, 0).w;
                    // Gx(c) = sum_{i>0, j, k} I(c + (i, j, k)) - I(c + (-i, j, k))
                    for (int ii = 1; ii <= mR; ++ii)
                        for (int j = -yR; j <= yR; ++j)
                            for (int k = -zR; k <= zR; ++k) acc += G(-ii, -j, -k).x - G(ii, -j, -k).x;
                    for (int jj = 1; jj <= mR; ++jj)
                        for (int ii = -xR; ii <= xR; ++ii)
                            for (int k = -zR; k <= zR; ++k) acc += G(-ii, -jj, -k).y - G(-ii, jj, -k).y;
                    for (int kk = 1; kk <= mR; ++kk)
                        for (int ii = -xR; ii <= xR; ++ii)
                            for (int j = -yR; j <= yR; ++j) acc += G(-ii, -j, -kk).z - G(-ii, -j, kk).z;
                }
                if (acc != 0.f) {
                    const int bx = clampi(cx0 - R + ix, 0, bw - 1);
                    const int by = clampi(cy0 - R + iy, 0, bh - 1);
                    const int bz = clampi(cz0 - R + iz, 0, bd - 1);
                    const long long gidx = tbase + ((long long)(B.origin[2] + bz) * p.H + (B.origin[1] + by)) * p.W +
                                           (B.origin[0] + bx);
                    if (in_range(gidx, a.n_in, a.err, 10)) atomicAdd(a.gin + gidx, acc);
                }
            }
        }
    }
}
template <int MZ>
int launch_adj_mz(const RadParams& p, const AdjParams& a, int grid, size_t smem, cudaStream_t st) {
    constexpr int CZ = cza_for_mag(MZ);
    auto k = radiality_adjoint_kernel<MZ, CZ>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    k<<<grid, kAdjThreads, smem, st>>>(p, a);
    return (int)cudaGetLastError();
}

template <int MZ>
int occ_adj_mz(int threads, size_t smem, int* out) {
    constexpr int CZ = cza_for_mag(MZ);
    auto k = radiality_adjoint_kernel<MZ, CZ>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, k, threads, smem);
}

}  // namespace

size_t radiality_adjoint_smem_bytes(const RadParams& p) {
    const int NW = cza_for_mag(p.mag[2]) + 4;
    size_t b = sizeof(float4) * (2 * (size_t)adj_nup(p.NU) * p.NV * NW +
                                 (size_t)adj_u_region_f4(p.NV, NW, p.NIX, p.NIY, p.NIZ));
    b += sizeof(float4) * kTileX + sizeof(int) * kTileX;  // x weights and first tap cell of each column
    b += sizeof(float) * p.smem_table_words;
    return (b + 15) & ~(size_t)15;
}

int launch_radiality_adjoint(const RadParams& p, const AdjParams& a, int grid, size_t smem, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (p.mag[2]) {
        case 1: return launch_adj_mz<1>(p, a, grid, smem, st);
        case 2: return launch_adj_mz<2>(p, a, grid, smem, st);
        case 3: return launch_adj_mz<3>(p, a, grid, smem, st);
        case 4: return launch_adj_mz<4>(p, a, grid, smem, st);
        case 5: return launch_adj_mz<5>(p, a, grid, smem, st);
        case 6: return launch_adj_mz<6>(p, a, grid, smem, st);
        case 7: return launch_adj_mz<7>(p, a, grid, smem, st);
        case 8: return launch_adj_mz<8>(p, a, grid, smem, st);
    }
    return (int)cudaErrorInvalidValue;
}

int radiality_adjoint_max_ctas_per_sm(const RadParams& p, int* out) {
    const size_t smem = radiality_adjoint_smem_bytes(p);
    const int threads = kAdjThreads;
    switch (p.mag[2]) {
        case 1: return occ_adj_mz<1>(threads, smem, out);
        case 2: return occ_adj_mz<2>(threads, smem, out);
        case 3: return occ_adj_mz<3>(threads, smem, out);
        case 4: return occ_adj_mz<4>(threads, smem, out);
        case 5: return occ_adj_mz<5>(threads, smem, out);
        case 6: return occ_adj_mz<6>(threads, smem, out);
        case 7: return occ_adj_mz<7>(threads, smem, out);
        case 8: return occ_adj_mz<8>(threads, smem, out);
    }
    return (int)cudaErrorInvalidValue;
}

int launch_temporal_adjoint(const BlockDev* blocks, long long vox, const float* rad, const float* inten,
                            const float* gmap, int T, int method, int itc, int order, int iw, int renorm, int poscon,
                            float* gS, float* gI, long long nmap, unsigned long long* err, void* stream) {
    if (vox == 0) return 0;
    const long long grid = (vox + 127) / 128;
    temporal_adjoint_kernel<<<(unsigned)grid, 128, 0, static_cast<cudaStream_t>(stream)>>>(
        blocks, rad, inten, gmap, T, method, itc, order, iw, renorm, poscon, gS, gI, nmap, err);
    return (int)cudaGetLastError();
}

int launch_shift_axis(const float* src, float* dst, int W, int H, int D, int T, int axis, const float* shifts, int mode,
                      unsigned long long* err, void* stream) {
    const long long n = (long long)W * H * D * T;
    const long long grid = std::min<long long>((n + 255) / 256, 152LL * 16);
    shift_axis_kernel<<<(unsigned)grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(src, dst, W, H, D, T, axis,
                                                                                     shifts, mode, err);
    return (int)cudaGetLastError();
}

namespace {
__global__ void d2f_kernel(const double* s, float* d, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = (float)s[i];
}
}  // namespace

int launch_double_to_float(const double* src, float* dst, int n, void* stream) {
    if (n <= 0) return 0;
    d2f_kernel<<<(n + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(src, dst, n);
    return (int)cudaGetLastError();
}

int launch_drift3d(const float* src, float* dst, const float* g, int W, int H, int D, int T, const float* shifts,
                   int mode, double* out, unsigned long long* err, void* stream) {
    (void)err;  // every tap index is clamped into the volume
    const int threads = W >= 256 ? 256 : (W >= 128 ? 128 : (W >= 64 ? 64 : 32));
    dim3 grid((unsigned)std::min<long long>((long long)D * H, std::max(152LL * 16 / std::max(T, 1), 8LL)),
              (unsigned)T);
    if (mode == 0)
        drift3d_kernel<0><<<grid, threads, 0, static_cast<cudaStream_t>(stream)>>>(src, dst, g, W, H, D, shifts, out);
    else
        drift3d_kernel<1><<<grid, threads, 0, static_cast<cudaStream_t>(stream)>>>(src, dst, g, W, H, D, shifts, out);
    return (int)cudaGetLastError();
}

int launch_drift_dot(const float* g, const float* dv, long long nv, int T, int axis, double* out,
                     unsigned long long* err, void* stream) {
    dim3 grid((unsigned)std::min<long long>((nv + 255) / 256, 64), (unsigned)T);
    drift_dot_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(g, dv, nv, axis, out, err);
    return (int)cudaGetLastError();
}

}  // namespace rfba

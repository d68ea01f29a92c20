// Temporal reduction of the radiality stack (sm_103a).
//
// One thread per output subvoxel reduces its radiality series rad[t] and the
// interpolated intensity series I[t] into the map value, with the reference's
// exact semantics:
//   TRM   kernel.cu:332-366  max(0, max_t rad*I)            (IW=0: rad)
//   TRA   kernel.cu:291-327  (1/T) sum_t rad*I              (IW=0: rad)
//   TRPPM kernel.cu:372-419  sum_{t0<=t1} r0+ r1+ / count * mean_t I, computed as
//                            ((sum r+)^2 + sum r+^2) / 2 / (T(T+1)/2): the same
//                            sum with every pair visited once, O(T) instead of O(T^2)
//   TRAC  kernel.cu:423-555  lag-1 cumulants of order 2/3/4 around the mean of
//                            the unweighted series; ITC=1 repeats on the series
//                            binned in place by the order, with the reference's
//                            accumulator carry-over (only AB is reset per level)
//                            and its binning order (entry 0 is cleared before it
//                            is read).
// All temporal sums are FP32 with Kahan compensation. The ITC=1 binning read
// one past the end of an odd-length series (beyond the reference's allocation)
// is defined as 0.
#include <cuda_runtime.h>

#include "srrf_internal.h"

namespace rfba {
namespace {

struct Kahan {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

__global__ void __launch_bounds__(256) temporal_kernel(const TemporalParams p) {
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= p.total_vox) return;
    // block of this voxel
    int lo = 0, hi = p.nblocks - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (p.vox_prefix[mid] <= gid) lo = mid;
        else hi = mid - 1;
    }
    const BlockDev& B = p.blocks[lo];
    const long long v = gid - p.vox_prefix[lo];
    const long long V = B.vox;
    float* rad = p.rad_stack + B.stack_off + v;
    const float* inten = p.int_stack + B.stack_off + v;
    const int T = p.T;
    float result;

    if (p.method == 1) {  // TRA
        Kahan k;
        if (p.iw == 1)
            for (int t = 0; t < T; ++t) k.add(rad[t * V] * inten[t * V]);
        else
            for (int t = 0; t < T; ++t) k.add(rad[t * V]);
        result = k.s / (float)T;
    } else if (p.method == 0) {  // TRM
        float mip = 0.f;
        for (int t = 0; t < T; ++t) mip = fmaxf(p.iw == 1 ? rad[t * V] * inten[t * V] : rad[t * V], mip);
        result = mip;
    } else if (p.method == 2) {  // TRPPM
        Kahan s1, s2, si;
        for (int t = 0; t < T; ++t) {
            const float r = fmaxf(rad[t * V], 0.f);
            s1.add(r);
            s2.add(r * r);
            if (p.iw == 1) si.add(inten[t * V]);
        }
        const float count = fmaxf(0.5f * (float)T * (float)(T + 1), 1.f);
        float pps = (0.5f * (s1.s * s1.s + s2.s)) / count;
        if (p.iw == 1) pps *= si.s / (float)T;
        result = pps;
    } else {  // TRAC
        const int k = p.order;
        Kahan km, kiw;
        for (int t = 0; t < T; ++t) {
            const float r = rad[t * V];
            kiw.add(r * inten[t * V]);
            km.add(r);
        }
        const float mean = km.s / (float)T;
        const float IW = kiw.s / (float)T;
        Kahan AB, ABC, ABCD, CD, AC, BD, AD, BC;
        float out = 0.f;
        if (p.itc != 1) {
            float A = rad[0] - mean;
            float Bv = T > 1 ? rad[V] - mean : 0.f;
            float C = T > 2 ? rad[2 * V] - mean : 0.f;
            for (int t = 0; t < T - k; ++t) {
                const float Dv = (k == 4) ? rad[(t + 3) * V] - mean : 0.f;
                AB.add(A * Bv);
                if (k == 3) ABC.add(A * Bv * C);
                if (k == 4) {
                    ABCD.add(A * Bv * C * Dv);
                    CD.add(C * Dv);
                    AC.add(A * C);
                    BD.add(Bv * Dv);
                    AD.add(A * Dv);
                    BC.add(Bv * C);
                }
                A = Bv;
                Bv = C;
                C = (k == 4) ? Dv : ((t + 3 < T) ? rad[(t + 3) * V] - mean : 0.f);
            }
            if (k == 3) out = fabsf(ABC.s) / (float)T;
            else if (k == 4) out = fabsf(ABCD.s - AB.s * CD.s - AC.s * BD.s - AD.s * BC.s) / (float)T;
            else out = fabsf(AB.s) / (float)T;
        } else {
            int nB = T;
            while (nB > k) {
                AB = Kahan();
                for (int t = 0; t < nB - k; ++t) {
                    const int tBin = t * k;
                    const float A = rad[t * V] - mean;
                    const float Bv = rad[(t + 1) * V] - mean;
                    AB.add(A * Bv);
                    if (k == 3) {
                        const float C = rad[(t + 2) * V] - mean;
                        ABC.add(A * Bv * C);
                    }
                    if (k == 4) {
                        const float C = rad[(t + 2) * V] - mean;
                        const float Dv = rad[(t + 3) * V] - mean;
                        ABCD.add(A * Bv * C * Dv);
                        CD.add(C * Dv);
                        AC.add(A * C);
                        BD.add(Bv * Dv);
                        AD.add(A * Dv);
                        BC.add(Bv * C);
                    }
                    float nv = 0.f;
                    if (tBin < nB) {
                        // entry t is cleared before the bin reads it (t = 0 reads itself
                        // as 0); a read past the end of the series at level 0 is 0
                        for (int j = 0; j < k; ++j) {
                            const int src = tBin + j;
                            const float rv = (src == t || src >= T) ? 0.f : rad[(long long)src * V];
                            nv += rv / (float)k;
                        }
                    }
                    rad[t * V] = nv;
                }
                if (k == 3) out += fabsf(ABC.s) / (float)nB;
                else if (k == 4) out += fabsf(ABCD.s - AB.s * CD.s - AC.s * BD.s - AD.s * BC.s) / (float)nB;
                else out += fabsf(AB.s) / (float)nB;
                nB = nB / k;
            }
        }
        if (p.iw == 1) out = IW * out;
        result = out;
    }

    // output position
    const long long nx = B.nreg[0], ny = B.nreg[1];
    long long x, y, z;
    if (v < 0x7fffffffLL) {
        // 32-bit division: a 64-bit one is a long integer sequence per thread
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

int launch_temporal(const TemporalParams& p, void* stream) {
    if (p.total_vox == 0) return 0;
    const long long grid = (p.total_vox + 255) / 256;
    temporal_kernel<<<(unsigned)grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(p);
    return (int)cudaGetLastError();
}

}  // namespace rfba

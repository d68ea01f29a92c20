// CPU oracle for the 3D SRRF radiality path of RFBA's GradientCalc library.
//
// TEST INFRASTRUCTURE ONLY. This file restates the reference algorithm on the
// host so that the CUDA path can be checked against it. Only tests/, the smoke
// check and the CPU-baseline leg of bench.py load it; the product library never
// links or calls it.
//
// Two instantiations:
//   * double: the FP64 oracle. Every value is computed in double from the
//     reference's float inputs (input voxels and the float ring table).
//     The one discrete decision that cannot be taken in double without changing
//     the reference's result is the interpolation window test ("return 0 when
//     x/mag is outside [1.5, dim-1.5]", kernel.cu:146 and :264): it decides
//     whether a subvoxel becomes NaN, so it is taken exactly as the reference
//     takes it, in float ((float)X + 0.5f + ring, then / (float)mag).
//   * float: a literal FP32 port of the reference device code, operation for
//     operation (same association order, absolute magnified coordinates, all n^2
//     ring samples, Catmull-Rom weights recomputed per tap). It reproduces the
//     reference compiled as host code bit for bit (checked in the tests) and is
//     the timed CPU baseline.
//
// Reference map (paths inside the RFBA project):
//   buildRing                 RFBA Main/GradientCalc/kernel.cu:23-33
//   gradKernel                kernel.cu:44-125
//   cubic                     kernel.cu:128-138
//   interpolateG              kernel.cu:141-169
//   _calculateDk              kernel.cu:174-183
//   calculateRadiality        kernel.cu:186-253
//   interpolateIntensity      kernel.cu:257-287
//   calculateAVE  (TRA)       kernel.cu:291-327
//   calculateMIP  (TRM)       kernel.cu:332-366
//   calculatePairwiseProductSum (TRPPM) kernel.cu:372-419
//   calculateACRF (TRAC)      kernel.cu:423-555
//   SRRFGradientCalcGPU       kernel.cu:560-657
//   getSplitCount/doSplit/doPutback/doSRRFGradientCalc  GradientCalc.cpp:47-163
//
// Generalisation kept from the extended interface: one magnification per axis
// (the reference has a single integer Magnification; with equal factors the
// arithmetic is the reference's).
//
// Out-of-range reads of the reference are defined here as follows:
//   * the tap u = dim read at q = dim - 1.5 (weight exactly 0) reads the
//     clamped edge voxel instead of the next row;
//   * the TRAC binning read past the end of an odd-length series at level 0
//     (kernel.cu:535 with tBin + _t == T) reads 0.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>

extern "C" {
typedef struct oconf {
    float ring_radius;
    int mag[3];
    int axes_in_ring;
    int main_range, x_range, y_range, z_range;
    int method, itc, trac_order;
    int remove_con, renormalize, gradient_smooth, intensity_w;
    int block_size[3];
} oconf;
}

namespace {

// kernel.cu:17 and :23-33: float angle step, float sin/cos, (r*sin)*cos order.
void build_ring(float r, int n, float* x, float* y, float* z) {
    const float PI_F = 3.141592654f;
    float step = (PI_F * 2.0f) / (float)n;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            int idx = i * n + j;
            x[idx] = r * std::sin(step * (float)i) * std::cos(step * (float)j);
            y[idx] = r * std::sin(step * (float)i) * std::sin(step * (float)j);
            z[idx] = r * std::cos(step * (float)i);
        }
}

template <class T>
inline T cubic(T xx) {  // kernel.cu:128-138
    const T a = T(0.5);
    T x = xx;
    if (x < T(0)) x = -x;
    T z = T(0);
    if (x < T(1))
        z = x * x * (x * (-a + T(2)) + (a - T(3))) + T(1);
    else if (x < T(2))
        z = -a * x * x * x + T(5) * a * x * x - T(8) * a * x + T(4) * a;
    return z;
}

// The reference's window test, always in float (kernel.cu:143-147, :260-265).
inline bool window_ok(float x0f, int mag, int dim) {
    float q = x0f / (float)mag;
    return !(q < 1.5f || q > (float)dim - 1.5f);
}

inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// A block of the input (all time points) and a coarse sub-box of it on which
// the gradient is evaluated. Arrays are [t][z][y][x] over the sub-box.
template <class T>
struct Field {
    int dim[3];      // block dims (coarse)
    int c0[3], c1[3];  // sub-box [c0, c1)
    int n[3];
    int nt;
    std::vector<T> g[3];
    std::vector<T> img;  // input on the sub-box (for intensity interpolation)
    size_t idx(int x, int y, int z, int t) const {
        return (((size_t)t * n[2] + (z - c0[2])) * n[1] + (y - c0[1])) * n[0] + (x - c0[0]);
    }
};

// gradKernel (kernel.cu:44-125) on the sub-box, reading the block input with
// clamp-to-edge of the block.
template <class T, class Tin>
void gradient(const Tin* in, const int dims[4], const oconf& c, Field<T>& F) {
    const int w = dims[0], h = dims[1], d = dims[2];
    auto I = [&](int x, int y, int z, int t) -> T {
        return (T)in[(((size_t)t * d + z) * h + y) * w + x];
    };
    const size_t tot = (size_t)F.n[0] * F.n[1] * F.n[2] * F.nt;
    for (int k = 0; k < 3; ++k) F.g[k].assign(tot, T(0));
    F.img.assign(tot, T(0));
    const int mR = c.main_range, xR = c.x_range, yR = c.y_range, zR = c.z_range;
#pragma omp parallel for collapse(2) schedule(static)
    for (int t = 0; t < F.nt; ++t)
        for (int z = F.c0[2]; z < F.c1[2]; ++z)
            for (int y = F.c0[1]; y < F.c1[1]; ++y)
                for (int x = F.c0[0]; x < F.c1[0]; ++x) {
                    size_t o = F.idx(x, y, z, t);
                    F.img[o] = I(x, y, z, t);
                    if (c.gradient_smooth == 0) {
                        int x0 = std::max(x - 1, 0), x1 = std::min(x + 1, w - 1);
                        int y0 = std::max(y - 1, 0), y1 = std::min(y + 1, h - 1);
                        int z0 = std::max(z - 1, 0), z1 = std::min(z + 1, d - 1);
                        F.g[0][o] = -I(x0, y, z, t) + I(x1, y, z, t);
                        F.g[1][o] = -I(x, y0, z, t) + I(x, y1, z, t);
                        F.g[2][o] = -I(x, y, z0, t) + I(x, y, z1, t);
                        continue;
                    }
                    T v = 0;
                    for (int i = -mR; i <= mR; ++i)
                        for (int j = -yR; j <= yR; ++j)
                            for (int k = -zR; k <= zR; ++k) {
                                T p = I(clampi(x + i, 0, w - 1), clampi(y + j, 0, h - 1), clampi(z + k, 0, d - 1), t);
                                if (i < 0) v -= p;
                                else if (i > 0) v += p;
                            }
                    F.g[0][o] = v;
                    v = 0;
                    for (int j = -mR; j <= mR; ++j)
                        for (int i = -xR; i <= xR; ++i)
                            for (int k = -zR; k <= zR; ++k) {
                                T p = I(clampi(x + i, 0, w - 1), clampi(y + j, 0, h - 1), clampi(z + k, 0, d - 1), t);
                                if (j < 0) v -= p;
                                else if (j > 0) v += p;
                            }
                    F.g[1][o] = v;
                    v = 0;
                    for (int k = -mR; k <= mR; ++k)
                        for (int i = -xR; i <= xR; ++i)
                            for (int j = -yR; j <= yR; ++j) {
                                T p = I(clampi(x + i, 0, w - 1), clampi(y + j, 0, h - 1), clampi(z + k, 0, d - 1), t);
                                if (k < 0) v -= p;
                                else if (k > 0) v += p;
                            }
                    F.g[2][o] = v;
                }
}

// interpolateG / interpolateIntensity body (kernel.cu:149-168, :266-285) for a
// position already divided by the magnification. Tap indices are clamped to the
// block (see the header note on the u = dim tap).
template <class T>
T interp(const Field<T>& F, const std::vector<T>& A, T x, T y, T z, int t) {
    int u0 = (int)std::floor(x - T(0.5));
    int v0 = (int)std::floor(y - T(0.5));
    int w0 = (int)std::floor(z - T(0.5));
    T s = T(0);
    for (int k = 0; k <= 3; ++k) {
        int w = w0 - 1 + k;
        T q = T(0);
        for (int j = 0; j <= 3; ++j) {
            int v = v0 - 1 + j;
            T p = T(0);
            for (int i = 0; i <= 3; ++i) {
                int u = u0 - 1 + i;
                int uc = clampi(u, F.c0[0], F.c1[0] - 1);
                int vc = clampi(v, F.c0[1], F.c1[1] - 1);
                int wc = clampi(w, F.c0[2], F.c1[2] - 1);
                p = p + A[F.idx(uc, vc, wc, t)] * cubic<T>(x - (T(u) + T(0.5)));
            }
            q = q + p * cubic<T>(y - (T(v) + T(0.5)));
        }
        s = s + q * cubic<T>(z - (T(w) + T(0.5)));
    }
    return s;
}

struct Ring {
    int n = 0;  // points per angle (2 * AxesinRing)
    std::vector<float> x, y, z;
};

// calculateRadiality (kernel.cu:186-253) for one subvoxel and one time point.
template <class T>
T radiality(const Field<T>& F, const Ring& R, const oconf& c, int X, int Y, int Z, int t) {
    const int mx = c.mag[0], my = c.mag[1], mz = c.mag[2];
    const T r = (T)c.ring_radius;
    const T Xc = T(X) + T(0.5), Yc = T(Y) + T(0.5), Zc = T(Z) + T(0.5);
    const float Xcf = (float)X + 0.5f, Ycf = (float)Y + 0.5f, Zcf = (float)Z + 0.5f;
    T S = T(0);
    const int n = R.n;
    for (int i1 = 0; i1 < n; ++i1)
        for (int i2 = 0; i2 < n; ++i2) {
            const int id = i1 * n + i2;
            const T rx = (T)R.x[id], ry = (T)R.y[id], rz = (T)R.z[id];
            const T x0 = Xc + rx, y0 = Yc + ry, z0 = Zc + rz;
            T Gx = 0, Gy = 0, Gz = 0;
            const bool ok = window_ok(Xcf + R.x[id], mx, F.dim[0]) && window_ok(Ycf + R.y[id], my, F.dim[1]) &&
                            window_ok(Zcf + R.z[id], mz, F.dim[2]);
            if (ok) {
                const T qx = x0 / T(mx), qy = y0 / T(my), qz = z0 / T(mz);
                Gx = interp(F, F.g[0], qx, qy, qz, t);
                Gy = interp(F, F.g[1], qx, qy, qz, t);
                Gz = interp(F, F.g[2], qx, qy, qz, t);
            }
            const T GMag = std::sqrt(Gx * Gx + Gy * Gy + Gz * Gz);
            const T GdotR = (Gx * rx + Gy * ry + Gz * rz) / (GMag * r);
            const bool div = (GdotR > 0) || (GdotR != GdotR);
            // _calculateDk (kernel.cu:174-183)
            const T tt = (Gx * (x0 - Xc) + Gy * (y0 - Yc) + Gz * (z0 - Zc)) / (GMag * GMag);
            const T xc = Gx * tt + Xc, yc = Gy * tt + Yc, zc = Gz * tt + Zc;
            const T dk = std::sqrt((x0 - xc) * (x0 - xc) + (y0 - yc) * (y0 - yc) + (z0 - zc) * (z0 - zc));
            T D = T(1) - dk / r;
            D = D * D;
            if (div) S -= D;
            else S += D;
        }
    S = S / T(n);
    if (c.renormalize == 1) S = T(0.5) + (S / T(2));
    if (c.remove_con == 1) S = std::fmax(S, T(0));
    return S;
}

// interpolateIntensity (kernel.cu:257-287) at the subvoxel centre.
template <class T>
T intensity(const Field<T>& F, const oconf& c, int X, int Y, int Z, int t) {
    const float xf = (float)X + 0.5f, yf = (float)Y + 0.5f, zf = (float)Z + 0.5f;
    if (!(window_ok(xf, c.mag[0], F.dim[0]) && window_ok(yf, c.mag[1], F.dim[1]) && window_ok(zf, c.mag[2], F.dim[2])))
        return T(0);
    const T qx = (T(X) + T(0.5)) / T(c.mag[0]);
    const T qy = (T(Y) + T(0.5)) / T(c.mag[1]);
    const T qz = (T(Z) + T(0.5)) / T(c.mag[2]);
    T s = interp(F, F.img, qx, qy, qz, t);
    return std::fmax(s, T(0));
}

// Temporal reductions for one subvoxel. rad has room for nt + 4 entries; the
// entries past nt are 0 (TRAC binning may read one of them).
template <class T>
T temporal(const oconf& c, T* rad, const T* inten, int nt) {
    const int IWf = c.intensity_w;
    if (c.method == 1) {  // calculateAVE, kernel.cu:291-327
        T mean = 0;
        if (IWf == 1)
            for (int t = 0; t < nt; ++t) mean += rad[t] * inten[t];
        else
            for (int t = 0; t < nt; ++t) mean += rad[t];
        return mean / T(nt);
    }
    if (c.method == 0) {  // calculateMIP, kernel.cu:332-366
        T mip = 0;
        for (int t = 0; t < nt; ++t) mip = std::fmax(IWf == 1 ? rad[t] * inten[t] : rad[t], mip);
        return mip;
    }
    if (c.method == 2) {  // calculatePairwiseProductSum, kernel.cu:372-419
        T pps = 0;
        long long counter = 0;
        for (int t0 = 0; t0 < nt; ++t0) {
            T r0 = std::fmax(rad[t0], T(0));
            if (r0 > 0) {
                for (int t1 = t0; t1 < nt; ++t1) {
                    T r1 = std::fmax(rad[t1], T(0));
                    pps += r0 * r1;
                    counter++;
                }
            } else
                counter += nt - t0;
        }
        pps /= std::fmax((T)counter, T(1));
        if (IWf == 1) {
            T iw = 0;
            for (int t = 0; t < nt; ++t) iw += inten[t] / T(nt);
            pps *= iw;
        }
        return pps;
    }
    // calculateACRF, kernel.cu:423-555
    const int order = c.trac_order;
    T mean = 0, IW = 0;
    for (int t = 0; t < nt; ++t) {
        IW += rad[t] * inten[t];
        mean += rad[t];
    }
    mean = mean / T(nt);
    IW = IW / T(nt);
    T out = 0;
    T ABCD = 0, ABC = 0, AB = 0, CD = 0, AC = 0, BD = 0, AD = 0, BC = 0;
    if (c.itc != 1) {
        for (int t = 0; t < nt - order; ++t) {
            AB += (rad[t] - mean) * (rad[t + 1] - mean);
            if (order == 3) ABC += (rad[t] - mean) * (rad[t + 1] - mean) * (rad[t + 2] - mean);
            if (order == 4) {
                T A = rad[t] - mean, B = rad[t + 1] - mean, C = rad[t + 2] - mean, D = rad[t + 3] - mean;
                ABCD += A * B * C * D;
                CD += C * D;
                AC += A * C;
                BD += B * D;
                AD += A * D;
                BC += B * C;
            }
        }
        if (order == 3) out = std::fabs(ABC) / T(nt);
        else if (order == 4) out = std::fabs(ABCD - AB * CD - AC * BD - AD * BC) / T(nt);
        else out = std::fabs(AB) / T(nt);
    } else {
        int nB = nt;
        while (nB > order) {
            AB = 0;
            for (int t = 0; t < nB - order; ++t) {
                int tBin = t * order;
                AB += (rad[t] - mean) * (rad[t + 1] - mean);
                if (order == 3) ABC += (rad[t] - mean) * (rad[t + 1] - mean) * (rad[t + 2] - mean);
                if (order == 4) {
                    T A = rad[t] - mean, B = rad[t + 1] - mean, C = rad[t + 2] - mean, D = rad[t + 3] - mean;
                    ABCD += A * B * C * D;
                    CD += C * D;
                    AC += A * C;
                    BD += B * D;
                    AD += A * D;
                    BC += B * C;
                }
                rad[t] = 0;
                if (tBin < nB)
                    for (int j = 0; j < order; ++j) rad[t] += rad[tBin + j] / T(order);
            }
            if (order == 3) out += std::fabs(ABC) / T(nB);
            else if (order == 4) out += std::fabs(ABCD - AB * CD - AC * BD - AD * BC) / T(nB);
            else out += std::fabs(AB) / T(nB);
            nB = nB / order;
        }
    }
    if (IWf == 1) out = IW * out;
    return out;
}

// One independent block: input dims[4] = {w,h,d,T} with layout [t][z][y][x];
// computes the magnified map on the fine region [lo, hi) (block-local fine
// coordinates), out is [z][y][x] over that region. Optional stacks receive the
// per-time radiality and interpolated intensity, [t][z][y][x] over the region.
template <class T>
void srrf_region(const float* in, const int dims[4], const oconf& c, const int lo[3], const int hi[3], T* out,
                 T* rad_stack, T* int_stack) {
    Ring R;
    R.n = 2 * c.axes_in_ring;
    R.x.resize(R.n * R.n);
    R.y.resize(R.n * R.n);
    R.z.resize(R.n * R.n);
    build_ring(c.ring_radius, R.n, R.x.data(), R.y.data(), R.z.data());
    float rmax[3] = {0, 0, 0};
    for (int i = 0; i < R.n * R.n; ++i) {
        rmax[0] = std::max(rmax[0], std::fabs(R.x[i]));
        rmax[1] = std::max(rmax[1], std::fabs(R.y[i]));
        rmax[2] = std::max(rmax[2], std::fabs(R.z[i]));
    }
    Field<T> F;
    F.nt = dims[3];
    for (int a = 0; a < 3; ++a) {
        F.dim[a] = dims[a];
        const double m = c.mag[a];
        int a0 = (int)std::floor((lo[a] + 0.5 - rmax[a]) / m - 0.5) - 2;
        int a1 = (int)std::floor((hi[a] - 1 + 0.5 + rmax[a]) / m - 0.5) + 3;
        F.c0[a] = std::max(a0, 0);
        F.c1[a] = std::min(a1 + 1, dims[a]);
        if (F.c1[a] <= F.c0[a]) F.c1[a] = F.c0[a] + 1;
        F.n[a] = F.c1[a] - F.c0[a];
    }
    gradient<T>(in, dims, c, F);
    const int nx = hi[0] - lo[0], ny = hi[1] - lo[1], nz = hi[2] - lo[2];
    const int nt = dims[3];
    const size_t nvox = (size_t)nx * ny * nz;
#pragma omp parallel
    {
        std::vector<T> rad(nt + 8), inten(nt + 8);
#pragma omp for schedule(dynamic, 4)
        for (long long v = 0; v < (long long)nvox; ++v) {
            const int X = lo[0] + (int)(v % nx);
            const int Y = lo[1] + (int)((v / nx) % ny);
            const int Z = lo[2] + (int)(v / ((size_t)nx * ny));
            std::fill(rad.begin(), rad.end(), T(0));
            for (int t = 0; t < nt; ++t) {
                rad[t] = radiality<T>(F, R, c, X, Y, Z, t);
                inten[t] = intensity<T>(F, c, X, Y, Z, t);
                if (rad_stack) rad_stack[(size_t)t * nvox + v] = rad[t];
                if (int_stack) int_stack[(size_t)t * nvox + v] = inten[t];
            }
            out[v] = temporal<T>(c, rad.data(), inten.data(), nt);
        }
    }
}

// GradientCalc.cpp:47-163 with border 2 and the INI block sizes. Regions that
// the reference never writes (the global low border) are left untouched here;
// callers pre-fill the output.
template <class T>
void legacy(const float* in, const int dims[4], const oconf& c, T* out) {
    const int border = 2;
    const int mag = c.mag[0];
    int maxDim[3] = {c.block_size[0], c.block_size[1], c.block_size[2]};
    int splitN[3];
    for (int i = 0; i < 3; ++i) {
        splitN[i] = (dims[i] - 2 * border) / (maxDim[i] - 2 * border);
        if ((dims[i] - 2 * border) % (maxDim[i] - 2 * border) != 0) splitN[i] += 1;
    }
    const int W = dims[0] * mag, H = dims[1] * mag;
    for (int k = 0; k < splitN[2]; ++k)
        for (int j = 0; j < splitN[1]; ++j)
            for (int i = 0; i < splitN[0]; ++i) {
                int pos[3] = {i, j, k}, res[4], start[3];
                for (int a = 0; a < 3; ++a) {
                    res[a] = (pos[a] == splitN[a] - 1) ? dims[a] - (splitN[a] - 1) * (maxDim[a] - 2 * border) : maxDim[a];
                    start[a] = pos[a] == 0 ? 0 : pos[a] * (maxDim[a] - 2 * border);
                }
                res[3] = dims[3];
                std::vector<float> blk((size_t)res[0] * res[1] * res[2] * res[3]);
                for (int t = 0; t < res[3]; ++t)
                    for (int z = 0; z < res[2]; ++z)
                        for (int y = 0; y < res[1]; ++y)
                            for (int x = 0; x < res[0]; ++x)
                                blk[(((size_t)t * res[2] + z) * res[1] + y) * res[0] + x] =
                                    in[(((size_t)t * dims[2] + z + start[2]) * dims[1] + y + start[1]) * dims[0] + x + start[0]];
                const int bm = border * mag;
                int lo[3] = {bm, bm, bm}, hi[3] = {res[0] * mag, res[1] * mag, res[2] * mag};
                if (hi[0] <= lo[0] || hi[1] <= lo[1] || hi[2] <= lo[2]) continue;
                std::vector<T> o((size_t)(hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]));
                oconf cb = c;
                cb.mag[1] = cb.mag[2] = mag;
                srrf_region<T>(blk.data(), res, cb, lo, hi, o.data(), nullptr, nullptr);
                const int nx = hi[0] - lo[0], ny = hi[1] - lo[1];
                for (int z = lo[2]; z < hi[2]; ++z)
                    for (int y = lo[1]; y < hi[1]; ++y)
                        for (int x = lo[0]; x < hi[0]; ++x)
                            out[((size_t)(z + start[2] * mag) * H + y + start[1] * mag) * W + x + start[0] * mag] =
                                o[((size_t)(z - lo[2]) * ny + (y - lo[1])) * nx + (x - lo[0])];
            }
}

// ---------------------------------------------------------------------------
// Differentiable path (FP64): drift shift, forward, and the adjoint of a scalar
// objective L(map) with respect to the input voxels and the per-volume shifts.
// The reference has no derivatives; this is the literal reverse of the forward
// above, sample by sample over all n^2 ring samples and all 64 interpolation
// taps, so it shares no factorisation with the CUDA adjoint.

// d/dx of the Catmull-Rom kernel (a = 0.5).
inline double dcubic(double xx) {
    const double a = 0.5;
    const double x = std::fabs(xx), s = xx < 0 ? -1.0 : 1.0;
    if (x < 1.0) return s * (3.0 * (2.0 - a) * x * x + 2.0 * (a - 3.0) * x);
    if (x < 2.0) return s * (-3.0 * a * x * x + 10.0 * a * x - 8.0 * a);
    return 0.0;
}

// One axis of the drift operator: out[x] = sum_k w(x + d - i_k) in[clamp(i_k)],
// i_k = floor(x + d) - 1 + k, w = cubic (or its derivative). With transpose,
// accumulates the adjoint into in from out.
void shift_axis(const double* src, double* dst, int W, int H, int D, int axis, double d, bool deriv, bool transpose) {
    const int n = axis == 0 ? W : (axis == 1 ? H : D);
    const size_t stride = axis == 0 ? 1 : (axis == 1 ? (size_t)W : (size_t)W * H);
    if (transpose) std::fill(dst, dst + (size_t)W * H * D, 0.0);
    for (int z = 0; z < D; ++z)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const int c = axis == 0 ? x : (axis == 1 ? y : z);
                const size_t line = (size_t)(z * H + y) * W + x - (size_t)c * stride;
                const double pos = c + d;
                const int base = (int)std::floor(pos);
                double acc = 0.0;
                for (int k = -1; k <= 2; ++k) {
                    const int i = std::min(std::max(base + k, 0), n - 1);
                    const double w = deriv ? dcubic(pos - (base + k)) : cubic<double>(pos - (base + k));
                    if (transpose)
                        dst[line + (size_t)i * stride] += w * src[line + (size_t)c * stride];
                    else
                        acc += w * src[line + (size_t)i * stride];
                }
                if (!transpose) dst[line + (size_t)c * stride] = acc;
            }
}

// I'_t = shift along x, then y, then z (axes with deriv_axis use derivative weights).
void shift_volume(const double* in, double* out, int W, int H, int D, const double d[3], int deriv_axis) {
    const size_t n = (size_t)W * H * D;
    std::vector<double> a(in, in + n), b(n);
    for (int ax = 0; ax < 3; ++ax) {
        shift_axis(a.data(), b.data(), W, H, D, ax, d[ax], ax == deriv_axis, false);
        a.swap(b);
    }
    std::copy(a.begin(), a.end(), out);
}

void shift_volume_adjoint(const double* g, double* out, int W, int H, int D, const double d[3]) {
    const size_t n = (size_t)W * H * D;
    std::vector<double> a(g, g + n), b(n);
    for (int ax = 2; ax >= 0; --ax) {
        shift_axis(a.data(), b.data(), W, H, D, ax, d[ax], false, true);
        a.swap(b);
    }
    std::copy(a.begin(), a.end(), out);
}

// Adjoint of TRAC with ITC 1 (kernel.cu:437-555) for one subvoxel. The forward
// bins the series in place level after level (entry t of level l + 1 is the
// mean of entries tk .. tk + k - 1 of level l for t < nB - k, entry 0 reading
// itself as the 0 it was just set to, entries past the series reading 0; the
// other entries keep their values) and accumulates, per level, AB (reset each
// level) and ABC / ABCD, CD, AC, BD, AD, BC (not reset) around the level-0
// mean; out = sum over levels of |C_level| / nB_level, times the intensity
// weight. Every level's series is a linear map of the input series, so the
// adjoint is reverse mode over the levels: the derivative of out with respect
// to each level's partial sums (suffix sums over the levels that see them),
// the sums' derivatives with respect to the level's entries, the transposed
// binning down to level 0, and the mean's share.
static bool temporal_adjoint_itc1(const oconf& c, const double* r, const double* I, int T, double g, double* gr,
                                  double* gi) {
    const int k = c.trac_order;
    const bool iw = c.intensity_w == 1;
    double m = 0, IW = 0;
    for (int t = 0; t < T; ++t) {
        m += r[t];
        IW += r[t] * I[t];
    }
    m /= T;
    IW /= T;
    std::vector<std::vector<double> > states;
    std::vector<int> nbs;
    std::vector<double> Cl, ABl, CDa, ACa, BDa, ADa, BCa;
    std::vector<double> s(T + 4, 0.0);
    for (int t = 0; t < T; ++t) s[t] = r[t];
    double ABC = 0, ABCD = 0, CD = 0, AC = 0, BD = 0, AD = 0, BC = 0, out_raw = 0;
    int nB = T;
    while (nB > k) {
        states.push_back(s);
        nbs.push_back(nB);
        double AB = 0;
        for (int t = 0; t < nB - k; ++t) {
            const double A = s[t] - m, B = s[t + 1] - m;
            AB += A * B;
            if (k == 3) ABC += A * B * (s[t + 2] - m);
            if (k == 4) {
                const double Cc = s[t + 2] - m, Dd = s[t + 3] - m;
                ABCD += A * B * Cc * Dd;
                CD += Cc * Dd;
                AC += A * Cc;
                BD += B * Dd;
                AD += A * Dd;
                BC += B * Cc;
            }
            s[t] = 0;
            if (t * k < nB)
                for (int j = 0; j < k; ++j) s[t] += s[t * k + j] / k;
        }
        const double C = k == 2 ? AB : (k == 3 ? ABC : ABCD - AB * CD - AC * BD - AD * BC);
        Cl.push_back(C);
        ABl.push_back(AB);
        CDa.push_back(CD);
        ACa.push_back(AC);
        BDa.push_back(BD);
        ADa.push_back(AD);
        BCa.push_back(BC);
        out_raw += std::fabs(C) / nB;
        nB = nB / k;
    }
    const int L = (int)Cl.size();
    // d out / d(partial sums of level l)
    std::vector<double> wM(L), wAB(L), wCD(L), wAC(L), wBD(L), wAD(L), wBC(L);
    double ss = 0, scd = 0, sac = 0, sbd = 0, sad = 0, sbc = 0;
    for (int l = L - 1; l >= 0; --l) {
        const double sl = (Cl[l] > 0 ? 1.0 : (Cl[l] < 0 ? -1.0 : 0.0)) / nbs[l];
        ss += sl;
        scd += sl * -ABl[l];
        sac += sl * -BDa[l];
        sbd += sl * -ACa[l];
        sad += sl * -BCa[l];
        sbc += sl * -ADa[l];
        wM[l] = k == 2 ? sl : ss;
        wAB[l] = sl * -CDa[l];
        wCD[l] = scd;
        wAC[l] = sac;
        wBD[l] = sbd;
        wAD[l] = sad;
        wBC[l] = sbc;
    }
    std::vector<double> G(T + 4, 0.0);
    double dm = 0;
    for (int l = L - 1; l >= 0; --l) {
        const std::vector<double>& S = states[l];
        const int nb = nbs[l], N = nb - k;
        std::vector<double> Gn(T + 4, 0.0);
        for (int p = 0; p < T; ++p)
            if (p >= N) Gn[p] = G[p];
        for (int t = 0; t < N; ++t)
            if (t * k < nb)
                for (int j = 0; j < k; ++j) {
                    const int src = t * k + j;
                    if (src != t && src < T) Gn[src] += G[t] / k;
                }
        for (int t = 0; t < N; ++t) {
            const double A = S[t] - m, B = S[t + 1] - m, Cc = S[t + 2] - m, Dd = S[t + 3] - m;
            double d[4] = {0, 0, 0, 0};
            if (k == 2) {
                d[0] = wM[l] * B;
                d[1] = wM[l] * A;
            } else if (k == 3) {
                d[0] = wM[l] * B * Cc;
                d[1] = wM[l] * A * Cc;
                d[2] = wM[l] * A * B;
            } else {
                d[0] = wM[l] * B * Cc * Dd + wAB[l] * B + wAC[l] * Cc + wAD[l] * Dd;
                d[1] = wM[l] * A * Cc * Dd + wAB[l] * A + wBD[l] * Dd + wBC[l] * Cc;
                d[2] = wM[l] * A * B * Dd + wCD[l] * Dd + wAC[l] * A + wBC[l] * B;
                d[3] = wM[l] * A * B * Cc + wCD[l] * Cc + wBD[l] * B + wAD[l] * A;
            }
            for (int q = 0; q < k; ++q) {
                Gn[t + q] += d[q];
                dm += d[q];
            }
        }
        G.swap(Gn);
    }
    const double scale = iw ? IW : 1.0;
    for (int t = 0; t < T; ++t) {
        gr[t] = g * (scale * (G[t] - dm / T) + (iw ? out_raw * I[t] / T : 0.0));
        gi[t] = iw ? g * out_raw * r[t] / T : 0.0;
    }
    return true;
}

// Adjoint of the temporal reduction for one subvoxel: dL/drad_t and dL/dI_t
// from dL/dmap. TRA (kernel.cu:291-327), TRM (kernel.cu:332-366: the maximum's
// first argmax carries the derivative, none when the maximum is the seed 0),
// TRPPM (kernel.cu:372-419, in the closed form ((sum r+)^2 + sum r+^2) / 2 /
// count) and TRAC with ITC 0 (kernel.cu:469-507).
bool temporal_adjoint(const oconf& c, const double* r, const double* I, int T, double g, double* gr, double* gi) {
    for (int t = 0; t < T; ++t) gr[t] = gi[t] = 0.0;
    const bool iw = c.intensity_w == 1;
    if (c.method == 1) {
        for (int t = 0; t < T; ++t) {
            gr[t] = g * (iw ? I[t] : 1.0) / T;
            gi[t] = iw ? g * r[t] / T : 0.0;
        }
        return true;
    }
    if (c.method == 0) {
        double mip = 0.0;
        int arg = -1;
        for (int t = 0; t < T; ++t) {
            const double v = iw ? r[t] * I[t] : r[t];
            if (v > mip) {
                mip = v;
                arg = t;
            }
        }
        if (arg >= 0) {
            gr[arg] = g * (iw ? I[arg] : 1.0);
            gi[arg] = iw ? g * r[arg] : 0.0;
        }
        return true;
    }
    if (c.method == 2) {
        double s1 = 0, s2 = 0, si = 0;
        for (int t = 0; t < T; ++t) {
            const double rp = r[t] > 0 ? r[t] : 0.0;
            s1 += rp;
            s2 += rp * rp;
            si += I[t];
        }
        const double count = std::max(0.5 * T * (T + 1), 1.0);
        const double scale = iw ? si / T : 1.0;
        const double pps = 0.5 * (s1 * s1 + s2) / count;
        for (int t = 0; t < T; ++t) {
            gr[t] = r[t] > 0 ? g * (s1 + r[t]) / count * scale : 0.0;
            gi[t] = iw ? g * pps / T : 0.0;
        }
        return true;
    }
    if (c.method == 3 && c.itc == 1) return temporal_adjoint_itc1(c, r, I, T, g, gr, gi);
    if (c.method != 3) return false;
    const int k = c.trac_order;
    double m = 0, IW = 0;
    for (int t = 0; t < T; ++t) {
        m += r[t];
        IW += r[t] * I[t];
    }
    m /= T;
    IW /= T;
    std::vector<double> a(T + 4, 0.0), dC(T + 4, 0.0);
    for (int t = 0; t < T; ++t) a[t] = r[t] - m;
    const int N = T - k;
    double C = 0;
    if (k == 2) {
        for (int t = 0; t < N; ++t) {
            C += a[t] * a[t + 1];
            dC[t] += a[t + 1];
            dC[t + 1] += a[t];
        }
    } else if (k == 3) {
        for (int t = 0; t < N; ++t) {
            C += a[t] * a[t + 1] * a[t + 2];
            dC[t] += a[t + 1] * a[t + 2];
            dC[t + 1] += a[t] * a[t + 2];
            dC[t + 2] += a[t] * a[t + 1];
        }
    } else {
        double S4 = 0, AB = 0, CD = 0, AC = 0, BD = 0, AD = 0, BC = 0;
        for (int t = 0; t < N; ++t) {
            const double A = a[t], B = a[t + 1], Cc = a[t + 2], Dd = a[t + 3];
            S4 += A * B * Cc * Dd;
            AB += A * B;
            CD += Cc * Dd;
            AC += A * Cc;
            BD += B * Dd;
            AD += A * Dd;
            BC += B * Cc;
        }
        C = S4 - AB * CD - AC * BD - AD * BC;
        for (int t = 0; t < N; ++t) {
            const double A = a[t], B = a[t + 1], Cc = a[t + 2], Dd = a[t + 3];
            // d/dA, d/dB, d/dC, d/dD of the per-t terms
            dC[t] += B * Cc * Dd - B * CD - Cc * BD - Dd * BC;
            dC[t + 1] += A * Cc * Dd - A * CD - Dd * AC - Cc * AD;
            dC[t + 2] += A * B * Dd - Dd * AB - A * BD - B * AD;
            dC[t + 3] += A * B * Cc - Cc * AB - B * AC - A * BC;
        }
    }
    double mean_dC = 0;
    for (int t = 0; t < T; ++t) mean_dC += dC[t];
    mean_dC /= T;
    const double sgn = C > 0 ? 1.0 : (C < 0 ? -1.0 : 0.0);
    const double scale = iw ? IW : 1.0;
    for (int t = 0; t < T; ++t) {
        gr[t] = g * (sgn / T * scale * (dC[t] - mean_dC) + (iw ? std::fabs(C) / T * I[t] / T : 0.0));
        gi[t] = iw ? g * std::fabs(C) / T * r[t] / T : 0.0;
    }
    return true;
}

// Forward + adjoint on one whole block (every temporal method).
bool objective_adjoint(const float* in, const int dims[4], const oconf& c, const double* shifts, const double* gmap,
                       double* map_out, double* dL_din, double* dL_dshift) {
    const int W = dims[0], H = dims[1], D = dims[2], T = dims[3];
    const size_t nv = (size_t)W * H * D;
    std::vector<double> Ip(nv * T);
#pragma omp parallel for
    for (int t = 0; t < T; ++t) {
        std::vector<double> v(in + (size_t)t * nv, in + (size_t)t * nv + nv);
        if (shifts)
            shift_volume(v.data(), Ip.data() + (size_t)t * nv, W, H, D, shifts + 3 * t, -1);
        else
            std::copy(v.begin(), v.end(), Ip.begin() + (size_t)t * nv);
    }
    Ring R;
    R.n = 2 * c.axes_in_ring;
    R.x.resize(R.n * R.n);
    R.y.resize(R.n * R.n);
    R.z.resize(R.n * R.n);
    build_ring(c.ring_radius, R.n, R.x.data(), R.y.data(), R.z.data());
    Field<double> F;
    F.nt = T;
    for (int a = 0; a < 3; ++a) {
        F.dim[a] = dims[a];
        F.c0[a] = 0;
        F.c1[a] = dims[a];
        F.n[a] = dims[a];
    }
    gradient<double>(Ip.data(), dims, c, F);
    const int mx = c.mag[0], my = c.mag[1], mz = c.mag[2];
    const int FX = W * mx, FY = H * my, FZ = D * mz;
    const size_t nfine = (size_t)FX * FY * FZ;
    std::vector<double> rad(nfine * T), inten(nfine * T), gS(nfine * T), gI(nfine * T);
    std::vector<char> valid(nfine, 1);
#pragma omp parallel
    {
        std::vector<double> rr(T + 8), ii(T + 8), gr(T), gi(T);
#pragma omp for schedule(dynamic, 8)
        for (long long v = 0; v < (long long)nfine; ++v) {
            const int X = (int)(v % FX), Y = (int)((v / FX) % FY), Z = (int)(v / ((size_t)FX * FY));
            std::fill(rr.begin(), rr.end(), 0.0);
            for (int t = 0; t < T; ++t) {
                rr[t] = radiality<double>(F, R, c, X, Y, Z, t);
                ii[t] = intensity<double>(F, c, X, Y, Z, t);
                rad[(size_t)t * nfine + v] = rr[t];
                inten[(size_t)t * nfine + v] = ii[t];
            }
            std::vector<double> rcopy(rr);
            const double mv = temporal<double>(c, rcopy.data(), ii.data(), T);
            map_out[v] = mv;
            const bool ok = std::isfinite(mv) && std::isfinite(gmap[v]);
            valid[v] = ok;
            if (ok) temporal_adjoint(c, rr.data(), ii.data(), T, gmap[v], gr.data(), gi.data());
            for (int t = 0; t < T; ++t) {
                double gs = ok ? gr[t] : 0.0;
                if (c.renormalize == 1) gs *= 0.5;
                if (c.remove_con == 1 && !(rr[t] > 0)) gs = 0.0;
                gS[(size_t)t * nfine + v] = gs;
                gI[(size_t)t * nfine + v] = (ok && ii[t] > 0) ? gi[t] : 0.0;
            }
        }
    }
    // radiality and intensity adjoint per time point
    const double r = c.ring_radius;
    const int n = R.n;
    std::vector<double> dIp(nv * T, 0.0);
#pragma omp parallel for schedule(dynamic, 1)
    for (int t = 0; t < T; ++t) {
        std::vector<double> dG[3] = {std::vector<double>(nv, 0.0), std::vector<double>(nv, 0.0),
                                     std::vector<double>(nv, 0.0)};
        double* dI = dIp.data() + (size_t)t * nv;
        auto taps = [&](double qx, double qy, double qz, auto&& fn) {
            const int u0 = (int)std::floor(qx - 0.5), v0 = (int)std::floor(qy - 0.5), w0 = (int)std::floor(qz - 0.5);
            for (int k = 0; k <= 3; ++k)
                for (int j = 0; j <= 3; ++j)
                    for (int i = 0; i <= 3; ++i) {
                        const int u = u0 - 1 + i, vv = v0 - 1 + j, w = w0 - 1 + k;
                        const double wt = cubic<double>(qx - (u + 0.5)) * cubic<double>(qy - (vv + 0.5)) *
                                          cubic<double>(qz - (w + 0.5));
                        fn((size_t)(clampi(w, 0, D - 1) * H + clampi(vv, 0, H - 1)) * W + clampi(u, 0, W - 1), wt);
                    }
        };
        for (long long v = 0; v < (long long)nfine; ++v) {
            const double gs = gS[(size_t)t * nfine + v];
            const double gi = gI[(size_t)t * nfine + v];
            if (!valid[v] || (gs == 0.0 && gi == 0.0)) continue;
            const int X = (int)(v % FX), Y = (int)((v / FX) % FY), Z = (int)(v / ((size_t)FX * FY));
            const double Xc = X + 0.5, Yc = Y + 0.5, Zc = Z + 0.5;
            if (gi != 0.0) taps(Xc / mx, Yc / my, Zc / mz, [&](size_t o, double wt) { dI[o] += gi * wt; });
            if (gs == 0.0) continue;
            for (int id = 0; id < n * n; ++id) {
                const double rx = R.x[id], ry = R.y[id], rz = R.z[id];
                const double qx = (Xc + rx) / mx, qy = (Yc + ry) / my, qz = (Zc + rz) / mz;
                double G[3] = {0, 0, 0};
                const size_t tofs = (size_t)t * nv;
                taps(qx, qy, qz, [&](size_t o, double wt) {
                    G[0] += wt * F.g[0][tofs + o];
                    G[1] += wt * F.g[1][tofs + o];
                    G[2] += wt * F.g[2][tofs + o];
                });
                const double G2 = G[0] * G[0] + G[1] * G[1] + G[2] * G[2];
                const double GdotR = (G[0] * rx + G[1] * ry + G[2] * rz) / (std::sqrt(G2) * r);
                const double sigma = (GdotR > 0 || GdotR != GdotR) ? -1.0 : 1.0;
                const double tt = (G[0] * rx + G[1] * ry + G[2] * rz) / G2;
                const double vv[3] = {rx - G[0] * tt, ry - G[1] * tt, rz - G[2] * tt};
                const double Dk = std::sqrt(vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2]);
                if (!(Dk > 0)) continue;
                // S = sum sigma (1 - Dk/r)^2 / n; dDk/dG = -(tt/Dk) v since v is perpendicular to G
                const double coef = gs * sigma / n * 2.0 * (1.0 - Dk / r) * (-1.0 / r) * (-tt / Dk);
                const double dg[3] = {coef * vv[0], coef * vv[1], coef * vv[2]};
                taps(qx, qy, qz, [&](size_t o, double wt) {
                    dG[0][o] += wt * dg[0];
                    dG[1][o] += wt * dg[1];
                    dG[2][o] += wt * dg[2];
                });
            }
        }
        // transpose of the gradient stencil with block-edge clamping
        int mR = c.main_range, xR = c.x_range, yR = c.y_range, zR = c.z_range;
        if (c.gradient_smooth == 0) {
            mR = 1;
            xR = yR = zR = 0;
        }
        for (int z = 0; z < D; ++z)
            for (int y = 0; y < H; ++y)
                for (int x = 0; x < W; ++x) {
                    const size_t o = (size_t)(z * H + y) * W + x;
                    auto P = [&](int dx, int dy, int dz) {
                        return (size_t)(clampi(z + dz, 0, D - 1) * H + clampi(y + dy, 0, H - 1)) * W +
                               clampi(x + dx, 0, W - 1);
                    };
                    for (int i = -mR; i <= mR; ++i)
                        for (int j = -yR; j <= yR; ++j)
                            for (int k = -zR; k <= zR; ++k)
                                if (i) dI[P(i, j, k)] += (i > 0 ? 1.0 : -1.0) * dG[0][o];
                    for (int j = -mR; j <= mR; ++j)
                        for (int i = -xR; i <= xR; ++i)
                            for (int k = -zR; k <= zR; ++k)
                                if (j) dI[P(i, j, k)] += (j > 0 ? 1.0 : -1.0) * dG[1][o];
                    for (int k = -mR; k <= mR; ++k)
                        for (int i = -xR; i <= xR; ++i)
                            for (int j = -yR; j <= yR; ++j)
                                if (k) dI[P(i, j, k)] += (k > 0 ? 1.0 : -1.0) * dG[2][o];
                }
    }
    // through the drift operator
#pragma omp parallel for
    for (int t = 0; t < T; ++t) {
        const double* g = dIp.data() + (size_t)t * nv;
        if (!shifts) {
            std::copy(g, g + nv, dL_din + (size_t)t * nv);
            continue;
        }
        shift_volume_adjoint(g, dL_din + (size_t)t * nv, W, H, D, shifts + 3 * t);
        if (dL_dshift) {
            std::vector<double> v(in + (size_t)t * nv, in + (size_t)t * nv + nv), dv(nv);
            for (int ax = 0; ax < 3; ++ax) {
                shift_volume(v.data(), dv.data(), W, H, D, shifts + 3 * t, ax);
                double s = 0;
                for (size_t i = 0; i < nv; ++i) s += g[i] * dv[i];
                dL_dshift[3 * t + ax] = s;
            }
        }
    }
    return true;
}

}  // namespace

extern "C" {

// Forward map and adjoint of L with dL/dmap = gmap (whole block). shifts (T x 3,
// x y z) may be NULL (no drift operator). Returns -2 for reductions without a
// derivative here.
int oracle_adjoint_f64(const float* in, const int* dims, const oconf* c, const double* shifts, const double* gmap,
                       double* map_out, double* dL_din, double* dL_dshift) {
    return objective_adjoint(in, dims, *c, shifts, gmap, map_out, dL_din, dL_dshift) ? 0 : -2;
}

// Forward map of the shifted input (FP64), for finite differences.
int oracle_forward_shifted_f64(const float* in, const int* dims, const oconf* c, const double* shifts,
                               double* map_out) {
    const int W = dims[0], H = dims[1], D = dims[2], T = dims[3];
    const size_t nv = (size_t)W * H * D;
    std::vector<double> Ip(nv * T);
#pragma omp parallel for
    for (int t = 0; t < T; ++t) {
        std::vector<double> v(in + (size_t)t * nv, in + (size_t)t * nv + nv);
        if (shifts)
            shift_volume(v.data(), Ip.data() + (size_t)t * nv, W, H, D, shifts + 3 * t, -1);
        else
            std::copy(v.begin(), v.end(), Ip.begin() + (size_t)t * nv);
    }
    Ring R;
    R.n = 2 * c->axes_in_ring;
    R.x.resize(R.n * R.n);
    R.y.resize(R.n * R.n);
    R.z.resize(R.n * R.n);
    build_ring(c->ring_radius, R.n, R.x.data(), R.y.data(), R.z.data());
    Field<double> F;
    F.nt = T;
    for (int a = 0; a < 3; ++a) {
        F.dim[a] = dims[a];
        F.c0[a] = 0;
        F.c1[a] = dims[a];
        F.n[a] = dims[a];
    }
    gradient<double>(Ip.data(), dims, *c, F);
    const int FX = W * c->mag[0], FY = H * c->mag[1], FZ = D * c->mag[2];
    const size_t nfine = (size_t)FX * FY * FZ;
#pragma omp parallel
    {
        std::vector<double> rr(T + 8), ii(T + 8);
#pragma omp for schedule(dynamic, 8)
        for (long long v = 0; v < (long long)nfine; ++v) {
            const int X = (int)(v % FX), Y = (int)((v / FX) % FY), Z = (int)(v / ((size_t)FX * FY));
            std::fill(rr.begin(), rr.end(), 0.0);
            for (int t = 0; t < T; ++t) {
                rr[t] = radiality<double>(F, R, *c, X, Y, Z, t);
                ii[t] = intensity<double>(F, *c, X, Y, Z, t);
            }
            map_out[v] = temporal<double>(*c, rr.data(), ii.data(), T);
        }
    }
    return 0;
}

// The drift operator alone (FP64), for tests of the CUDA resampling.
int oracle_shift_f64(const float* in, const int* dims, const double* shifts, double* out) {
    const int W = dims[0], H = dims[1], D = dims[2], T = dims[3];
    const size_t nv = (size_t)W * H * D;
#pragma omp parallel for
    for (int t = 0; t < T; ++t) {
        std::vector<double> v(in + (size_t)t * nv, in + (size_t)t * nv + nv);
        shift_volume(v.data(), out + (size_t)t * nv, W, H, D, shifts + 3 * t, -1);
    }
    return 0;
}

int oracle_ring_f32(float r, int axes, float* x, float* y, float* z) {
    build_ring(r, 2 * axes, x, y, z);
    return 0;
}

int oracle_srrf_region_f64(const float* in, const int* dims, const oconf* c, const int* lo, const int* hi, double* out,
                           double* rad_stack, double* int_stack) {
    srrf_region<double>(in, dims, *c, lo, hi, out, rad_stack, int_stack);
    return 0;
}

int oracle_srrf_region_f32(const float* in, const int* dims, const oconf* c, const int* lo, const int* hi, float* out,
                           float* rad_stack, float* int_stack) {
    srrf_region<float>(in, dims, *c, lo, hi, out, rad_stack, int_stack);
    return 0;
}

int oracle_legacy_f64(const float* in, const int* dims, const oconf* c, double* out) {
    legacy<double>(in, dims, *c, out);
    return 0;
}

int oracle_legacy_f32(const float* in, const int* dims, const oconf* c, float* out) {
    legacy<float>(in, dims, *c, out);
    return 0;
}

// Temporal reduction alone on a given series (tests of the reduction quirks).
int oracle_temporal_f64(const oconf* c, const double* rad, const double* inten, int nt, double* out) {
    std::vector<double> r(nt + 8, 0.0);
    std::memcpy(r.data(), rad, sizeof(double) * nt);
    *out = temporal<double>(*c, r.data(), inten, nt);
    return 0;
}
}

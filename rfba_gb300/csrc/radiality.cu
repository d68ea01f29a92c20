// Fused gradient + Catmull-Rom magnification + radiality kernel (sm_103a).
//
// Replaces the reference's gradKernel (kernel.cu:44-125) and calculateRadiality
// (kernel.cu:186-253, with interpolateG kernel.cu:141-169, _calculateDk
// kernel.cu:174-183 and interpolateIntensity kernel.cu:257-287) by one
// persistent kernel. Per work item (block, subvoxel tile, time chunk) and time
// point:
//
//   1. the input tile plus halo is staged into shared memory by a TMA tensor
//      copy (requested one time point ahead) and converted to float with the
//      reference's block-edge clamp (its fminf/fmaxf clamps); inputs whose rows
//      a tensor map cannot address are read with plain loads instead;
//   2. the smoothed gradient G = (Gx, Gy, Gz) and the intensity I of every
//      coarse cell the tile's taps reach is formed in shared memory (float4);
//   3. the ring's n^2 samples are reduced to their distinct points (62 for
//      n = 12) and factorised per axis. Catmull-Rom interpolation is separable,
//      and a sample's x taps and weights depend only on the subvoxel's x phase
//      (X mod mag_x) and the ring point's x coordinate, so for each distinct ring
//      x value the x-filtered field U is formed once in shared memory;
//   4. each thread owns two subvoxel columns (X, Y) and (X, Y + mag_y): same y
//      phase, adjacent coarse rows, so the y pass reads 5 rows of U for both.
//      For each distinct (x, y) ring pair it y-filters U into a register column
//      T[w] over coarse z (one float2 per w: the two columns), and for each ring
//      point of that pair it z-filters T (4 taps; the tap offset per z phase is
//      uniform over the warp, so both offsets are unrolled with static register
//      indices) for its FZ subvoxels per column and accumulates the radiality
//      term. The per-point work runs on packed f32x2 FMAs (two columns per
//      instruction);
//   5. radiality and interpolated intensity per subvoxel and time point are
//      written to the stack that the temporal kernel reduces.
//
// The radiality term of a sample with interpolated gradient g and ring offset
// rho (kernel.cu:224-240), with u = rho / r, is evaluated in a rotated frame:
// (x, y) is turned about z so that u lies in the x'z plane, u = |u| (h x' + c z).
// Then g.u / |u| = h g_x' + c g_z, the part of g perpendicular to u has the
// components g_y' and h g_z - c g_x', and
//   Dk / r = |u| sin(angle(g, u)) = |u| sqrt(|g_perp|^2 / |g|^2),
//   D = (1 - Dk/r)^2,   S -= D if g.u > 0, S += D otherwise.
// The perpendicular part is formed directly, so Dk has full relative accuracy
// even when g is almost parallel to u; g = 0 gives 0 * inf = NaN exactly as the
// reference's 0/0 does. Coordinates are local (phase + ring offset), so no
// precision is lost at large volume coordinates. The sample window test
// (kernel.cu:146) makes a whole subvoxel NaN; it is evaluated on the host per
// axis with the reference's float arithmetic and applied here as a per-block
// valid box.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include <cudaTypedefs.h>

#include "srrf_internal.h"

namespace rfba {
namespace {

// ---- TMA staging of the input tile ----------------------------------------
// The tile's input box (x rounded down to a 16-byte boundary, so the box is
// wider by up to 15 bytes) is copied by one cp.async.bulk.tensor per time point
// into a staging area, completion signalled on an mbarrier. The next time
// point's box is requested as soon as the current one has been converted, so
// the copy overlaps the radiality work. Coordinates outside the volume read
// zeros; the reference's block-edge clamp is applied when the staging area is
// converted to float (clamped positions always lie inside the box).
__device__ __forceinline__ unsigned smem_u32(const void* ptr) {
    return (unsigned)__cvta_generic_to_shared(ptr);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tma_load_box(void* dst, const CUtensorMap* map, uint64_t* bar, unsigned bytes, int x,
                                             int y, int z, int t) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(t), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait for the staging phase: false once about a second of wall time
// (%globaltimer) has passed without the phase completing, whatever the time a
// single try_wait suspends for; an iteration cap backs the clock up.
constexpr unsigned long long kWaitLimitNs = 1000000000ull;
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (int i = 1; i < (1 << 26); ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 15) == 0 && global_ns() - t0 > kWaitLimitNs) return false;
    }
    return false;
}

__device__ __forceinline__ float rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

template <int V>
struct IntC {
    static constexpr int value = V;
};
// copysign(w, -d) for w >= 0: -w when d > 0 (diverging), +w when d < 0. At
// d = 0 the sample is perpendicular to g, s = |u| and D vanishes, so the sign
// taken there does not matter.
__device__ __forceinline__ float sign_weight(float w, float d) {
    return __int_as_float(__float_as_int(w) | (~__float_as_int(d) & 0x80000000));
}

__device__ __forceinline__ float2 dup(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }

template <typename Tin>
__device__ __forceinline__ float load_in(const Tin* p, long long i);
template <>
__device__ __forceinline__ float load_in<float>(const float* p, long long i) {
    return __ldg(p + i);
}
template <>
__device__ __forceinline__ float load_in<uint16_t>(const uint16_t* p, long long i) {
    return (float)__ldg(p + i);
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__device__ __forceinline__ int floordiv(int a, int b) {  // b > 0
    int q = a / b;
    return (a % b != 0 && a < 0) ? q - 1 : q;
}

// gradKernel's smoothed gradient (kernel.cu:73-124) at one coarse cell from the
// clamped input tile: Gx = sum over i in [1, mR], j in [-yR, yR], k in
// [-zR, zR] of I(+i, j, k) - I(-i, j, k), and likewise for y and z; with
// smoothing off the reference's central difference is the case mR = 1 and all
// lateral ranges 0. The .w component carries I at the cell. Fixed ranges are
// fully unrolled; integer inputs make the sums exact in float whatever the order.
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

template <int MZ, int CZ, typename Tin, bool WIDE>
__global__ void __launch_bounds__(WIDE ? kMaxThreads : 128, WIDE ? 2 : RFBA_FWD_CTAS)
    radiality_kernel(const RadParams p, const __grid_constant__ CUtensorMap tmap) {
    constexpr int FZ = MZ * CZ;
    constexpr int NW = CZ + 4;
    extern __shared__ float4 smem4[];

    // Shared layout: [G tile float4][U tile float4][input tile][tables][TMA staging, 128-byte aligned]
    const int NU = p.NU, NV = p.NV;
    float4* gt = smem4;                           // [NW][NV][NU]
    float4* ut = gt + NU * NV * NW;               // [NW][NV][16]
    float* inp = reinterpret_cast<float*>(ut + kTileX * NV * NW);  // [NIZ][NIY][NIX]
    float* tab = inp + ((p.NIX * p.NIY * p.NIZ + 3) & ~3);         // 16-byte aligned (float4 reads)
    Tin* stage = reinterpret_cast<Tin*>((reinterpret_cast<uintptr_t>(tab + p.smem_table_words) + 127) &
                                        ~(uintptr_t)127);           // [NIZ][NIY][tma_bx]
    __shared__ unsigned int s_item;
    __shared__ alignas(8) uint64_t s_bar;
    const bool use_tma = p.use_tma != 0;
    unsigned phase = 0;
    if (use_tma && threadIdx.x == 0) {
        mbar_init(&s_bar, 1);
        fence_mbar_init();
    }

    const int nthr = blockDim.x;
    const int tid = threadIdx.x;
    const int mx = p.mag[0], my = p.mag[1];
    // column pair of this thread: (X, Ya) and (X, Ya + my)
    const int xf = tid & (kTileX - 1);
    const int q = tid / kTileX;                   // 0 .. TY/2 - 1
    const int yfa = (q / my) * (2 * my) + (q % my);

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

    const Tin* in = static_cast<const Tin*>(p.in);
    const int NIX = p.NIX, NIY = p.NIY, NIZ = p.NIZ, R = p.R;
    const int ncell = NU * NV * NW;
    const int nut = kTileX * NV * NW;

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

        // Tile geometry (block-local fine and coarse coordinates).
        const int X0 = B.lo[0] + td.tx * kTileX;
        const int Y0 = B.lo[1] + td.ty * p.TY;
        const int Z0 = B.zbase + td.tz * FZ;
        const int cx0 = floordiv(X0, mx) - 2;
        const int cy0 = floordiv(Y0, my) - 2;
        const int cz0 = Z0 / MZ - 2;
        const int X = X0 + xf;
        const int Ya = Y0 + yfa, Yb = Ya + my;
        const int xi = floordiv(X, mx), xr = X - xi * mx;
        const int yi = floordiv(Ya, my), yr = Ya - yi * my;  // Yb: yi + 1, same phase
        const bool xin = X < B.hi[0];
        const bool ina = xin && Ya < B.hi[1];
        const bool inb = xin && Yb < B.hi[1];
        const bool xrad = X >= B.rad_lo[0] && X <= B.rad_hi[0];
        const bool xint = X >= B.int_lo[0] && X <= B.int_hi[0];
        const bool rada = xrad && Ya >= B.rad_lo[1] && Ya <= B.rad_hi[1];
        const bool radb = xrad && Yb >= B.rad_lo[1] && Yb <= B.rad_hi[1];
        const bool inta = xint && Ya >= B.int_lo[1] && Ya <= B.int_hi[1];
        const bool intb = xint && Yb >= B.int_lo[1] && Yb <= B.int_hi[1];
        const long long V = B.vox;
        const long long va = ((long long)(Ya - B.lo[1])) * B.nreg[0] + (X - B.lo[0]);
        const long long vb = ((long long)(Yb - B.lo[1])) * B.nreg[0] + (X - B.lo[0]);
        const long long zstride = (long long)B.nreg[0] * B.nreg[1];

        const int t0 = p.t_lo + chunk * p.t_chunk;
        const int t1 = min(p.t_hi > 0 ? p.t_hi : p.T, t0 + p.t_chunk);
        // TMA box origin: x rounded down to a 16-byte boundary; the offset back
        // (0 .. 16 bytes / element size - 1) is where the tile starts in a staged row
        constexpr int kAl = 16 / (int)sizeof(Tin);
        auto box_ox = [&]() {
            const int gx0 = B.origin[0] + cx0 - R;
            return ((gx0 % kAl) + kAl) % kAl;
        };
        auto issue = [&](int tt) {
            const int gx0 = B.origin[0] + cx0 - R;
            tma_load_box(stage, &tmap, &s_bar, (unsigned)(p.tma_bx * NIY * NIZ * (int)sizeof(Tin)), gx0 - box_ox(),
                         B.origin[1] + cy0 - R, B.origin[2] + cz0 - R, tt);
        };
        if (use_tma && tid == 0) {
            fence_proxy_async();  // the previous item's generic reads of the staging area come first
            // failure-detection test hook: without the request the wait below
            // runs out, the CTA records the timeout and leaves
            if (!p.test_skip_copy) issue(t0);
        }
        for (int t = t0; t < t1; ++t) {
            const long long sbase = B.stack_off + (long long)(t - p.stack_t0) * V;
            // 1. input tile with block-edge clamp; 16 lanes per row, one division
            //    per row
            const long long tbase = (long long)t * p.D * p.H * p.W;
            if (use_tma) {
                const bool ok = mbar_wait_bounded(&s_bar, phase);
                if (__syncthreads_or(!ok)) {
                    // the copy did not land: record it, give it a bounded time to
                    // finish so no write is pending into this CTA's shared memory
                    if (tid == 0) {
                        if (p.err) atomicCAS(p.err, 0ull, (0x54ull << 56) | (unsigned long long)item);
                        mbar_wait_bounded(&s_bar, phase);
                    }
                    return;
                }
                phase ^= 1u;
                for (int r = tid / kTileX; r < NIY * NIZ; r += nthr / kTileX) {
                    const int iy = r % NIY, iz = r / NIY;
                    const int sy = clampi(cy0 - R + iy, 0, bh - 1) - (cy0 - R);
                    const int sz = clampi(cz0 - R + iz, 0, bd - 1) - (cz0 - R);
                    const Tin* srow = stage + (sz * NIY + sy) * p.tma_bx + box_ox();
                    float* rows = inp + r * NIX;
                    for (int ix = xf; ix < NIX; ix += kTileX)
                        rows[ix] = (float)srow[clampi(cx0 - R + ix, 0, bw - 1) - (cx0 - R)];
                }
                __syncthreads();
                if (tid == 0 && t + 1 < t1) {
                    fence_proxy_async();  // the staging area's generic reads before the next async write
                    issue(t + 1);
                }
            } else {
                for (int r = tid / kTileX; r < NIY * NIZ; r += nthr / kTileX) {
                    const int iy = r % NIY, iz = r / NIY;
                    const int by = clampi(cy0 - R + iy, 0, bh - 1);
                    const int bz = clampi(cz0 - R + iz, 0, bd - 1);
                    const long long rowg = tbase + ((long long)(B.origin[2] + bz) * p.H + (B.origin[1] + by)) * p.W +
                                           B.origin[0];
                    float* rows = inp + r * NIX;
                    for (int ix = xf; ix < NIX; ix += kTileX)
                        rows[ix] = load_in<Tin>(in, rowg + clampi(cx0 - R + ix, 0, bw - 1));
                }
                __syncthreads();
            }
            // 2. gradient + intensity per coarse cell
            for (int c = tid; c < ncell; c += nthr) {
                const int u = c % NU;
                const int v = (c / NU) % NV;
                const int w = c / (NU * NV);
                const int cu = cx0 + u, cv = cy0 + v, cw = cz0 + w;
                float4 g4 = make_float4(0.f, 0.f, 0.f, 0.f);
                if (cu >= 0 && cu < bw && cv >= 0 && cv < bh && cw >= 0 && cw < bd) {
                    const float* base = inp + ((w + R) * NIY + (v + R)) * NIX + (u + R);
                    if (p.grad_mode == 1)
                        g4 = gradient_fixed<1, 1, 1, 1>(base, NIX, NIY);
                    else if (p.grad_mode == 2)
                        g4 = gradient_fixed<1, 0, 0, 0>(base, NIX, NIY);
                    else
                        g4 = gradient_generic(base, NIX, NIY, p.gr);
                }
                gt[c] = g4;
            }

            float2 S[FZ];
#pragma unroll
            for (int z = 0; z < FZ; ++z) S[z] = make_float2(0.f, 0.f);

            for (int gi = 0; gi < p.ngroups; ++gi) {
                __syncthreads();  // gt ready / previous U consumed
                // 3. x-filter for ring x value a
                const int a = grp_xval[gi];
                {
                    const int o = offx[a * mx + xr];
                    const float4 wv = *reinterpret_cast<const float4*>(wx + (a * mx + xr) * 4);
                    const int ub = xi - cx0 - 2 + o;
                    for (int e = tid; e < nut; e += nthr) {
                        const int vw = e / kTileX;  // (w * NV + v)
                        const float4* src = gt + vw * NU + ub;
                        const float4 g0 = src[0], g1 = src[1], g2 = src[2], g3 = src[3];
                        float4 r;
                        r.x = fmaf(wv.w, g3.x, fmaf(wv.z, g2.x, fmaf(wv.y, g1.x, wv.x * g0.x)));
                        r.y = fmaf(wv.w, g3.y, fmaf(wv.z, g2.y, fmaf(wv.y, g1.y, wv.x * g0.y)));
                        r.z = fmaf(wv.w, g3.z, fmaf(wv.z, g2.z, fmaf(wv.y, g1.z, wv.x * g0.z)));
                        r.w = fmaf(wv.w, g3.w, fmaf(wv.z, g2.w, fmaf(wv.y, g1.w, wv.x * g0.w)));
                        ut[e] = r;
                    }
                }
                __syncthreads();
                // 4. pairs of this x value
                for (int pi = grp[gi]; pi < grp[gi + 1]; ++pi) {
                    const int b = pair_yval[pi];
                    const int o = offy[b * my + yr];
                    const float4 wv = *reinterpret_cast<const float4*>(wy + (b * my + yr) * 4);
                    const int vbase = yi - cy0 - 2 + o;  // column a rows vbase..+3, column b rows vbase+1..+4
                    if (pi == p.zero_pair) {
                        // intensity at the subvoxel centre (interpolateIntensity): the
                        // (0, 0) pair's x/y passes are the intensity's; z pass with rho_z = 0
                        float2 Tw[NW];
#pragma unroll
                        for (int w = 0; w < NW; ++w) {
                            const float4* src = ut + (w * NV + vbase) * kTileX + xf;
                            const float u0 = src[0].w, u1 = src[kTileX].w, u2 = src[2 * kTileX].w,
                                        u3 = src[3 * kTileX].w, u4 = src[4 * kTileX].w;
                            Tw[w].x = fmaf(wv.w, u3, fmaf(wv.z, u2, fmaf(wv.y, u1, wv.x * u0)));
                            Tw[w].y = fmaf(wv.w, u4, fmaf(wv.z, u3, fmaf(wv.y, u2, wv.x * u1)));
                        }
#pragma unroll
                        for (int z = 0; z < FZ; ++z) {
                            const int zr = z % MZ, zi = z / MZ;
                            const float* qz = wzi + zr * 5;
                            // exactly the reference's 4 taps (kernel.cu:268-283), so a
                            // non-finite voxel reaches the same subvoxels: they start one
                            // coarse cell later when floor((zr + 0.5) / mz - 0.5) = 0,
                            // i.e. when 2 zr + 1 >= mz (the fifth weight is 0)
                            const int m0 = (2 * zr + 1 >= MZ) ? 1 : 0;
                            float2 acc = mul2(dup(qz[m0]), Tw[zi + m0]);
#pragma unroll
                            for (int m = m0 + 1; m < m0 + 4; ++m) acc = fma2(dup(qz[m]), Tw[zi + m], acc);
                            const int Z = Z0 + z;
                            if (Z >= B.lo[2] && Z < B.hi[2]) {
                                const bool zint = Z >= B.int_lo[2] && Z <= B.int_hi[2];
                                const long long zo = sbase + (long long)(Z - B.lo[2]) * zstride;
                                if (ina) p.int_stack[zo + va] = (inta && zint) ? fmaxf(acc.x, 0.f) : 0.f;
                                if (inb) p.int_stack[zo + vb] = (intb && zint) ? fmaxf(acc.y, 0.f) : 0.f;
                            }
                        }
                    }
                    float2 Tx[NW], Ty[NW], Tz[NW];
#pragma unroll
                    for (int w = 0; w < NW; ++w) {
                        const float4* src = ut + (w * NV + vbase) * kTileX + xf;
                        const float4 u0 = src[0], u1 = src[kTileX], u2 = src[2 * kTileX], u3 = src[3 * kTileX],
                                     u4 = src[4 * kTileX];
                        Tx[w].x = fmaf(wv.w, u3.x, fmaf(wv.z, u2.x, fmaf(wv.y, u1.x, wv.x * u0.x)));
                        Ty[w].x = fmaf(wv.w, u3.y, fmaf(wv.z, u2.y, fmaf(wv.y, u1.y, wv.x * u0.y)));
                        Tz[w].x = fmaf(wv.w, u3.z, fmaf(wv.z, u2.z, fmaf(wv.y, u1.z, wv.x * u0.z)));
                        Tx[w].y = fmaf(wv.w, u4.x, fmaf(wv.z, u3.x, fmaf(wv.y, u2.x, wv.x * u1.x)));
                        Ty[w].y = fmaf(wv.w, u4.y, fmaf(wv.z, u3.y, fmaf(wv.y, u2.y, wv.x * u1.y)));
                        Tz[w].y = fmaf(wv.w, u4.z, fmaf(wv.z, u3.z, fmaf(wv.y, u2.z, wv.x * u1.z)));
                    }
                    // rotate (x, y) about z so that the pair's ring direction lies in the
                    // x'z plane: P = g.x', E = g.y' (x' = (ux, uy)/h, y' = z x x')
                    {
                        const float2 rot = pair_rot[pi];
                        const float2 ca = dup(rot.x), sb = dup(rot.y), nsb = dup(-rot.y);
#pragma unroll
                        for (int w = 0; w < NW; ++w) {
                            const float2 gx = Tx[w], gy = Ty[w];
                            Tx[w] = fma2(gy, sb, mul2(gx, ca));
                            Ty[w] = fma2(gy, ca, mul2(gx, nsb));
                        }
                    }
                    for (int qi = pair_pt[pi]; qi < pair_pt[pi + 1]; ++qi) {
                        // point u = |u| (h x' + c z): dot = g.u/|u| = h P + c Z, the
                        // perpendicular part of g is (E, h Z - c P), and Dk/r = |u| sin(angle)
                        const float4 pv = pt_vec[qi];
                        const float2 hh = dup(pv.x), cc = dup(pv.y), ncc = dup(-pv.y);
                        const float wgt = pv.z;
                        const float2 nun = dup(pv.w);  // -|u|
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
                                // gx = P, gy = E, gz = Z after the pair rotation
                                const float2 dot = fma2(cc, gz, mul2(hh, gx));
                                const float2 cp = fma2(hh, gz, mul2(ncc, gx));
                                const float2 c2 = fma2(cp, cp, mul2(gy, gy));  // |g_perp|^2
                                const float2 g2 = fma2(dot, dot, c2);          // |g|^2
                                // sin = sqrt(c2) / sqrt(g2): g parallel to u gives 0, g = 0
                                // gives 0 * inf = NaN (the reference's 0/0).
                                const float2 sn = mul2(make_float2(sqrt_approx(c2.x), sqrt_approx(c2.y)),
                                                       make_float2(rsqrt_approx(g2.x), rsqrt_approx(g2.y)));
                                const float2 om = fma2(sn, nun, dup(1.0f));     // 1 - Dk/r
                                const float2 D = mul2(om, om);
                                const float2 sw = make_float2(sign_weight(wgt, dot.x), sign_weight(wgt, dot.y));
                                S[z] = fma2(D, sw, S[z]);
                            }
                        };
#pragma unroll
                        for (int zr = 0; zr < MZ; ++zr) {
                            // weights of one phase at a time keep register pressure low;
                            // the tap offset is uniform over the warp
                            float2 w4[4];
#pragma unroll
                            for (int m = 0; m < 4; ++m) w4[m] = dup(wzc[zr * 4 + m]);
                            if ((offmask >> zr) & 1)
                                zpass(IntC<1>{}, zr, w4);
                            else
                                zpass(IntC<0>{}, zr, w4);
                        }
                    }
                }
            }

            // 5. finalize and store radiality
#pragma unroll
            for (int z = 0; z < FZ; ++z) {
                const int Z = Z0 + z;
                if (Z < B.lo[2] || Z >= B.hi[2]) continue;
                const bool zok = Z >= B.rad_lo[2] && Z <= B.rad_hi[2];
                const long long zo = sbase + (long long)(Z - B.lo[2]) * zstride;
                float ra = (rada && zok) ? S[z].x : __int_as_float(0x7fc00000);
                float rb = (radb && zok) ? S[z].y : __int_as_float(0x7fc00000);
                if (p.renorm) {
                    ra = 0.5f + ra * 0.5f;
                    rb = 0.5f + rb * 0.5f;
                }
                if (p.poscon) {
                    ra = fmaxf(ra, 0.f);
                    rb = fmaxf(rb, 0.f);
                }
                if (ina) p.rad_stack[zo + va] = ra;
                if (inb) p.rad_stack[zo + vb] = rb;
            }
        }
    }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda
// link dependency).
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
        else
            cudaGetLastError();
    });
    return fn;
}

// 4D tensor map (x, y, z, t) of the input with the tile's staging box; false
// (plain loads) when TMA staging is off for this launch or the input cannot be
// described (base or row pitch not 16-byte aligned).
bool encode_input_map(const RadParams& p, int es, CUtensorMap* map) {
    std::memset(map, 0, sizeof *map);
    if (p.tma_bx <= 0) return false;
    if ((reinterpret_cast<uintptr_t>(p.in) & 15) != 0 || ((long long)p.W * es) % 16 != 0) return false;
    if (p.tma_bx > 256 || p.NIY > 256 || p.NIZ > 256 || (p.tma_bx * es) % 16 != 0) return false;
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dim[4] = {(cuuint64_t)p.W, (cuuint64_t)p.H, (cuuint64_t)p.D, (cuuint64_t)p.T};
    const cuuint64_t stride[3] = {(cuuint64_t)p.W * es, (cuuint64_t)p.W * p.H * es, (cuuint64_t)p.W * p.H * p.D * es};
    const cuuint32_t box[4] = {(cuuint32_t)p.tma_bx, (cuuint32_t)p.NIY, (cuuint32_t)p.NIZ, 1u};
    const cuuint32_t estr[4] = {1u, 1u, 1u, 1u};
    const CUresult r = fn(map, es == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                          const_cast<void*>(p.in), dim, stride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

template <int MZ, typename Tin>
int launch_mz(const RadParams& p, int grid, size_t smem, cudaStream_t st) {
    constexpr int CZ = cz_for_mag(MZ);
    auto k = p.TY > 16 ? radiality_kernel<MZ, CZ, Tin, true> : radiality_kernel<MZ, CZ, Tin, false>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    RadParams q = p;
    CUtensorMap map;
    q.use_tma = encode_input_map(p, (int)sizeof(Tin), &map) ? 1 : 0;
    k<<<grid, p.TY * (kTileX / 2), smem, st>>>(q, map);
    return (int)cudaGetLastError();
}

template <int MZ, typename Tin>
int occ_mz(int threads, size_t smem, int* out) {
    constexpr int CZ = cz_for_mag(MZ);
    auto k = threads > 128 ? radiality_kernel<MZ, CZ, Tin, true> : radiality_kernel<MZ, CZ, Tin, false>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, k, threads, smem);
}

template <typename Tin>
int dispatch(const RadParams& p, int grid, size_t smem, cudaStream_t st) {
    switch (p.mag[2]) {
        case 1: return launch_mz<1, Tin>(p, grid, smem, st);
        case 2: return launch_mz<2, Tin>(p, grid, smem, st);
        case 3: return launch_mz<3, Tin>(p, grid, smem, st);
        case 4: return launch_mz<4, Tin>(p, grid, smem, st);
        case 5: return launch_mz<5, Tin>(p, grid, smem, st);
        case 6: return launch_mz<6, Tin>(p, grid, smem, st);
        case 7: return launch_mz<7, Tin>(p, grid, smem, st);
        case 8: return launch_mz<8, Tin>(p, grid, smem, st);
    }
    return (int)cudaErrorInvalidValue;
}

template <typename Tin>
int occ_dispatch(int mz, int threads, size_t smem, int* out) {
    switch (mz) {
        case 1: return occ_mz<1, Tin>(threads, smem, out);
        case 2: return occ_mz<2, Tin>(threads, smem, out);
        case 3: return occ_mz<3, Tin>(threads, smem, out);
        case 4: return occ_mz<4, Tin>(threads, smem, out);
        case 5: return occ_mz<5, Tin>(threads, smem, out);
        case 6: return occ_mz<6, Tin>(threads, smem, out);
        case 7: return occ_mz<7, Tin>(threads, smem, out);
        case 8: return occ_mz<8, Tin>(threads, smem, out);
    }
    return (int)cudaErrorInvalidValue;
}

}  // namespace

// Tile height (subvoxel rows) for a y magnification: a multiple of 2*my (each
// thread pairs row y with y + my) and of 4 (whole warps of 16 x 2 threads).
int tile_rows_for_mag(int my) {
    switch (my) {
        case 1: case 2: case 4: case 8: return 16;
        case 3: case 6: return 12;
        case 5: return 20;
        default: return 28;  // 7
    }
}

size_t radiality_smem_bytes(const RadParams& p) {
    const int NW = cz_for_mag(p.mag[2]) + 4;
    size_t b = sizeof(float4) * ((size_t)p.NU * p.NV * NW + (size_t)kTileX * p.NV * NW);
    b += sizeof(float) * ((((size_t)p.NIX * p.NIY * p.NIZ + 3) & ~(size_t)3) + p.smem_table_words);
    if (p.tma_bx > 0) {
        // staging box (element size 4 covers both input types), 128-byte aligned start
        b += 128 + (size_t)p.tma_bx * p.NIY * p.NIZ * 4;
    }
    return (b + 15) & ~(size_t)15;
}

int radiality_tma_box_x(const RadParams& p, int in_u16) {
    const int es = in_u16 ? 2 : 4;
    const int al = 16 / es;
    if (((long long)p.W * es) % 16 != 0) return 0;
    const char* e = std::getenv("RFBA_TMA");
    if (e && e[0] == '0' && e[1] == 0) return 0;
    const int bx = ((p.NIX + al - 1 + al - 1) / al) * al;  // NIX + up to al - 1 of alignment slack
    return bx <= 256 ? bx : 0;
}

int launch_radiality(const RadParams& p, int grid, size_t smem, int in_u16, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return in_u16 ? dispatch<uint16_t>(p, grid, smem, st) : dispatch<float>(p, grid, smem, st);
}

int radiality_max_ctas_per_sm(const RadParams& p, int in_u16, int* out) {
    const size_t smem = radiality_smem_bytes(p);
    const int threads = p.TY * (kTileX / 2);
    return in_u16 ? occ_dispatch<uint16_t>(p.mag[2], threads, smem, out)
                  : occ_dispatch<float>(p.mag[2], threads, smem, out);
}

}  // namespace rfba

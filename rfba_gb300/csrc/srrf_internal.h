// Internal definitions shared by the host planner (plan.cpp, capi.cpp) and the
// CUDA kernels (radiality.cu, temporal.cu). Not part of the public C-ABI.
#pragma once
#include <vector_types.h>

#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>

#include "../../include/rfba_srrf.h"

namespace rfba {

// Output tile of the radiality kernel: 16 x TY subvoxel columns (two per
// thread, TY from tile_rows_for_mag) and FZ = MZ * CZ subvoxels deep along z,
// held in registers.
constexpr int kTileX = 16;
constexpr int kMaxThreads = 224;  // 16 x 14 threads for the 28-row tile (mag_y 7)
constexpr int kMaxMag = 8;
constexpr int kMaxGradRange = 3;
// Adjoint tile: 16 x 16 subvoxel columns (two consecutive rows per thread).
constexpr int kAdjRows = 16;
constexpr int kAdjThreads = kTileX * kAdjRows / 2;

// Coarse z cells per tile for a given z magnification (FZ = MZ * CZ), and the
// forward kernel's resident CTAs per SM (launch bound; 128-thread tiles).
// Compile-time tuning knobs: -DRFBA_CZ_MZ2=n / -DRFBA_FWD_CTAS=n.
#ifndef RFBA_CZ_MZ2
#define RFBA_CZ_MZ2 8
#endif
#ifndef RFBA_FWD_CTAS
#define RFBA_FWD_CTAS 3
#endif
constexpr int cz_for_mag(int mz) {
    return mz == 1 ? 8 : mz == 2 ? RFBA_CZ_MZ2 : mz == 3 ? 5 : mz == 4 ? 4 : mz == 5 ? 3 : 2;
}

// Coarse z cells per tile of the adjoint kernel (it holds twice the register
// columns of the forward).
constexpr int cza_for_mag(int mz) { return mz <= 2 ? 4 : (mz <= 4 ? 2 : 1); }

// One independent block of the input with the fine region it computes.
struct BlockDev {
    int origin[3];   // input voxel origin in the full volume
    int size[3];     // block dims (input voxels)
    int lo[3];       // fine region [lo, hi) in block-local magnified coords
    int hi[3];
    int rad_lo[3];   // fine indices whose ring samples all pass the window (inclusive)
    int rad_hi[3];
    int int_lo[3];   // fine indices whose centre passes the window (inclusive)
    int int_hi[3];
    int zbase;       // first fine z of the tile grid (multiple of mz, <= lo[2])
    int ntile[3];    // tiles along x, y, z
    int nreg[3];     // region extent hi - lo
    int pad;
    long long vox;        // region voxels
    long long stack_off;  // element offset of this block's [t][v] stack slice
    long long out_offset;
    long long out_stride[3];
};

// Tile work unit: block index and tile coordinates.
struct TileDesc {
    int block, tx, ty, tz;
};

// Deduplicated ring and its factorisation per axis. The n^2 ring samples of
// kernel.cu:23-33 collapse to distinct points (62 for n = 12) with integer
// multiplicities; distinct x / y / z coordinate values index the separable
// Catmull-Rom weight tables.
struct RingPlan {
    int n = 0;                     // samples per angle (2 * AxesinRing)
    std::vector<float> xv, yv, zv; // distinct coordinate values per axis
    // Point list grouped by x value, then y value: group g covers pairs
    // [grp[g], grp[g+1]); pair p covers points [pair_pt[p], pair_pt[p+1]).
    std::vector<int> grp_xval;     // per group: x value index
    std::vector<int> grp;          // ngroups + 1
    std::vector<int> pair_yval;    // per pair: y value index
    std::vector<int> pair_pt;      // npairs + 1
    std::vector<int> pt_zval;      // per point: z value index
    std::vector<float> pt_vec;     // per point: h, c, multiplicity/n, -|u| (u = (x, y, z)/radius
                                   // = |u| (h x' + c z) in the pair's rotated frame)
    std::vector<float> pair_rot;   // per pair: x' = (ux, uy)/|(ux, uy)|, (1, 0) on the z axis
    int zero_x = -1, zero_y = -1;  // value index of 0 on x and y
    int npoints_raw = 0;
    // Raw float ring (n*n points) exactly as the reference builds it.
    std::vector<float> rx, ry, rz;
};

// Device-side tables (one contiguous buffer), offsets in 4-byte words.
struct TableLayout {
    int wx, offx, wy, offy, wz, offz, wzi, grp_xval, grp, pair_yval, pair_pt, pt_zval, pt_vec, pair_rot;
    int words;
};

// Everything the radiality kernel needs; passed by value.
struct RadParams {
    const void* in;       // input volume [t][z][y][x]
    int W, H, D, T;       // full input dims
    int mag[3];
    int nxv, nyv, nzv;    // distinct ring values per axis
    int ngroups, npairs, npoints;
    int zero_pair;        // pair index of (x=0, y=0), carries the intensity
    int gr[4];            // gradient ranges: main, x, y, z (smooth=0 => 1,0,0,0)
    int grad_mode;        // 1: ranges (1,1,1,1), 2: (1,0,0,0), 0: generic loops
    int R;                // gradient halo
    int TY;               // subvoxel rows per tile (threads = 8 * TY)
    int NU, NV, NW;       // coarse G tile extents
    int NIX, NIY, NIZ;    // input tile extents (G tile + halo)
    int renorm, poscon;
    int t_chunk, nchunks;
    int ntiles;
    long long nitems;
    const float* tables;  // TableLayout words
    TableLayout tl;
    const BlockDev* blocks;
    const TileDesc* tiles;
    float* rad_stack;     // [block slice][t][v]
    float* int_stack;
    unsigned int* work_counter;
    int smem_table_words;
    // TMA staging of the input tile (forward only): box width in elements
    // (0 = no staging area) and whether this launch uses it
    int tma_bx;
    int use_tma;
    unsigned long long* err;  // bounded-wait failures (may be null)
    // failure-detection test (RFBA_TEST_TMA_STALL): the first copy request of
    // every work item is left out, so the bounded staging wait gives up
    int test_skip_copy;
    // time window of this launch: volumes [t_lo, t_hi) (t_hi 0: up to T), and
    // the volume held by the first [t] row of the stacks (0 when they hold the
    // whole series, t_lo when they hold one batch)
    int t_lo, t_hi, stack_t0;
};

// Temporal reduction parameters.
struct TemporalParams {
    const BlockDev* blocks;
    const long long* vox_prefix;  // nblocks + 1 cumulative region voxels
    int nblocks;
    long long total_vox;
    int T;
    int method, itc, order, iw;
    float* rad_stack;             // ITC=1 bins the series in place
    const float* int_stack;
    float* out;
};

// Temporal reduction of one time batch into the carried state
// (temporal_stream.cu).
struct StreamParams {
    const BlockDev* blocks;
    const long long* vox_prefix;
    int nblocks;
    long long total_vox;
    int T;                 // the whole series
    int t_lo, t_hi;        // this batch; the stacks hold its [t_hi - t_lo][v]
    int method, order, iw;
    int last;              // write the map after this batch
    int keep;              // after the last batch, store the state as well (for a backward)
    float* state;          // [field][state_stride]
    long long state_stride;
    const float* rad_stack;
    const float* int_stack;
    float* out;
};

// Adjoint of the carried temporal reduction for one batch of one block
// (temporal_stream.cu): dL/dS and dL/dI of the volumes [t_lo, t_hi) from
// dL/dmap, the final carried state and the window stacks [w_lo, w_hi).
struct StreamAdjParams {
    const BlockDev* block;  // stack_off 0
    int T, t_lo, t_hi, w_lo, w_hi;
    int method, order, iw, renorm, poscon;
    const float* state;
    long long state_stride;
    const float* rad;    // [t - w_lo][v]
    const float* inten;
    const float* gmap;
    long long nmap;
    float* gS;           // [t - t_lo][v]
    float* gI;
    unsigned long long* err;
};

// Adjoint inputs and output of the radiality adjoint kernel.
struct AdjParams {
    const float* gS;  // dL/d(radiality before transforms) per subvoxel and time, [t][v]
    const float* gI;  // dL/d(interpolated intensity), [t][v]
    float* gin;       // dL/dI' accumulated, [t][z][y][x] of the full input
    long long n_in;   // elements of the input / gin
    long long n_stack;  // elements of gS / gI
    unsigned long long* err;  // first out-of-range global index (site << 56 | index), 0 if none
};

// Launchers (radiality.cu / temporal.cu / adjoint.cu). Return a cudaError_t as int.
int launch_radiality_adjoint(const RadParams& p, const AdjParams& a, int grid, size_t smem, void* stream);
size_t radiality_adjoint_smem_bytes(const RadParams& p);
int radiality_adjoint_max_ctas_per_sm(const RadParams& p, int* out);
int launch_temporal_adjoint(const BlockDev* blocks, long long vox, const float* rad, const float* inten,
                            const float* gmap, int T, int method, int itc, int order, int iw, int renorm, int poscon,
                            float* gS, float* gI, long long nmap, unsigned long long* err, void* stream);
int launch_shift_axis(const float* src, float* dst, int W, int H, int D, int T, int axis, const float* shifts, int mode,
                      unsigned long long* err, void* stream);
// Drift operator, all axes fused: mode 0 resamples src into dst; mode 1 adds
// sum_voxels g * dI'/dd_a into out[3 t + a] (FP64).
int launch_drift3d(const float* src, float* dst, const float* g, int W, int H, int D, int T, const float* shifts,
                   int mode, double* out, unsigned long long* err, void* stream);
int launch_drift_dot(const float* g, const float* dv, long long nv, int T, int axis, double* out,
                     unsigned long long* err, void* stream);
int launch_double_to_float(const double* src, float* dst, int n, void* stream);
int launch_radiality(const RadParams& p, int grid, size_t smem, int in_u16, void* stream);
// Box width (elements) of the TMA input staging for this tile, 0 when the input
// rows cannot be addressed by a tensor map (row pitch not a multiple of 16 B).
int radiality_tma_box_x(const RadParams& p, int in_u16);
size_t radiality_smem_bytes(const RadParams& p);
int tile_rows_for_mag(int my);
int radiality_max_ctas_per_sm(const RadParams& p, int in_u16, int* out);
int launch_temporal(const TemporalParams& p, void* stream);
int launch_temporal_stream(const StreamParams& p, void* stream);
int launch_temporal_stream_adjoint(const StreamAdjParams& p, long long vox, void* stream);
// state floats per subvoxel for a method (0 TRM, 1 TRA, 2 TRPPM, 3 TRAC ITC 0) and TRAC order
int temporal_stream_fields(int method, int order);
int launch_combine(const double* spots, long long n, int zoom, int Xp, int Yp, int Zp, int r, int rz, int thr,
                   const uint16_t* psf, int Kx, int Ky, int Kz, unsigned int* hist, unsigned char* L,
                   unsigned short* S, unsigned long long* idx, unsigned int* val, unsigned long long cap,
                   unsigned long long* counters, unsigned long long* out, uint16_t* out16, void* stream);
int launch_seed_spots(const float* map, const int map_dims[3], int mag, const int* vox, long long nvox, int nspots,
                      unsigned long long seed, float* xyz, double* w, double* sums, double* carry,
                      unsigned long long* err, void* stream);

// Host planning (plan.cpp).
bool build_ring_plan(const rfba_srrf_config& c, RingPlan* rp, std::string* err);
bool build_tables(const rfba_srrf_config& c, const RingPlan& rp, std::vector<float>* words, TableLayout* tl,
                  std::string* err);
bool window_range(float ring_radius_dummy, const std::vector<float>& rcoord, int mag, int dim, int* lo, int* hi);
int fine_window_int(int mag, int dim, int* lo, int* hi);

void set_error(const std::string& msg);

// FP32 FMA throughput probe (probe.cu): best of three timed launches, TFLOP/s.
int probe_fp32_fma(int device, double* tflops);

// 3B Gibbs sampling of the spot states (gibbs.cu): one chain per launch,
// frames dealt out to co-resident CTAs (cooperative launch).
struct GibbsParams {
    const double* pix;        // [F][P] data
    const double* si;         // [K][P] each spot's intensity at every pixel
    const int* moff;          // [K + 1] mask offsets
    const int* midx;          // mask pixel indices
    int K, F, P;
    double A[9], pi[3];
    double variance;          // noise variance (when var_draw is null)
    const double* var_draw;   // [n_draws] variance of each draw, or null
    int sweeps;               // sweeps over all spots per draw
    int n_draws;
    unsigned long long seed;
    unsigned long long draw_base;  // counter offset of the first draw
    unsigned char* state;     // [K][F] current states, in/out
    double* cur;              // [F][P] current sample intensities, in/out
    double* em;               // [2][F][4] scratch: emission mantissas / exponents (two buffers)
    unsigned int* bar;        // grid barrier: count, generation (zeroed)
    unsigned long long* err;  // barrier failures (site << 56 | spot)
    unsigned char* out_state;  // [n_draws][K][F] or null
    double* out_int;           // [n_draws][F][P] or null
    int exclude_spot;          // >= 0: out_int without that spot where it is on (all pixels)
    double* out_err;           // [n_draws][F] sums of squared residuals, or null
    double* rec_lp;            // [K][F][2] log p(on), log p(off) of the first sweep, or null
    double* rec_filt;          // [K][F][3] filtering distribution of the first sweep, or null
};
size_t gibbs_smem_bytes(int F);
int gibbs_max_blocks(int F, int* out);
// chains_dev: nchains parameter sets in device memory, all with the same F.
int launch_gibbs(const GibbsParams* chains_dev, int nchains, int grid_per_chain, int F, void* stream);
int launch_spot_intensity(const int* pixels, int P, const double* spots, int K, double zf, double* out, void* stream);

// 3B sampled-background spot Hessian (hessian.cu). Sizes: tab [P][21],
// part [nc][S * F][22], gg [15], frame [S][F][20], out [S][20].
struct HessParams {
    const double* bg;      // [S][F][P] background samples (the spot taken off)
    const double* pix;     // [F][P] data
    const int* pixels;     // [P][3]
    const double* phi;     // [5] spot, device
    double zf, variance;
    double A[9], pi[3];
    int S, F, P, nc, bs;
    unsigned long long seed;
    double *tab, *part, *gg, *frame, *out;
};
int hessian_chunks(long long S, long long F, int P, int sm_count);
size_t hessian_ffbs_smem(int F);
int launch_spot_hessian(const HessParams& h, void* stream);
// The table, the per-(frame, sample) parts and sum g g^T only (part, gg);
// samples_hold_spot: the draws include the spot (e = data - sample).
int launch_hessian_parts(const HessParams& h, bool samples_hold_spot, void* stream);

// 3B spot gradient (threeb.cu): spot voxel table, emission sums per (sample,
// frame), forward algorithm per sample; res[s] = (gradient[5], log probability).
int launch_threeb(const double* bg, const double* pix, const int* pixels, int S, int F, int P, const double* phi_dev,
                  double zf, double variance, double c0, const double* A_dev, const double* pi_dev,
                  double* val, double* der, double* em, double* res, const float2* dfd, float2* vdf,
                  void* stream);
// The samples' residuals (data minus background) as double-floats [S][F][P],
// for the gradient-only evaluations of launch_threeb (dfd; vdf is [P][6]).
int launch_threeb_residual(const double* bg, const double* pix, int S, int F, int P, float2* dfd, void* stream);

}  // namespace rfba

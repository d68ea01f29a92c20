// C-ABI of librfba_srrf.so: the reference's GradientCalc exports
// (GradientCalc.cpp:169-178, kernel.cu:560) and the extended interface
// declared in include/rfba_srrf.h.
//
// The reference allocates and frees every buffer on every call and runs one
// block after another (kernel.cu:575-654, GradientCalc.cpp:144-160). Here a
// context owns the device buffers (grown on demand and kept), the ring plan and
// weight tables (cached per configuration), and launches every block of a call
// in one persistent radiality kernel followed by one temporal kernel per pass.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <set>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <limits>
#include <mutex>
#include <string>
#include <vector>

#include "cg_only.h"
#include "devbuf.h"
#include "srrf_internal.h"

namespace rfba {

void config_default(rfba_srrf_config* c);
bool config_load_ini(const char* path, rfba_srrf_config* c);
bool config_validate(const rfba_srrf_config& c, std::string* err);
int ring_zero_pair(const RingPlan& rp);
int blocks_gradientcalc(const rfba_srrf_config& c, const int dims[4], rfba_block* out, int cap, std::string* err);
int blocks_dosplit(const rfba_srrf_config& c, const int dims[4], const int max_size[3], int border, rfba_block* out,
                   int cap, long long* out_elems, std::string* err);

static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }

// RFBA_CHECKS=1: the differentiable path reads back its kernels' bounds checks
// after each call (synchronising) and fails on an out-of-range index.
static bool checks_enabled() {
    static int v = -1;
    if (v < 0) {
        const char* e = std::getenv("RFBA_CHECKS");
        v = (e && *e && *e != '0') ? 1 : 0;
    }
    return v == 1;
}

static int test_tma_stall();
static int device_status(rfba_ctx* ctx, cudaStream_t st, const char* what);

static bool verbose() {
    static int v = -1;
    if (v < 0) {
        const char* e = std::getenv("RFBA_VERBOSE");
        v = (e && *e && *e != '0') ? 1 : 0;
    }
    return v == 1;
}

static int cuda_fail(cudaError_t e, const char* what) {
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? RFBA_ERR_NOMEM : RFBA_ERR_CUDA;
}

#define RFBA_CUDA(call, what)                          \
    do {                                               \
        cudaError_t e__ = (call);                      \
        if (e__ != cudaSuccess) return cuda_fail(e__, what); \
    } while (0)

struct PlanCache {
    bool valid = false;
    float ring_radius = 0.f;
    int axes = 0, mag[3] = {0, 0, 0};
    RingPlan ring;
    std::vector<float> words;
    TableLayout tl;
    int zero_pair = -1;
};

// Schedule choices of the forward: tile rows (tile shape) and tile order
// (block-to-CTA schedule). 0 = defaults.
struct Tuning {
    int ty = 0;
    int order = 0;  // 0: largest blocks first, raster inside a block; 1: tiles interleaved across blocks
};

// One pass = the blocks whose radiality + intensity stacks fit the budget
// together; lists of all passes are concatenated (tile block indices are
// relative to the pass's first block).
struct PassPlan {
    size_t b0 = 0, b1 = 0, t0 = 0, t1 = 0, p0 = 0;
    long long stack_elems = 0;
    int chunk = 1, nchunks = 1, grid = 1;
    size_t smem = 0;
    long long nitems = 0, units = 0;
};
struct PassSet {
    std::vector<BlockDev> blocks;
    std::vector<TileDesc> tiles;
    std::vector<long long> prefix;
    std::vector<PassPlan> passes;
    long long max_stack = 0;
    int ty = 0;
};


// A captured forward: the whole launch sequence of one call (copies, clears,
// all passes) replayed with one cudaGraphLaunch while the call's arguments and
// the scratch it was captured on are unchanged.
struct GraphPlan {
    std::string key;
    std::vector<const void*> deps;  // scratch pointers baked into the graph
    cudaGraphExec_t exec = nullptr;
    PassSet ps;
    DevBuf blocks, tiles, prefix, counters;
    std::vector<cudaEvent_t> evs;
    ~GraphPlan() {
        if (exec) cudaGraphExecDestroy(exec);
        for (cudaEvent_t e : evs) cudaEventDestroy(e);
        blocks.release();
        tiles.release();
        prefix.release();
        counters.release();
    }
};

}  // namespace rfba

struct rfba_ctx {
    int device = 0;
    int sm_count = 0;
    size_t budget = 0;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    rfba::DevBuf in, out, rad, inten, blocks, tiles, tables, counter, prefix;
    rfba::PlanCache plan;
    bool timing = false;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // calls share the scratch: a call on another stream than the previous call
    // first waits for that call's work
    cudaEvent_t xev = nullptr;
    cudaStream_t last_stream = nullptr;
    bool have_last = false;
    double last_rad_ms = 0.0, last_temporal_ms = 0.0;
    long long launches = 0;
    long long last_flop_units = 0;  // subvoxel-time-points computed by the last call
    int grid_override = 0;          // CTAs for the radiality kernel (0 = occupancy x SMs)
    int chunk_override = 0;         // time points per work item (0 = automatic)
    int last_passes = 0;            // passes of the last forward (1 = its stacks are all resident)
    // differentiable path: buffers and the forward the backward can reuse
    rfba::DevBuf shifted, tmp1, tmp2, gS, gI, gin, dshift, ablocks, atiles, acounter, errw;
    struct Train {
        bool valid = false;
        rfba_srrf_config cfg;
        int dims[4] = {0, 0, 0, 0};
        const void* in = nullptr;
        const void* shifts = nullptr;
        const float* iprime = nullptr;
        rfba::BlockDev blk;
    } train;
    double last_backward_ms = 0.0;
    // forward schedule: per-pass timing events, autotuned schedules, captured graphs
    std::vector<cudaEvent_t> pev;
    cudaStream_t cap = nullptr;  // stream the graphs are captured on
    std::map<std::string, std::pair<int, int>> tunes;  // schedule key -> (tile rows, tile order)
    std::vector<std::unique_ptr<rfba::GraphPlan>> graphs;  // most recent first
    // spot seeding scratch
    rfba::DevBuf seed_w, seed_sums, seed_carry, seed_map, seed_vox, seed_xyz;
    // 3B spot-gradient scratch
    rfba::DevBuf tb_val, tb_der, tb_em, tb_res, tb_par, tb_bg, tb_pix, tb_pixels;
    // 3B Gibbs sampler scratch
    rfba::DevBuf gb_pix, gb_pixels, gb_spots, gb_si, gb_moff, gb_midx, gb_state, gb_cur, gb_em, gb_bar, gb_var,
        gb_ostate, gb_oint, gb_oerr, gb_lp, gb_filt;
    int last_ty = 0, last_order = 0, last_graph = 0, last_tuned = 0;
};

namespace rfba {

static int ctx_init(rfba_ctx* c, int device, size_t budget) {
    c->device = device;
    RFBA_CUDA(cudaSetDevice(device), "cudaSetDevice");
    RFBA_CUDA(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device), "SM count");
    RFBA_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream");
    for (auto& e : c->ev) RFBA_CUDA(cudaEventCreate(&e), "event");
    RFBA_CUDA(cudaEventCreateWithFlags(&c->xev, cudaEventDisableTiming), "event");
    if (budget == 0) {
        size_t fr = 0, tot = 0;
        RFBA_CUDA(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
        budget = fr / 4;
    }
    c->budget = budget;
    // device-side status word, zero until a kernel records a failure
    if (int s = c->errw.ensure(256, "status word")) return s;
    RFBA_CUDA(cudaMemset(c->errw.p, 0, 256), "status word clear");
    return RFBA_OK;
}

static rfba_ctx* g_default = nullptr;
static std::mutex g_default_mu;

static int default_ctx(rfba_ctx** out) {
    std::lock_guard<std::mutex> lk(g_default_mu);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (g_default && g_default->device != dev) {
        // the reference always used the current device; follow it
        g_default = nullptr;
    }
    if (!g_default) {
        rfba_ctx* c = new rfba_ctx();
        int st = ctx_init(c, dev, 0);
        if (st != RFBA_OK) {
            delete c;
            return st;
        }
        g_default = c;
    }
    *out = g_default;
    return RFBA_OK;
}

static int ensure_plan(rfba_ctx* ctx, const rfba_srrf_config& cfg, cudaStream_t st) {
    PlanCache& P = ctx->plan;
    if (P.valid && P.ring_radius == cfg.ring_radius && P.axes == cfg.axes_in_ring && P.mag[0] == cfg.mag[0] &&
        P.mag[1] == cfg.mag[1] && P.mag[2] == cfg.mag[2])
        return RFBA_OK;
    std::string err;
    P.valid = false;
    if (!build_ring_plan(cfg, &P.ring, &err) || !build_tables(cfg, P.ring, &P.words, &P.tl, &err)) {
        set_error(err);
        return RFBA_ERR_UNSUPPORTED;
    }
    P.zero_pair = ring_zero_pair(P.ring);
    if (P.zero_pair < 0) {
        set_error("ring has no (0, 0) pair");
        return RFBA_ERR_UNSUPPORTED;
    }
    const int rc = ctx->tables.ensure(P.words.size() * 4, "tables");
    if (rc) return rc;
    RFBA_CUDA(cudaMemcpyAsync(ctx->tables.p, P.words.data(), P.words.size() * 4, cudaMemcpyHostToDevice, st),
              "tables upload");
    P.ring_radius = cfg.ring_radius;
    P.axes = cfg.axes_in_ring;
    for (int a = 0; a < 3; ++a) P.mag[a] = cfg.mag[a];
    P.valid = true;
    return RFBA_OK;
}

static int fz_for(int mz) { return mz * cz_for_mag(mz); }

// Order this call's work after the previous call's when the streams differ.
static int order_streams(rfba_ctx* ctx, cudaStream_t st) {
    if (ctx->have_last && ctx->last_stream != st) {
        RFBA_CUDA(cudaEventRecord(ctx->xev, ctx->last_stream), "stream order event");
        RFBA_CUDA(cudaStreamWaitEvent(st, ctx->xev, 0), "stream order wait");
    }
    ctx->last_stream = st;
    ctx->have_last = true;
    return RFBA_OK;
}

// Turn caller blocks into device block descriptors, splitting regions along z
// so that one pass's radiality + intensity stack fits the scratch budget.
static int make_blocks(rfba_ctx* ctx, const rfba_srrf_config& cfg, const int dims[4], const rfba_block* blocks,
                       int nblocks, std::vector<BlockDev>* outb, int ty = 0) {
    const RingPlan& rp = ctx->plan.ring;
    const int T = dims[3];
    const int FZ = fz_for(cfg.mag[2]);
    outb->clear();
    const size_t per_vox = (size_t)T * 2 * sizeof(float);
    const long long max_vox = std::max<long long>((long long)(ctx->budget / per_vox), 1);
    for (int i = 0; i < nblocks; ++i) {
        const rfba_block& b = blocks[i];
        BlockDev d;
        std::memset(&d, 0, sizeof d);
        for (int a = 0; a < 3; ++a) {
            if (b.size[a] < 1 || b.origin[a] < 0 || (long long)b.origin[a] + b.size[a] > dims[a]) {
                set_error("block outside the input volume");
                return RFBA_ERR_INVALID;
            }
            if (b.lo[a] < 0 || b.hi[a] > b.size[a] * cfg.mag[a]) {
                set_error("block region outside the block's magnified grid");
                return RFBA_ERR_INVALID;
            }
            d.origin[a] = b.origin[a];
            d.size[a] = b.size[a];
            d.lo[a] = b.lo[a];
            d.hi[a] = b.hi[a];
            const std::vector<float>& rc = a == 0 ? rp.rx : (a == 1 ? rp.ry : rp.rz);
            window_range(cfg.ring_radius, rc, cfg.mag[a], b.size[a], &d.rad_lo[a], &d.rad_hi[a]);
            fine_window_int(cfg.mag[a], b.size[a], &d.int_lo[a], &d.int_hi[a]);
        }
        if (b.hi[0] <= b.lo[0] || b.hi[1] <= b.lo[1] || b.hi[2] <= b.lo[2]) continue;
        d.out_offset = b.out_offset;
        for (int a = 0; a < 3; ++a) d.out_stride[a] = b.out_stride[a];
        // z slabs under the budget
        const long long plane = (long long)(b.hi[0] - b.lo[0]) * (b.hi[1] - b.lo[1]);
        long long slab = std::max<long long>(max_vox / plane, 1);
        if (slab < b.hi[2] - b.lo[2]) slab = std::max<long long>((slab / FZ) * FZ, FZ);
        for (int z0 = b.lo[2]; z0 < b.hi[2]; z0 += (int)slab) {
            BlockDev s = d;
            s.lo[2] = z0;
            s.hi[2] = (int)std::min<long long>(b.hi[2], z0 + slab);
            s.out_offset = d.out_offset + (long long)(z0 - b.lo[2]) * d.out_stride[2];
            for (int a = 0; a < 3; ++a) s.nreg[a] = s.hi[a] - s.lo[a];
            s.zbase = (s.lo[2] / cfg.mag[2]) * cfg.mag[2];
            const int TY = ty > 0 ? ty : tile_rows_for_mag(cfg.mag[1]);
            s.ntile[0] = (s.nreg[0] + kTileX - 1) / kTileX;
            s.ntile[1] = (s.nreg[1] + TY - 1) / TY;
            s.ntile[2] = (s.hi[2] - s.zbase + FZ - 1) / FZ;
            s.vox = (long long)s.nreg[0] * s.nreg[1] * s.nreg[2];
            outb->push_back(s);
        }
    }
    return RFBA_OK;
}

static size_t elem_size(rfba_dtype dt) { return dt == RFBA_U16 ? 2 : 4; }

// Kernel parameters common to the forward and adjoint radiality kernels
// (everything but the block / tile lists and the schedule).
static RadParams fill_rad_params(rfba_ctx* ctx, const rfba_srrf_config& cfg, const void* in_dev, const int dims[4],
                                 int CZ, int ty = 0) {
    const PlanCache& P = ctx->plan;
    const int T = dims[3];
    RadParams rp;
    std::memset(&rp, 0, sizeof rp);
    rp.in = in_dev;
    rp.W = dims[0];
    rp.H = dims[1];
    rp.D = dims[2];
    rp.T = T;
    for (int a = 0; a < 3; ++a) rp.mag[a] = cfg.mag[a];
    rp.nxv = (int)P.ring.xv.size();
    rp.nyv = (int)P.ring.yv.size();
    rp.nzv = (int)P.ring.zv.size();
    rp.ngroups = (int)P.ring.grp_xval.size();
    rp.npairs = (int)P.ring.pair_yval.size();
    rp.npoints = (int)P.ring.pt_zval.size();
    rp.zero_pair = P.zero_pair;
    if (cfg.gradient_smooth == 0) {
        rp.gr[0] = 1;
        rp.gr[1] = rp.gr[2] = rp.gr[3] = 0;
    } else {
        rp.gr[0] = cfg.main_range;
        rp.gr[1] = cfg.x_range;
        rp.gr[2] = cfg.y_range;
        rp.gr[3] = cfg.z_range;
    }
    rp.R = std::max(std::max(rp.gr[0], rp.gr[1]), std::max(rp.gr[2], rp.gr[3]));
    if (rp.gr[0] == 1 && rp.gr[1] == 1 && rp.gr[2] == 1 && rp.gr[3] == 1)
        rp.grad_mode = 1;
    else if (rp.gr[0] == 1 && rp.gr[1] == 0 && rp.gr[2] == 0 && rp.gr[3] == 0)
        rp.grad_mode = 2;
    else
        rp.grad_mode = 0;
    rp.TY = ty > 0 ? ty : tile_rows_for_mag(cfg.mag[1]);
    rp.NU = (kTileX - 1) / cfg.mag[0] + 2 + 4;
    rp.NV = (rp.TY - 1) / cfg.mag[1] + 2 + 4;
    rp.NW = CZ + 4;
    rp.NIX = rp.NU + 2 * rp.R;
    rp.NIY = rp.NV + 2 * rp.R;
    rp.NIZ = rp.NW + 2 * rp.R;
    rp.renorm = cfg.renormalize == 1;
    rp.poscon = cfg.remove_con == 1;
    rp.tables = static_cast<const float*>(ctx->tables.p);
    rp.tl = P.tl;
    rp.smem_table_words = P.tl.words;
    return rp;
}

static int plan_passes(rfba_ctx* ctx, const rfba_srrf_config& cfg, rfba_dtype dtype, const int dims[4],
                       const std::vector<BlockDev>& all, const Tuning& tune, PassSet* ps) {
    const int T = dims[3];
    const size_t per_vox = (size_t)T * sizeof(float);
    ps->blocks.clear();
    ps->tiles.clear();
    ps->prefix.clear();
    ps->passes.clear();
    ps->max_stack = 0;
    ps->ty = tune.ty > 0 ? tune.ty : tile_rows_for_mag(cfg.mag[1]);
    RadParams rp = fill_rad_params(ctx, cfg, nullptr, dims, cz_for_mag(cfg.mag[2]), ps->ty);
    rp.tma_bx = radiality_tma_box_x(rp, dtype == RFBA_U16);
    const size_t smem = radiality_smem_bytes(rp);
    if (smem > 227 * 1024) {
        set_error("shared memory tile too large for this configuration");
        return RFBA_ERR_UNSUPPORTED;
    }
    int per_sm = 0;
    int ce = radiality_max_ctas_per_sm(rp, dtype == RFBA_U16, &per_sm);
    if (ce != 0) return cuda_fail((cudaError_t)ce, "occupancy");
    if (per_sm < 1) {
        set_error("radiality kernel does not fit on an SM");
        return RFBA_ERR_UNSUPPORTED;
    }
    const int slots = per_sm * ctx->sm_count;
    size_t i0 = 0;
    while (i0 < all.size()) {
        size_t i1 = i0;
        long long vox = 0;
        while (i1 < all.size()) {
            const long long nv = vox + all[i1].vox;
            if (i1 > i0 && (size_t)nv * per_vox * 2 > ctx->budget) break;
            vox = nv;
            ++i1;
        }
        PassPlan pp;
        pp.b0 = ps->blocks.size();
        pp.t0 = ps->tiles.size();
        pp.p0 = ps->prefix.size();
        long long off = 0, pre = 0;
        ps->prefix.push_back(0);
        for (size_t b = i0; b < i1; ++b) {
            BlockDev d = all[b];
            d.stack_off = off;
            off += d.vox * T;
            pre += d.vox;
            ps->prefix.push_back(pre);
            ps->blocks.push_back(d);
        }
        const int nb = (int)(i1 - i0);
        const BlockDev* pb = ps->blocks.data() + pp.b0;
        auto ntiles = [&](int b) { return (long long)pb[b].ntile[0] * pb[b].ntile[1] * pb[b].ntile[2]; };
        if (tune.order == 1) {
            // round robin over blocks, one tile at a time
            long long most = 0;
            for (int b = 0; b < nb; ++b) most = std::max(most, ntiles(b));
            for (long long k = 0; k < most; ++k)
                for (int b = 0; b < nb; ++b) {
                    if (k >= ntiles(b)) continue;
                    const int tx = (int)(k % pb[b].ntile[0]);
                    const int ty = (int)((k / pb[b].ntile[0]) % pb[b].ntile[1]);
                    const int tz = (int)(k / ((long long)pb[b].ntile[0] * pb[b].ntile[1]));
                    ps->tiles.push_back({b, tx, ty, tz});
                }
        } else {
            // largest blocks first for balance, raster order inside a block
            std::vector<int> order(nb);
            for (int b = 0; b < nb; ++b) order[b] = b;
            std::stable_sort(order.begin(), order.end(), [&](int u, int v) { return ntiles(u) > ntiles(v); });
            for (int b : order)
                for (int tz = 0; tz < pb[b].ntile[2]; ++tz)
                    for (int ty = 0; ty < pb[b].ntile[1]; ++ty)
                        for (int tx = 0; tx < pb[b].ntile[0]; ++tx) ps->tiles.push_back({b, tx, ty, tz});
        }
        pp.b1 = ps->blocks.size();
        pp.t1 = ps->tiles.size();
        pp.stack_elems = off;
        pp.units = vox * T;
        const long long nt = (long long)(pp.t1 - pp.t0);
        // time chunk: enough work items for ~8 per CTA slot
        int chunk = ctx->chunk_override;
        if (chunk <= 0) {
            const long long want = 8LL * slots;
            long long nch = (want + nt - 1) / nt;
            nch = std::max<long long>(1, std::min<long long>(nch, T));
            chunk = (int)((T + nch - 1) / nch);
        }
        pp.chunk = chunk;
        pp.nchunks = (T + chunk - 1) / chunk;
        pp.nitems = nt * pp.nchunks;
        int grid = ctx->grid_override > 0 ? ctx->grid_override : slots;
        grid = (int)std::min<long long>(grid, pp.nitems);
        pp.grid = std::max(grid, 1);
        pp.smem = smem;
        ps->max_stack = std::max(ps->max_stack, off);
        ps->passes.push_back(pp);
        i0 = i1;
    }
    return RFBA_OK;
}

// Queue the passes on st: counter reset, radiality, temporal per pass. The
// device lists hold ps's concatenated blocks / tiles / prefixes; evs (3 per
// pass) are recorded around the kernels when given.
static int enqueue_passes(rfba_ctx* ctx, const rfba_srrf_config& cfg, const void* in_dev, rfba_dtype dtype,
                          const int dims[4], const PassSet& ps, const BlockDev* dblocks, const TileDesc* dtiles,
                          const long long* dprefix, unsigned int* dcounters, float* out_dev, cudaStream_t st,
                          const cudaEvent_t* evs, bool capturing = false) {
    // inside a stream capture the events become event-record nodes of the graph
    auto rec = [&](cudaEvent_t e) {
        return capturing ? cudaEventRecordWithFlags(e, st, cudaEventRecordExternal) : cudaEventRecord(e, st);
    };
    for (size_t i = 0; i < ps.passes.size(); ++i) {
        const PassPlan& pp = ps.passes[i];
        unsigned int* counter = dcounters + 64 * i;
        RFBA_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned int), st), "counter reset");
        RadParams rp = fill_rad_params(ctx, cfg, in_dev, dims, cz_for_mag(cfg.mag[2]), ps.ty);
        rp.tma_bx = radiality_tma_box_x(rp, dtype == RFBA_U16);
        rp.err = static_cast<unsigned long long*>(ctx->errw.p);
        rp.test_skip_copy = test_tma_stall();
        rp.blocks = dblocks + pp.b0;
        rp.tiles = dtiles + pp.t0;
        rp.ntiles = (int)(pp.t1 - pp.t0);
        rp.rad_stack = static_cast<float*>(ctx->rad.p);
        rp.int_stack = static_cast<float*>(ctx->inten.p);
        rp.work_counter = counter;
        rp.t_chunk = pp.chunk;
        rp.nchunks = pp.nchunks;
        rp.nitems = pp.nitems;
        TemporalParams tp;
        std::memset(&tp, 0, sizeof tp);
        tp.blocks = rp.blocks;
        tp.vox_prefix = dprefix + pp.p0;
        tp.nblocks = (int)(pp.b1 - pp.b0);
        tp.total_vox = ps.prefix[pp.p0 + (pp.b1 - pp.b0)];
        tp.T = dims[3];
        tp.method = cfg.method;
        tp.itc = cfg.itc;
        tp.order = cfg.trac_order;
        tp.iw = cfg.intensity_w;
        tp.rad_stack = rp.rad_stack;
        tp.int_stack = rp.int_stack;
        tp.out = out_dev;
        if (evs) RFBA_CUDA(rec(evs[3 * i]), "event");
        int le = launch_radiality(rp, pp.grid, pp.smem, dtype == RFBA_U16, st);
        if (le != 0) return cuda_fail((cudaError_t)le, "radiality launch");
        if (evs) RFBA_CUDA(rec(evs[3 * i + 1]), "event");
        le = launch_temporal(tp, st);
        if (le != 0) return cuda_fail((cudaError_t)le, "temporal launch");
        if (evs) RFBA_CUDA(rec(evs[3 * i + 2]), "event");
        if (verbose())
            std::fprintf(stderr, "rfba: pass blocks=%zu tiles=%d ty=%d chunk=%d items=%lld grid=%d smem=%zu\n",
                         pp.b1 - pp.b0, rp.ntiles, ps.ty, pp.chunk, pp.nitems, pp.grid, pp.smem);
    }
    return RFBA_OK;
}

static int ensure_events(std::vector<cudaEvent_t>* evs, size_t n) {
    while (evs->size() < n) {
        cudaEvent_t e;
        RFBA_CUDA(cudaEventCreate(&e), "event");
        evs->push_back(e);
    }
    return RFBA_OK;
}

// Per-pass kernel times from the events of the last run.
static int collect_timing(rfba_ctx* ctx, const PassSet& ps, const std::vector<cudaEvent_t>& evs) {
    ctx->last_rad_ms = ctx->last_temporal_ms = 0.0;
    for (size_t i = 0; i < ps.passes.size(); ++i) {
        RFBA_CUDA(cudaEventSynchronize(evs[3 * i + 2]), "event sync");
        float a = 0.f, b = 0.f;
        RFBA_CUDA(cudaEventElapsedTime(&a, evs[3 * i], evs[3 * i + 1]), "event time");
        RFBA_CUDA(cudaEventElapsedTime(&b, evs[3 * i + 1], evs[3 * i + 2]), "event time");
        ctx->last_rad_ms += a;
        ctx->last_temporal_ms += b;
    }
    return RFBA_OK;
}

static void account(rfba_ctx* ctx, const PassSet& ps) {
    ctx->last_passes = (int)ps.passes.size();
    ctx->launches += 2 * (long long)ps.passes.size();
    ctx->last_flop_units = 0;
    for (const PassPlan& pp : ps.passes) ctx->last_flop_units += pp.units;
}

// Run the device pipeline for all blocks now (no graph). in_dev / out_dev are
// device pointers.
static int run_device(rfba_ctx* ctx, const rfba_srrf_config& cfg, const void* in_dev, rfba_dtype dtype,
                      const int dims[4], const std::vector<BlockDev>& all, float* out_dev, cudaStream_t st,
                      const Tuning& tune = Tuning()) {
    ctx->train.valid = false;
    PassSet ps;
    int s;
    if ((s = ctx->errw.ensure(256, "check word"))) return s;
    if ((s = plan_passes(ctx, cfg, dtype, dims, all, tune, &ps))) return s;
    const size_t np = ps.passes.size();
    if ((s = ctx->rad.ensure((size_t)ps.max_stack * 4, "radiality stack"))) return s;
    if ((s = ctx->inten.ensure((size_t)ps.max_stack * 4, "intensity stack"))) return s;
    if ((s = ctx->blocks.ensure(ps.blocks.size() * sizeof(BlockDev), "blocks"))) return s;
    if ((s = ctx->tiles.ensure(ps.tiles.size() * sizeof(TileDesc), "tiles"))) return s;
    if ((s = ctx->prefix.ensure(ps.prefix.size() * sizeof(long long), "prefix"))) return s;
    if ((s = ctx->counter.ensure(np * 256, "counter"))) return s;
    RFBA_CUDA(cudaMemcpyAsync(ctx->blocks.p, ps.blocks.data(), ps.blocks.size() * sizeof(BlockDev),
                              cudaMemcpyHostToDevice, st), "blocks upload");
    RFBA_CUDA(cudaMemcpyAsync(ctx->tiles.p, ps.tiles.data(), ps.tiles.size() * sizeof(TileDesc),
                              cudaMemcpyHostToDevice, st), "tiles upload");
    RFBA_CUDA(cudaMemcpyAsync(ctx->prefix.p, ps.prefix.data(), ps.prefix.size() * sizeof(long long),
                              cudaMemcpyHostToDevice, st), "prefix upload");
    if (ctx->timing && (s = ensure_events(&ctx->pev, 3 * np))) return s;
    if ((s = enqueue_passes(ctx, cfg, in_dev, dtype, dims, ps, static_cast<const BlockDev*>(ctx->blocks.p),
                            static_cast<const TileDesc*>(ctx->tiles.p), static_cast<const long long*>(ctx->prefix.p),
                            static_cast<unsigned int*>(ctx->counter.p), out_dev, st,
                            ctx->timing ? ctx->pev.data() : nullptr)))
        return s;
    account(ctx, ps);
    if (ctx->timing && (s = collect_timing(ctx, ps, ctx->pev))) return s;
    return RFBA_OK;
}

static int validate_common(const rfba_srrf_config* cfg, const void* in, const int* dims, const void* out) {
    if (!cfg || !in || !dims || !out) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    std::string err;
    if (!config_validate(*cfg, &err)) {
        set_error(err);
        return RFBA_ERR_INVALID;
    }
    for (int a = 0; a < 4; ++a)
        if (dims[a] < 1) {
            set_error("dims must be positive");
            return RFBA_ERR_INVALID;
        }
    const long long plane = (long long)dims[0] * dims[1] * dims[2];
    if (plane * dims[3] > (1LL << 40)) {
        set_error("input too large");
        return RFBA_ERR_INVALID;
    }
    return RFBA_OK;
}

static int forward_blocks_locked(rfba_ctx* ctx, const rfba_srrf_config* cfg, const void* in, rfba_dtype dtype,
                                 const int dims[4], const rfba_block* blocks, int nblocks, float* out,
                                 long long out_elems, int flags, cudaStream_t st, bool zero_out, bool fast = false);

static int forward_blocks_impl(rfba_ctx* ctx, const rfba_srrf_config* cfg, const void* in, rfba_dtype dtype,
                               const int dims[4], const rfba_block* blocks, int nblocks, float* out, long long out_elems,
                               int flags, cudaStream_t st, bool zero_out, bool fast = false) {
    std::lock_guard<std::mutex> lk(ctx->mu);
    return forward_blocks_locked(ctx, cfg, in, dtype, dims, blocks, nblocks, out, out_elems, flags, st, zero_out,
                                 fast);
}

static bool env_on(const char* name, bool dflt) {
    const char* e = std::getenv(name);
    if (!e || !*e) return dflt;
    return !(e[0] == '0' && e[1] == 0);
}

// Failure-detection test hook (RFBA_TEST_TMA_STALL=1): the radiality kernel
// leaves out the first input copy request of every work item, so its bounded
// staging wait gives up and the call reports RFBA_ERR_TIMEOUT. Read per call.
static int test_tma_stall() { return env_on("RFBA_TEST_TMA_STALL", false) ? 1 : 0; }

// Calls below this many voxel-volumes keep the default schedule (RFBA_TUNE_MIN overrides).
static long long tune_min_work() {
    const char* e = std::getenv("RFBA_TUNE_MIN");
    return (e && *e) ? std::atoll(e) : 200000000LL;
}

static bool host_pinned(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

template <typename T>
static void key_put(std::string* k, const T* p, size_t n) {
    k->append(reinterpret_cast<const char*>(p), n * sizeof(T));
}

// Schedule key: what the best tile shape / order depends on.
static std::string sched_key(const rfba_srrf_config& cfg, rfba_dtype dtype, const int dims[4],
                             const rfba_block* blocks, int nblocks) {
    std::string k;
    key_put(&k, &cfg, 1);
    key_put(&k, &dtype, 1);
    key_put(&k, dims, 4);
    for (int i = 0; i < nblocks; ++i) {
        key_put(&k, blocks[i].size, 3);
        key_put(&k, blocks[i].lo, 3);
        key_put(&k, blocks[i].hi, 3);
    }
    return k;
}

// Autotuner: time every candidate schedule (tile rows valid for mag_y, and for
// block lists the two tile orders) on the first few volumes of this call's
// own input, keep the fastest.
static int autotune(rfba_ctx* ctx, const rfba_srrf_config& cfg, const void* in_dev, rfba_dtype dtype,
                    const int dims[4], const rfba_block* blocks, int nblocks, float* out_dev, cudaStream_t st,
                    Tuning* best) {
    const int my = cfg.mag[1];
    std::vector<int> tys;
    for (int ty : {8, 12, 16, 24})
        if (ty % (2 * my) == 0 && ty * (kTileX / 2) <= kMaxThreads) tys.push_back(ty);
    const int dty = tile_rows_for_mag(my);
    if (std::find(tys.begin(), tys.end(), dty) == tys.end()) tys.push_back(dty);
    std::vector<int> orders = {0};
    if (nblocks > 1) orders.push_back(1);
    const int sd[4] = {dims[0], dims[1], dims[2], std::min(dims[3], 3)};
    cudaEvent_t e0, e1;
    RFBA_CUDA(cudaEventCreate(&e0), "event");
    RFBA_CUDA(cudaEventCreate(&e1), "event");
    float best_ms = 0.f;
    int rc = RFBA_OK;
    bool have = false;
    const bool timing = ctx->timing;
    ctx->timing = false;
    for (int ty : tys) {
        for (int order : orders) {
            Tuning t;
            t.ty = ty;
            t.order = order;
            std::vector<BlockDev> all;
            if ((rc = make_blocks(ctx, cfg, sd, blocks, nblocks, &all, ty))) break;
            float ms = 0.f;
            for (int rep = 0; rep < 2 && !rc; ++rep) {
                if (rep == 1) cudaEventRecord(e0, st);
                rc = run_device(ctx, cfg, in_dev, dtype, sd, all, out_dev, st, t);
                if (rep == 1) cudaEventRecord(e1, st);
            }
            if (rc) break;
            if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
                rc = cuda_fail(cudaGetLastError(), "autotune timing");
                break;
            }
            if (verbose()) std::fprintf(stderr, "rfba: autotune ty=%d order=%d %.3f ms\n", ty, order, ms);
            if (!have || ms < best_ms) {
                best_ms = ms;
                *best = t;
                have = true;
            }
        }
        if (rc) break;
    }
    ctx->timing = timing;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

static int forward_blocks_locked(rfba_ctx* ctx, const rfba_srrf_config* cfg, const void* in, rfba_dtype dtype,
                                 const int dims[4], const rfba_block* blocks, int nblocks, float* out,
                                 long long out_elems, int flags, cudaStream_t st, bool zero_out, bool fast) {
    int s = validate_common(cfg, in, dims, out);
    if (s) return s;
    if (nblocks < 0 || (nblocks > 0 && !blocks) || out_elems < 0) {
        set_error("bad block list");
        return RFBA_ERR_INVALID;
    }
    if (dtype != RFBA_F32 && dtype != RFBA_U16) {
        set_error("dtype must be RFBA_F32 or RFBA_U16");
        return RFBA_ERR_INVALID;
    }
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    if ((s = order_streams(ctx, st))) return s;
    if ((s = ensure_plan(ctx, *cfg, st))) return s;
    std::vector<BlockDev> all;
    if ((s = make_blocks(ctx, *cfg, dims, blocks, nblocks, &all))) return s;
    long long work = 0;
    for (const BlockDev& b : all) {
        const long long last = b.out_offset + (long long)(b.nreg[0] - 1) * b.out_stride[0] +
                               (long long)(b.nreg[1] - 1) * b.out_stride[1] + (long long)(b.nreg[2] - 1) * b.out_stride[2];
        if (b.out_offset < 0 || last >= out_elems || b.out_stride[0] < 0 || b.out_stride[1] < 0 || b.out_stride[2] < 0) {
            set_error("block output outside the output array");
            return RFBA_ERR_INVALID;
        }
        work += b.vox * dims[3];
    }
    const size_t in_bytes = (size_t)dims[0] * dims[1] * dims[2] * dims[3] * elem_size(dtype);
    ctx->last_ty = tile_rows_for_mag(cfg->mag[1]);
    ctx->last_order = 0;
    ctx->last_graph = 0;
    ctx->last_tuned = 0;
    if (fast) {
        // schedule: autotuned once per (configuration, dims, block shapes)
        Tuning tune;
        const std::string tkey = sched_key(*cfg, dtype, dims, blocks, nblocks);
        auto it = ctx->tunes.find(tkey);
        if (it != ctx->tunes.end()) {
            tune.ty = it->second.first;
            tune.order = it->second.second;
        } else if (env_on("RFBA_TUNE", true) && work >= tune_min_work()) {
            const void* tin = in;
            float* tout = out;
            if (flags == RFBA_HOST_PTRS) {
                // the first volumes of the input are enough for the timing runs
                const size_t sample = (size_t)dims[0] * dims[1] * dims[2] * std::min(dims[3], 3) * elem_size(dtype);
                if ((s = ctx->in.ensure(in_bytes, "input"))) return s;
                if ((s = ctx->out.ensure((size_t)out_elems * 4, "output"))) return s;
                RFBA_CUDA(cudaMemcpyAsync(ctx->in.p, in, sample, cudaMemcpyHostToDevice, st), "input copy");
                tin = ctx->in.p;
                tout = static_cast<float*>(ctx->out.p);
            }
            if ((s = autotune(ctx, *cfg, tin, dtype, dims, blocks, nblocks, tout, st, &tune))) return s;
            ctx->tunes[tkey] = std::make_pair(tune.ty, tune.order);
            ctx->last_tuned = 1;
        }
        if (tune.ty > 0 && tune.ty != tile_rows_for_mag(cfg->mag[1]) &&
            (s = make_blocks(ctx, *cfg, dims, blocks, nblocks, &all, tune.ty)))
            return s;
        ctx->last_ty = tune.ty > 0 ? tune.ty : tile_rows_for_mag(cfg->mag[1]);
        ctx->last_order = tune.order;
        // replay: the whole call as one CUDA graph (device pointers, or pinned host buffers)
        const bool graphable = flags == RFBA_DEVICE_PTRS || (host_pinned(in) && host_pinned(out));
        if (graphable && env_on("RFBA_GRAPH", true)) {
            std::string gkey = tkey;
            key_put(&gkey, &in, 1);
            key_put(&gkey, &out, 1);
            key_put(&gkey, &out_elems, 1);
            key_put(&gkey, &flags, 1);
            key_put(&gkey, &zero_out, 1);
            const int stall = test_tma_stall();
            key_put(&gkey, &stall, 1);
            key_put(&gkey, blocks, (size_t)nblocks);
            const bool host = flags == RFBA_HOST_PTRS;
            auto deps_now = [&]() {
                return std::vector<const void*>{ctx->rad.p, ctx->inten.p, ctx->tables.p, ctx->errw.p,
                                                host ? ctx->in.p : nullptr, host ? ctx->out.p : nullptr};
            };
            GraphPlan* gp = nullptr;
            for (size_t i = 0; i < ctx->graphs.size(); ++i)
                if (ctx->graphs[i]->key == gkey && ctx->graphs[i]->deps == deps_now()) {
                    std::unique_ptr<GraphPlan> g = std::move(ctx->graphs[i]);
                    ctx->graphs.erase(ctx->graphs.begin() + i);
                    ctx->graphs.insert(ctx->graphs.begin(), std::move(g));
                    gp = ctx->graphs.front().get();
                    break;
                }
            if (!gp) {
                std::unique_ptr<GraphPlan> g(new GraphPlan());
                g->key = gkey;
                Tuning t2 = tune;
                if ((s = ctx->errw.ensure(256, "check word"))) return s;
                if ((s = plan_passes(ctx, *cfg, dtype, dims, all, t2, &g->ps))) return s;
                const PassSet& ps = g->ps;
                const size_t np = ps.passes.size();
                if ((s = ctx->rad.ensure((size_t)ps.max_stack * 4, "radiality stack"))) return s;
                if ((s = ctx->inten.ensure((size_t)ps.max_stack * 4, "intensity stack"))) return s;
                if (host) {
                    if ((s = ctx->in.ensure(in_bytes, "input"))) return s;
                    if ((s = ctx->out.ensure((size_t)out_elems * 4, "output"))) return s;
                }
                if ((s = g->blocks.ensure(ps.blocks.size() * sizeof(BlockDev), "blocks")) ||
                    (s = g->tiles.ensure(ps.tiles.size() * sizeof(TileDesc), "tiles")) ||
                    (s = g->prefix.ensure(ps.prefix.size() * sizeof(long long), "prefix")) ||
                    (s = g->counters.ensure(np * 256, "counters")) || (s = ensure_events(&g->evs, 3 * np)))
                    return s;
                RFBA_CUDA(cudaMemcpy(g->blocks.p, ps.blocks.data(), ps.blocks.size() * sizeof(BlockDev),
                                     cudaMemcpyHostToDevice), "blocks upload");
                RFBA_CUDA(cudaMemcpy(g->tiles.p, ps.tiles.data(), ps.tiles.size() * sizeof(TileDesc),
                                     cudaMemcpyHostToDevice), "tiles upload");
                RFBA_CUDA(cudaMemcpy(g->prefix.p, ps.prefix.data(), ps.prefix.size() * sizeof(long long),
                                     cudaMemcpyHostToDevice), "prefix upload");
                if (!ctx->cap) RFBA_CUDA(cudaStreamCreateWithFlags(&ctx->cap, cudaStreamNonBlocking), "stream");
                const void* gin = host ? ctx->in.p : in;
                float* gout = host ? static_cast<float*>(ctx->out.p) : out;
                RFBA_CUDA(cudaStreamBeginCapture(ctx->cap, cudaStreamCaptureModeThreadLocal), "graph capture");
                int cs = RFBA_OK;
                cudaError_t ce = cudaSuccess;
                if (host) {
                    ce = cudaMemcpyAsync(ctx->in.p, in, in_bytes, cudaMemcpyHostToDevice, ctx->cap);
                    if (ce == cudaSuccess) ce = cudaMemsetAsync(gout, 0, (size_t)out_elems * 4, ctx->cap);
                } else if (zero_out) {
                    ce = cudaMemsetAsync(gout, 0, (size_t)out_elems * 4, ctx->cap);
                }
                if (ce == cudaSuccess)
                    cs = enqueue_passes(ctx, *cfg, gin, dtype, dims, ps, static_cast<const BlockDev*>(g->blocks.p),
                                        static_cast<const TileDesc*>(g->tiles.p),
                                        static_cast<const long long*>(g->prefix.p),
                                        static_cast<unsigned int*>(g->counters.p), gout, ctx->cap, g->evs.data(),
                                        true);
                if (ce == cudaSuccess && cs == RFBA_OK && host)
                    ce = cudaMemcpyAsync(out, gout, (size_t)out_elems * 4, cudaMemcpyDeviceToHost, ctx->cap);
                cudaGraph_t graph = nullptr;
                const cudaError_t ee = cudaStreamEndCapture(ctx->cap, &graph);
                if (ce != cudaSuccess || cs != RFBA_OK || ee != cudaSuccess) {
                    if (graph) cudaGraphDestroy(graph);
                    if (cs != RFBA_OK) return cs;
                    return cuda_fail(ce != cudaSuccess ? ce : ee, "graph capture");
                }
                ce = cudaGraphInstantiate(&g->exec, graph, 0);
                cudaGraphDestroy(graph);
                if (ce != cudaSuccess) return cuda_fail(ce, "graph instantiate");
                g->deps = deps_now();
                ctx->graphs.insert(ctx->graphs.begin(), std::move(g));
                while (ctx->graphs.size() > 4) ctx->graphs.pop_back();
                gp = ctx->graphs.front().get();
            }
            ctx->train.valid = false;
            RFBA_CUDA(cudaGraphLaunch(gp->exec, st), "graph launch");
            account(ctx, gp->ps);
            ctx->last_graph = 1;
            if (ctx->timing && (s = collect_timing(ctx, gp->ps, gp->evs))) return s;
            if (host) return device_status(ctx, st, "forward");
            return RFBA_OK;
        }
        const void* in_dev = in;
        float* out_dev = out;
        if (flags == RFBA_HOST_PTRS) {
            if ((s = ctx->in.ensure(in_bytes, "input"))) return s;
            if ((s = ctx->out.ensure((size_t)out_elems * 4, "output"))) return s;
            RFBA_CUDA(cudaMemcpyAsync(ctx->in.p, in, in_bytes, cudaMemcpyHostToDevice, st), "input copy");
            in_dev = ctx->in.p;
            out_dev = static_cast<float*>(ctx->out.p);
            RFBA_CUDA(cudaMemsetAsync(out_dev, 0, (size_t)out_elems * 4, st), "output clear");
        } else if (zero_out) {
            RFBA_CUDA(cudaMemsetAsync(out_dev, 0, (size_t)out_elems * 4, st), "output clear");
        }
        if ((s = run_device(ctx, *cfg, in_dev, dtype, dims, all, out_dev, st, tune))) return s;
        if (flags == RFBA_HOST_PTRS) {
            RFBA_CUDA(cudaMemcpyAsync(out, out_dev, (size_t)out_elems * 4, cudaMemcpyDeviceToHost, st), "output copy");
            return device_status(ctx, st, "forward");
        }
        return RFBA_OK;
    }
    const void* in_dev = in;
    float* out_dev = out;
    if (flags == RFBA_HOST_PTRS) {
        if ((s = ctx->in.ensure(in_bytes, "input"))) return s;
        if ((s = ctx->out.ensure((size_t)out_elems * 4, "output"))) return s;
        RFBA_CUDA(cudaMemcpyAsync(ctx->in.p, in, in_bytes, cudaMemcpyHostToDevice, st), "input copy");
        in_dev = ctx->in.p;
        out_dev = static_cast<float*>(ctx->out.p);
        RFBA_CUDA(cudaMemsetAsync(out_dev, 0, (size_t)out_elems * 4, st), "output clear");
    } else if (zero_out) {
        RFBA_CUDA(cudaMemsetAsync(out_dev, 0, (size_t)out_elems * 4, st), "output clear");
    }
    if ((s = run_device(ctx, *cfg, in_dev, dtype, dims, all, out_dev, st))) return s;
    if (flags == RFBA_HOST_PTRS) {
        RFBA_CUDA(cudaMemcpyAsync(out, out_dev, (size_t)out_elems * 4, cudaMemcpyDeviceToHost, st), "output copy");
        return device_status(ctx, st, "forward");
    }
    return RFBA_OK;
}

// ---------------------------------------------------------------------------
// Differentiable path

static bool same_cfg(const rfba_srrf_config& a, const rfba_srrf_config& b) {
    return std::memcmp(&a, &b, sizeof a) == 0;
}

// I' = drift(in) into ctx->shifted (x, then y, then z), or in itself.
static int apply_drift(rfba_ctx* ctx, const float* in, const float* shifts, const int dims[4], cudaStream_t st,
                       const float** iprime) {
    if (!shifts) {
        *iprime = in;
        return RFBA_OK;
    }
    const size_t n = (size_t)dims[0] * dims[1] * dims[2] * dims[3];
    int s;
    if ((s = ctx->shifted.ensure(n * 4, "shifted input")) || (s = ctx->tmp1.ensure(n * 4, "scratch")) ||
        (s = ctx->tmp2.ensure(n * 4, "scratch")))
        return s;
    float* out = static_cast<float*>(ctx->shifted.p);
    unsigned long long* err = static_cast<unsigned long long*>(ctx->errw.p);
    const int e = launch_drift3d(in, out, nullptr, dims[0], dims[1], dims[2], dims[3], shifts, 0, nullptr, err, st);
    if (e) return cuda_fail((cudaError_t)e, "drift resampling");
    ctx->launches += 1;
    *iprime = out;
    return RFBA_OK;
}

// The device status word: 0, or the first failure a kernel recorded, with the
// site in the top byte and the work item or global index below. Site 0x54 is
// the radiality kernel's bounded input-staging wait (a copy that did not land
// within about a second); the other sites are the RFBA_CHECKS index checks.
static int decode_status(unsigned long long w, const char* what) {
    if (!w) return RFBA_OK;
    char buf[200];
    if ((w >> 56) == 0x54) {
        std::snprintf(buf, sizeof buf,
                      "%s: a bounded device wait gave up (the input staging copy of work item %llu did not land)",
                      what, w & 0x00ffffffffffffffull);
        set_error(buf);
        return RFBA_ERR_TIMEOUT;
    }
    std::snprintf(buf, sizeof buf, "%s: out-of-range global index %llu at check site %llu", what,
                  w & 0x00ffffffffffffffull, w >> 56);
    set_error(buf);
    return RFBA_ERR_CUDA;
}

// Wait for stream st, read the status word, clear it when set.
static int device_status(rfba_ctx* ctx, cudaStream_t st, const char* what) {
    if (!ctx->errw.p) return RFBA_OK;
    unsigned long long w = 0;
    RFBA_CUDA(cudaMemcpyAsync(&w, ctx->errw.p, 8, cudaMemcpyDeviceToHost, st), "status word read");
    RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    if (w) RFBA_CUDA(cudaMemsetAsync(ctx->errw.p, 0, 8, st), "status word clear");
    return decode_status(w, what);
}

static int read_checks(rfba_ctx* ctx, cudaStream_t st, const char* what) {
    if (!checks_enabled() || !ctx->errw.p) return RFBA_OK;
    return device_status(ctx, st, what);
}

// The whole volume as one block computing the fine region [lo, hi) (all of the
// map when lo / hi are null), its output packed [z][y][x]; n receives the
// region's element count.
static int region_block(const rfba_srrf_config* cfg, const int dims[4], const int* lo, const int* hi, rfba_block* b,
                        int64_t* n) {
    std::memset(b, 0, sizeof *b);
    for (int a = 0; a < 3; ++a) {
        b->size[a] = dims[a];
        b->lo[a] = lo ? lo[a] : 0;
        b->hi[a] = hi ? hi[a] : dims[a] * cfg->mag[a];
        if (b->lo[a] < 0 || b->hi[a] <= b->lo[a] || b->hi[a] > dims[a] * cfg->mag[a]) {
            set_error("region outside the magnified grid or empty");
            return RFBA_ERR_INVALID;
        }
    }
    const int64_t nx = b->hi[0] - b->lo[0], ny = b->hi[1] - b->lo[1], nz = b->hi[2] - b->lo[2];
    b->out_stride[0] = 1;
    b->out_stride[1] = nx;
    b->out_stride[2] = nx * ny;
    *n = nx * ny * nz;
    return RFBA_OK;
}

static int forward_shifted_locked(rfba_ctx* ctx, const rfba_srrf_config* cfg, const float* in, const float* shifts,
                                  const int dims[4], float* out, cudaStream_t st, const int* rlo = nullptr,
                                  const int* rhi = nullptr) {
    int s = validate_common(cfg, in, dims, out);
    if (s) return s;
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    if ((s = order_streams(ctx, st))) return s;
    if ((s = ctx->errw.ensure(256, "check word"))) return s;
    RFBA_CUDA(cudaMemsetAsync(ctx->errw.p, 0, 8, st), "check word clear");
    rfba_block b;
    int64_t n = 0;
    if ((s = region_block(cfg, dims, rlo, rhi, &b, &n))) return s;
    const float* ip = nullptr;
    if ((s = apply_drift(ctx, in, shifts, dims, st, &ip))) return s;
    if ((s = forward_blocks_locked(ctx, cfg, ip, RFBA_F32, dims, &b, 1, out, n, RFBA_DEVICE_PTRS, st, false)))
        return s;
    // the backward can reuse this forward's stacks when they are all resident and
    // the temporal reduction left them intact (ITC 1 bins the series in place)
    if (!rlo && ctx->last_passes == 1 && !(cfg->method == 3 && cfg->itc == 1)) {
        std::vector<BlockDev> all;
        if ((s = make_blocks(ctx, *cfg, dims, &b, 1, &all))) return s;
        if (all.size() == 1) {
            ctx->train.valid = true;
            ctx->train.cfg = *cfg;
            for (int a = 0; a < 4; ++a) ctx->train.dims[a] = dims[a];
            ctx->train.in = in;
            ctx->train.shifts = shifts;
            ctx->train.iprime = ip;
            ctx->train.blk = all[0];
            ctx->train.blk.stack_off = 0;
        }
    }
    return read_checks(ctx, st, "forward_shifted");
}

// Adjoint of one block slice whose radiality and intensity stacks sit at
// offset 0 of the context's stacks: temporal adjoint, then the radiality
// adjoint adding into dL/dI' (ctx->gin, cleared by the caller).
static int adjoint_slab(rfba_ctx* ctx, const rfba_srrf_config* cfg, const float* iprime, const int dims[4],
                        BlockDev blk, const float* gmap, long long ngmap, cudaStream_t st) {
    int s;
    const int T = dims[3];
    const size_t nin = (size_t)dims[0] * dims[1] * dims[2] * T;
    const long long V = blk.vox;
    blk.stack_off = 0;
    const int FZ = cfg->mag[2] * cza_for_mag(cfg->mag[2]);
    blk.ntile[1] = (blk.hi[1] - blk.lo[1] + kAdjRows - 1) / kAdjRows;
    blk.ntile[2] = (blk.hi[2] - blk.zbase + FZ - 1) / FZ;
    std::vector<TileDesc> tiles;
    for (int tz = 0; tz < blk.ntile[2]; ++tz)
        for (int ty = 0; ty < blk.ntile[1]; ++ty)
            for (int tx = 0; tx < blk.ntile[0]; ++tx) tiles.push_back({0, tx, ty, tz});
    if ((s = ctx->gS.ensure((size_t)V * T * 4, "adjoint stack")) || (s = ctx->gI.ensure((size_t)V * T * 4, "adjoint stack")) ||
        (s = ctx->ablocks.ensure(sizeof(BlockDev), "blocks")) ||
        (s = ctx->atiles.ensure(tiles.size() * sizeof(TileDesc), "tiles")) || (s = ctx->acounter.ensure(256, "counter")) ||
        (s = ctx->errw.ensure(256, "check word")))
        return s;
    RFBA_CUDA(cudaMemcpyAsync(ctx->ablocks.p, &blk, sizeof blk, cudaMemcpyHostToDevice, st), "blocks upload");
    RFBA_CUDA(cudaMemcpyAsync(ctx->atiles.p, tiles.data(), tiles.size() * sizeof(TileDesc), cudaMemcpyHostToDevice, st),
              "tiles upload");
    RFBA_CUDA(cudaMemsetAsync(ctx->acounter.p, 0, 256, st), "counter reset");
    const BlockDev* dblk = static_cast<const BlockDev*>(ctx->ablocks.p);
    float* gS = static_cast<float*>(ctx->gS.p);
    float* gI = static_cast<float*>(ctx->gI.p);
    unsigned long long* err = static_cast<unsigned long long*>(ctx->errw.p);
    int e = launch_temporal_adjoint(dblk, V, static_cast<const float*>(ctx->rad.p),
                                    static_cast<const float*>(ctx->inten.p), gmap, T, cfg->method, cfg->itc,
                                    cfg->trac_order,
                                    cfg->intensity_w, cfg->renormalize == 1, cfg->remove_con == 1, gS, gI, ngmap, err,
                                    st);
    if (e) return cuda_fail((cudaError_t)e, "temporal adjoint launch");
    RadParams rp = fill_rad_params(ctx, *cfg, iprime, dims, cza_for_mag(cfg->mag[2]));
    rp.TY = kAdjRows;
    rp.NV = (kAdjRows - 1) / cfg->mag[1] + 2 + 4;
    rp.NIY = rp.NV + 2 * rp.R;
    rp.blocks = dblk;
    rp.tiles = static_cast<const TileDesc*>(ctx->atiles.p);
    rp.ntiles = (int)tiles.size();
    rp.work_counter = static_cast<unsigned int*>(ctx->acounter.p);
    const size_t smem = radiality_adjoint_smem_bytes(rp);
    if (smem > 227 * 1024) {
        set_error("shared memory tile too large for the adjoint of this configuration");
        return RFBA_ERR_UNSUPPORTED;
    }
    int per_sm = 0;
    e = radiality_adjoint_max_ctas_per_sm(rp, &per_sm);
    if (e) return cuda_fail((cudaError_t)e, "occupancy");
    if (per_sm < 1) {
        set_error("adjoint kernel does not fit on an SM");
        return RFBA_ERR_UNSUPPORTED;
    }
    const int slots = per_sm * ctx->sm_count;
    long long nch = (8LL * slots + rp.ntiles - 1) / rp.ntiles;
    nch = std::max<long long>(1, std::min<long long>(nch, T));
    rp.t_chunk = (int)((T + nch - 1) / nch);
    rp.nchunks = (T + rp.t_chunk - 1) / rp.t_chunk;
    rp.nitems = (long long)rp.ntiles * rp.nchunks;
    const int grid = (int)std::max<long long>(1, std::min<long long>(slots, rp.nitems));
    AdjParams ap{gS, gI, static_cast<float*>(ctx->gin.p), (long long)nin, (long long)V * T, err};
    e = launch_radiality_adjoint(rp, ap, grid, smem, st);
    if (e) return cuda_fail((cudaError_t)e, "radiality adjoint launch");
    ctx->launches += 2;
    return RFBA_OK;
}

static int backward_locked(rfba_ctx* ctx, const rfba_srrf_config* cfg, const float* in, const float* shifts,
                           const int dims[4], const float* gmap, float* din, float* dshift, cudaStream_t st,
                           const int* rlo = nullptr, const int* rhi = nullptr) {
    int s = validate_common(cfg, in, dims, gmap);
    if (s) return s;
    rfba_block b;
    int64_t nreg = 0;
    if ((s = region_block(cfg, dims, rlo, rhi, &b, &nreg))) return s;
    if (!din) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    if ((s = order_streams(ctx, st))) return s;
    const bool reuse = !rlo && ctx->train.valid && same_cfg(ctx->train.cfg, *cfg) && ctx->train.in == in &&
                       ctx->train.shifts == shifts && ctx->train.dims[0] == dims[0] && ctx->train.dims[1] == dims[1] &&
                       ctx->train.dims[2] == dims[2] && ctx->train.dims[3] == dims[3];
    if (ctx->timing) RFBA_CUDA(cudaEventRecord(ctx->ev[0], st), "event");
    const int T = dims[3];
    const size_t nin = (size_t)dims[0] * dims[1] * dims[2] * T;
    if ((s = ensure_plan(ctx, *cfg, st))) return s;
    if ((s = ctx->gin.ensure(nin * 4, "input adjoint"))) return s;
    if ((s = ctx->errw.ensure(256, "check word"))) return s;
    if (reuse) {
        RFBA_CUDA(cudaMemsetAsync(ctx->gin.p, 0, nin * 4, st), "adjoint clear");
        if ((s = adjoint_slab(ctx, cfg, ctx->train.iprime, dims, ctx->train.blk, gmap, nreg, st))) return s;
    } else {
        // The whole volume's slices under the stack budget: each slice's stacks are
        // recomputed by the forward kernels, then its adjoint runs (one slice when
        // everything fits).
        if ((s = ctx->out.ensure((size_t)nreg * 4, "map"))) return s;
        RFBA_CUDA(cudaMemsetAsync(ctx->errw.p, 0, 8, st), "check word clear");
        const float* ip = nullptr;
        if ((s = apply_drift(ctx, in, shifts, dims, st, &ip))) return s;
        std::vector<BlockDev> all;
        if ((s = make_blocks(ctx, *cfg, dims, &b, 1, &all))) return s;
        RFBA_CUDA(cudaMemsetAsync(ctx->gin.p, 0, nin * 4, st), "adjoint clear");
        // the recomputed stacks must stay as the radiality kernel wrote them: TRAC
        // with ITC 1 would bin them in place, so its map (unused here) is formed
        // with ITC 0, which only reads them
        rfba_srrf_config fcfg = *cfg;
        if (fcfg.method == 3) fcfg.itc = 0;
        for (const BlockDev& slab : all) {
            std::vector<BlockDev> one(1, slab);
            if ((s = run_device(ctx, fcfg, ip, RFBA_F32, dims, one, static_cast<float*>(ctx->out.p), st))) return s;
            BlockDev blk = slab;
            blk.stack_off = 0;
            if ((s = adjoint_slab(ctx, cfg, ip, dims, blk, gmap, nreg, st))) return s;
        }
    }
    // through the drift operator
    float* gin = static_cast<float*>(ctx->gin.p);
    unsigned long long* err = static_cast<unsigned long long*>(ctx->errw.p);
    int e = 0;
    if (shifts) {
        float* t1 = static_cast<float*>(ctx->tmp1.p);
        float* t2 = static_cast<float*>(ctx->tmp2.p);
        e = launch_shift_axis(gin, t1, dims[0], dims[1], dims[2], T, 2, shifts, 2, err, st);
        if (!e) e = launch_shift_axis(t1, t2, dims[0], dims[1], dims[2], T, 1, shifts, 2, err, st);
        if (!e) e = launch_shift_axis(t2, din, dims[0], dims[1], dims[2], T, 0, shifts, 2, err, st);
        ctx->launches += 3;
        if (!e && dshift) {
            if ((s = ctx->dshift.ensure((size_t)T * 3 * sizeof(double), "drift adjoint"))) return s;
            double* ds = static_cast<double*>(ctx->dshift.p);
            RFBA_CUDA(cudaMemsetAsync(ds, 0, (size_t)T * 3 * sizeof(double), st), "drift adjoint clear");
            e = launch_drift3d(in, nullptr, gin, dims[0], dims[1], dims[2], T, shifts, 1, ds, err, st);
            ctx->launches += 1;
            if (!e) e = launch_double_to_float(ds, dshift, 3 * T, st);
            ctx->launches += 1;
        }
        if (e) return cuda_fail((cudaError_t)e, "drift adjoint");
    } else {
        RFBA_CUDA(cudaMemcpyAsync(din, gin, nin * 4, cudaMemcpyDeviceToDevice, st), "adjoint copy");
        if (dshift) RFBA_CUDA(cudaMemsetAsync(dshift, 0, (size_t)T * 3 * 4, st), "drift adjoint clear");
    }
    if (ctx->timing) {
        RFBA_CUDA(cudaEventRecord(ctx->ev[3], st), "event");
        RFBA_CUDA(cudaEventSynchronize(ctx->ev[3]), "event sync");
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[3]);
        ctx->last_backward_ms = ms;
    }
    return read_checks(ctx, st, "backward");
}

// ---- 3B spot gradient ------------------------------------------------------

static int threeb_validate(const rfba_3b_model* m, int S, int F, int P, int ptr_flags) {
    if (S < 1 || F < 1 || P < 1 || (long long)S * F >= (1LL << 31) || !(m->variance > 0) || m->z_factor == 0) {
        set_error("bad sizes or model (S, F, P >= 1, S*F < 2^31, variance > 0, z_factor != 0)");
        return RFBA_ERR_INVALID;
    }
    if (ptr_flags != RFBA_HOST_PTRS && ptr_flags != RFBA_DEVICE_PTRS) {
        set_error("ptr_flags must be RFBA_HOST_PTRS or RFBA_DEVICE_PTRS");
        return RFBA_ERR_INVALID;
    }
    for (int n = 0; n < 12; ++n) {
        const double v = n < 9 ? m->A[n] : m->pi[n - 9];
        if (!(v >= 0 && v <= 1)) {
            set_error("transition and initial probabilities must lie in [0, 1]");
            return RFBA_ERR_INVALID;
        }
    }
    return RFBA_OK;
}

struct ThreeBData {
    const double* bg = nullptr;
    const double* pix = nullptr;
    const int* pixels = nullptr;
    int S = 0, F = 0, P = 0;
};

// Scratch for one evaluation, and the data on the device (copied in once when
// the caller's pointers are host memory).
static int threeb_stage(rfba_ctx* ctx, const double* sample_bg, const double* pixel_intensities, const int* pixels,
                        int S, int F, int P, int ptr_flags, cudaStream_t st, ThreeBData* d) {
    int s;
    const size_t nbg = (size_t)S * F * P, npix = (size_t)F * P;
    if ((s = ctx->tb_val.ensure((size_t)P * 8, "3B spot table")) || (s = ctx->tb_der.ensure((size_t)P * 40, "3B spot table")) ||
        (s = ctx->tb_em.ensure((size_t)S * F * 80, "3B emissions")) || (s = ctx->tb_res.ensure((size_t)S * 48 + 48, "3B results")) ||
        (s = ctx->tb_par.ensure(17 * 8, "3B parameters")))
        return s;
    d->bg = sample_bg;
    d->pix = pixel_intensities;
    d->pixels = pixels;
    d->S = S;
    d->F = F;
    d->P = P;
    if (ptr_flags == RFBA_HOST_PTRS) {
        if ((s = ctx->tb_bg.ensure(nbg * 8, "3B samples")) || (s = ctx->tb_pix.ensure(npix * 8, "3B data")) ||
            (s = ctx->tb_pixels.ensure((size_t)P * 12, "3B mask")))
            return s;
        RFBA_CUDA(cudaMemcpyAsync(ctx->tb_bg.p, sample_bg, nbg * 8, cudaMemcpyHostToDevice, st), "samples copy");
        RFBA_CUDA(cudaMemcpyAsync(ctx->tb_pix.p, pixel_intensities, npix * 8, cudaMemcpyHostToDevice, st), "data copy");
        RFBA_CUDA(cudaMemcpyAsync(ctx->tb_pixels.p, pixels, (size_t)P * 12, cudaMemcpyHostToDevice, st), "mask copy");
        d->bg = static_cast<const double*>(ctx->tb_bg.p);
        d->pix = static_cast<const double*>(ctx->tb_pix.p);
        d->pixels = static_cast<const int*>(ctx->tb_pixels.p);
    }
    return RFBA_OK;
}

// One evaluation at `spot` (brightness and blur > 0) on staged data: the four
// kernels, the samples' results back, their mean plus the priors' derivatives.
static int threeb_eval(rfba_ctx* ctx, const rfba_3b_model* m, const ThreeBData& d, const double* spot, double* out,
                       double* log_prob, cudaStream_t st) {
    const int S = d.S, F = d.F, P = d.P;
    // parameters: spot, A (row-major), pi
    double par[17];
    for (int n = 0; n < 5; ++n) par[n] = spot[n];
    for (int n = 0; n < 9; ++n) par[5 + n] = m->A[n];
    for (int n = 0; n < 3; ++n) par[14 + n] = m->pi[n];
    RFBA_CUDA(cudaMemcpyAsync(ctx->tb_par.p, par, sizeof par, cudaMemcpyHostToDevice, st), "parameter upload");
    const unsigned int n_pix = (unsigned int)P;
    const double c0 = n_pix * ::log(2 * M_PI * m->variance) / 2;  // spot_with_background.hh:126-127
    const double* dpar = static_cast<const double*>(ctx->tb_par.p);
    int e = launch_threeb(d.bg, d.pix, d.pixels, S, F, P, dpar, m->z_factor, m->variance, c0, dpar + 5, dpar + 14,
                          static_cast<double*>(ctx->tb_val.p), static_cast<double*>(ctx->tb_der.p),
                          static_cast<double*>(ctx->tb_em.p), static_cast<double*>(ctx->tb_res.p), st);
    if (e) return cuda_fail((cudaError_t)e, "3B spot gradient launch");
    ctx->launches += 4;
    std::vector<double> res((size_t)S * 6);
    RFBA_CUDA(cudaMemcpyAsync(res.data(), ctx->tb_res.p, res.size() * 8, cudaMemcpyDeviceToHost, st), "result copy");
    RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    double sum[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < S; ++i)
        for (int n = 0; n < 5; ++n) sum[n] += res[(size_t)i * 6 + n];
    // storm.h:431-434: derivatives of the log-normal priors on brightness and blur
    auto dlln = [&](double x, double mu, double sg) { return -(1 + (std::log(x) - mu) / (sg * sg)) / x; };
    const double prior[5] = {dlln(spot[0], m->mu_brightness, m->sigma_brightness),
                             dlln(spot[1], m->mu_blur, m->sigma_blur), 0, 0, 0};
    for (int n = 0; n < 5; ++n) out[n] = -(sum[n] / (double)S + prior[n]);
    if (log_prob)
        for (int i = 0; i < S; ++i) log_prob[i] = res[(size_t)i * 6 + 5];
    return RFBA_OK;
}


// ---- 3B Gibbs sampler -------------------------------------------------------

// getBall (multispot5.cc:1259-1272): the integer offsets p, z outermost then y
// then x over [-r, r] with r = ceil(radius + 1), kept when |p|^2 (unsigned)
// <= radius^2 in float.
static std::vector<int> ball(float radius) {
    std::vector<int> pts;
    const int r = (int)std::ceil(radius + 1);
    for (int z = -r; z <= r; ++z)
        for (int y = -r; y <= r; ++y)
            for (int x = -r; x <= r; ++x) {
                const unsigned int m2 = (unsigned int)(x * x) + (unsigned int)(y * y) + (unsigned int)(z * z);
                if ((float)m2 <= radius * radius) {
                    pts.push_back(x);
                    pts.push_back(y);
                    pts.push_back(z);
                }
            }
    return pts;
}

// ir_rounded3D (multispot5.cc:989-995): round half away from zero.
static int round_away(double v) { return static_cast<int>(v > 0.0 ? v + 0.5 : v - 0.5); }

// Masks and pixel/spot validation shared by the Gibbs entry points. Masks are
// host copies (read back when the caller's pointers are device memory).
static int gibbs_masks(const int* moff, const int* midx, int K, int P, int ptr_flags, cudaStream_t st,
                       std::vector<int>* hoff, std::vector<int>* hidx) {
    hoff->assign((size_t)K + 1, 0);
    if (ptr_flags == RFBA_HOST_PTRS)
        std::memcpy(hoff->data(), moff, ((size_t)K + 1) * sizeof(int));
    else {
        RFBA_CUDA(cudaMemcpyAsync(hoff->data(), moff, ((size_t)K + 1) * sizeof(int), cudaMemcpyDeviceToHost, st),
                  "mask offsets read-back");
        RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    }
    if ((*hoff)[0] != 0) {
        set_error("mask_offsets[0] must be 0");
        return RFBA_ERR_INVALID;
    }
    for (int k = 0; k < K; ++k)
        if ((*hoff)[k + 1] < (*hoff)[k]) {
            set_error("mask_offsets must not decrease");
            return RFBA_ERR_INVALID;
        }
    const size_t nnz = (size_t)(*hoff)[K];
    hidx->assign(nnz, 0);
    if (nnz) {
        if (ptr_flags == RFBA_HOST_PTRS)
            std::memcpy(hidx->data(), midx, nnz * sizeof(int));
        else {
            RFBA_CUDA(cudaMemcpyAsync(hidx->data(), midx, nnz * sizeof(int), cudaMemcpyDeviceToHost, st),
                      "mask read-back");
            RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
        }
    }
    // every index inside [0, P), no pixel twice in one spot's mask (a spot's
    // pixels are updated in parallel)
    std::vector<int> seen((size_t)P, -1);
    for (int k = 0; k < K; ++k)
        for (int q = (*hoff)[k]; q < (*hoff)[k + 1]; ++q) {
            const int p = (*hidx)[q];
            if (p < 0 || p >= P) {
                set_error("mask pixel index outside [0, P)");
                return RFBA_ERR_INVALID;
            }
            if (seen[p] == k) {
                set_error("a pixel appears twice in one spot's mask");
                return RFBA_ERR_INVALID;
            }
            seen[p] = k;
        }
    return RFBA_OK;
}

struct GibbsCall {
    int K = 0, F = 0, P = 0;
    int sweeps = 1, n_draws = 1;
    unsigned long long seed = 0;
    int exclude = -1;
    const double* var_draw = nullptr;  // host, n_draws
    bool want_state = false, want_int = false, want_err = false, trace = false;
};

// Stage the data, compute the spot intensities, run one chain from all spots
// off. Outputs stay in the context's gb_* buffers; returns after the kernel
// has finished and its status has been read.
static int gibbs_run(rfba_ctx* ctx, const rfba_3b_model* m, const double* pix, const int* pixels,
                     const double* spots, const std::vector<int>& hoff, const std::vector<int>& hidx,
                     const GibbsCall& c, int ptr_flags, cudaStream_t st) {
    int s;
    const size_t K = (size_t)c.K, F = (size_t)c.F, P = (size_t)c.P, nnz = hidx.size();
    if ((s = ctx->gb_moff.ensure((K + 1) * 4, "3B mask offsets")) || (s = ctx->gb_midx.ensure(nnz * 4 + 4, "3B masks")) ||
        (s = ctx->gb_si.ensure(K * P * 8 + 8, "3B spot intensities")) ||
        (s = ctx->gb_state.ensure(K * F + 1, "3B spot states")) || (s = ctx->gb_cur.ensure(F * P * 8, "3B sample intensities")) ||
        (s = ctx->gb_em.ensure(F * 64, "3B emissions")) || (s = ctx->gb_bar.ensure(256, "3B barrier")))
        return s;
    const double* dpix = pix;
    const int* dpixels = pixels;
    const double* dspots = spots;
    if (ptr_flags == RFBA_HOST_PTRS) {
        if ((s = ctx->gb_pix.ensure(F * P * 8, "3B data")) || (s = ctx->gb_pixels.ensure(P * 12, "3B pixels")) ||
            (s = ctx->gb_spots.ensure(K * 40 + 8, "3B spots")))
            return s;
        RFBA_CUDA(cudaMemcpyAsync(ctx->gb_pix.p, pix, F * P * 8, cudaMemcpyHostToDevice, st), "data copy");
        RFBA_CUDA(cudaMemcpyAsync(ctx->gb_pixels.p, pixels, P * 12, cudaMemcpyHostToDevice, st), "pixels copy");
        if (K) RFBA_CUDA(cudaMemcpyAsync(ctx->gb_spots.p, spots, K * 40, cudaMemcpyHostToDevice, st), "spots copy");
        dpix = static_cast<const double*>(ctx->gb_pix.p);
        dpixels = static_cast<const int*>(ctx->gb_pixels.p);
        dspots = static_cast<const double*>(ctx->gb_spots.p);
    }
    RFBA_CUDA(cudaMemcpyAsync(ctx->gb_moff.p, hoff.data(), (K + 1) * 4, cudaMemcpyHostToDevice, st), "mask offsets copy");
    if (nnz) RFBA_CUDA(cudaMemcpyAsync(ctx->gb_midx.p, hidx.data(), nnz * 4, cudaMemcpyHostToDevice, st), "mask copy");
    if (K) {
        int e = launch_spot_intensity(dpixels, c.P, dspots, c.K, m->z_factor, static_cast<double*>(ctx->gb_si.p), st);
        if (e) return cuda_fail((cudaError_t)e, "3B spot intensity launch");
        ++ctx->launches;
    }
    // all spots off (state 2), no spot intensity in the current sample
    RFBA_CUDA(cudaMemsetAsync(ctx->gb_state.p, 2, K * F + 1, st), "state init");
    RFBA_CUDA(cudaMemsetAsync(ctx->gb_cur.p, 0, F * P * 8, st), "sample init");
    RFBA_CUDA(cudaMemsetAsync(ctx->gb_bar.p, 0, 256, st), "barrier init");
    RFBA_CUDA(cudaMemsetAsync(ctx->errw.p, 0, 8, st), "status clear");
    const size_t nd = (size_t)c.n_draws;
    if (c.var_draw) {
        if ((s = ctx->gb_var.ensure(nd * 8, "3B variance schedule"))) return s;
        RFBA_CUDA(cudaMemcpyAsync(ctx->gb_var.p, c.var_draw, nd * 8, cudaMemcpyHostToDevice, st), "schedule copy");
    }
    if (c.want_state && (s = ctx->gb_ostate.ensure(nd * K * F + 1, "3B drawn states"))) return s;
    if (c.want_int && (s = ctx->gb_oint.ensure(nd * F * P * 8, "3B drawn intensities"))) return s;
    if (c.want_err && (s = ctx->gb_oerr.ensure(nd * F * 8, "3B residual sums"))) return s;
    if (c.trace && ((s = ctx->gb_lp.ensure(K * F * 16 + 16, "3B trace")) || (s = ctx->gb_filt.ensure(K * F * 24 + 24, "3B trace"))))
        return s;
    GibbsParams g;
    std::memset(&g, 0, sizeof g);
    g.pix = dpix;
    g.si = static_cast<const double*>(ctx->gb_si.p);
    g.moff = static_cast<const int*>(ctx->gb_moff.p);
    g.midx = static_cast<const int*>(ctx->gb_midx.p);
    g.K = c.K;
    g.F = c.F;
    g.P = c.P;
    for (int n = 0; n < 9; ++n) g.A[n] = m->A[n];
    for (int n = 0; n < 3; ++n) g.pi[n] = m->pi[n];
    g.variance = m->variance;
    g.var_draw = c.var_draw ? static_cast<const double*>(ctx->gb_var.p) : nullptr;
    g.sweeps = c.sweeps;
    g.n_draws = c.n_draws;
    g.seed = c.seed;
    g.draw_base = 0;
    g.state = static_cast<unsigned char*>(ctx->gb_state.p);
    g.cur = static_cast<double*>(ctx->gb_cur.p);
    g.em = static_cast<double*>(ctx->gb_em.p);
    g.bar = static_cast<unsigned int*>(ctx->gb_bar.p);
    g.err = static_cast<unsigned long long*>(ctx->errw.p);
    g.out_state = c.want_state ? static_cast<unsigned char*>(ctx->gb_ostate.p) : nullptr;
    g.out_int = c.want_int ? static_cast<double*>(ctx->gb_oint.p) : nullptr;
    g.exclude_spot = c.exclude;
    g.out_err = c.want_err ? static_cast<double*>(ctx->gb_oerr.p) : nullptr;
    g.rec_lp = c.trace ? static_cast<double*>(ctx->gb_lp.p) : nullptr;
    g.rec_filt = c.trace ? static_cast<double*>(ctx->gb_filt.p) : nullptr;
    int maxb = 0;
    int e = gibbs_max_blocks(c.F, &maxb);
    if (e) return cuda_fail((cudaError_t)e, "3B Gibbs occupancy");
    if (maxb < 1) {
        set_error("3B Gibbs kernel does not fit on an SM");
        return RFBA_ERR_UNSUPPORTED;
    }
    const int grid = std::min(std::min(c.F, maxb), ctx->sm_count);
    e = launch_gibbs(g, grid, st);
    if (e) return cuda_fail((cudaError_t)e, "3B Gibbs launch");
    ++ctx->launches;
    unsigned long long w = 0;
    RFBA_CUDA(cudaMemcpyAsync(&w, ctx->errw.p, 8, cudaMemcpyDeviceToHost, st), "status read");
    RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    if (w) {
        RFBA_CUDA(cudaMemsetAsync(ctx->errw.p, 0, 8, st), "status clear");
        char buf[160];
        std::snprintf(buf, sizeof buf, "3B Gibbs sampler: a grid barrier gave up (spot %llu)", w & 0xffffffffffffull);
        set_error(buf);
        return RFBA_ERR_TIMEOUT;
    }
    return RFBA_OK;
}

static int gibbs_check(rfba_ctx* ctx, const rfba_3b_model* m, int K, int F, int P, int ptr_flags) {
    if (!ctx || !m) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    if (K < 0 || F < 1 || P < 1 || F > 2048 || (long long)F * P >= (1LL << 40) / 8) {
        set_error("bad sizes (K >= 0, 1 <= F <= 2048, P >= 1)");
        return RFBA_ERR_INVALID;
    }
    return threeb_validate(m, 1, F, P, ptr_flags);
}

static void copy_out(void* dst, const void* src, size_t n, int ptr_flags, cudaStream_t st, int* s) {
    if (*s || !dst || n == 0) return;
    const cudaError_t e = cudaMemcpyAsync(dst, src, n, ptr_flags == RFBA_HOST_PTRS ? cudaMemcpyDeviceToHost
                                                                                  : cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) *s = cuda_fail(e, "3B Gibbs output copy");
}

// variance_from_sample (multispot5.cc:321-328)
static double variance_from_sample(double sample, double samples, double base_sigma, double scale_pow) {
    const double scale = std::pow(1.25, sample * 1. / samples * scale_pow);
    const double sigma = base_sigma * scale;
    return sigma * sigma;
}

// log_log_normal (storm.h:417-420) with the reference's ln (forward_algorithm.h:34-40)
static double ref_ln(double x) { return x == 0 ? -1e100 : std::log(x); }
static double log_log_normal(double x, double mu, double sigma) {
    const double a = ref_ln(x) - mu;
    return -(a * a) / (2 * (sigma * sigma)) - ref_ln(x) - ref_ln(sigma * std::sqrt(2 * M_PI));
}

}  // namespace rfba

using namespace rfba;

extern "C" {

int rfba_3b_spot_masks(const int* pixels, int P, const double* spots, int K, int* mask_offsets, int* mask_pixels,
                       long long cap, long long* nnz) {
    if (!pixels || P < 1 || K < 0 || (K > 0 && !spots) || !mask_offsets || !nnz) {
        set_error("null argument or bad sizes");
        return RFBA_ERR_INVALID;
    }
    // pixels must be in the reference's Ref3D order (z, then y, then x)
    auto less = [&](int a, int b) {
        const int* p = pixels + 3 * a;
        const int* q = pixels + 3 * b;
        return p[2] < q[2] || (p[2] == q[2] && p[1] < q[1]) || (p[2] == q[2] && p[1] == q[1] && p[0] < q[0]);
    };
    for (int i = 1; i < P; ++i)
        if (!less(i - 1, i)) {
            set_error("pixels must be sorted by (z, y, x) without repeats");
            return RFBA_ERR_INVALID;
        }
    long long n = 0;
    mask_offsets[0] = 0;
    for (int k = 0; k < K; ++k) {
        const double* sp = spots + 5 * (size_t)k;
        const std::vector<int> b = ball((float)(sp[1] * 6 + 1));
        const int ox = round_away(sp[2]), oy = round_away(sp[3]), oz = round_away(sp[4]);
        for (size_t j = 0; j < b.size(); j += 3) {
            const int t[3] = {b[j] + ox, b[j + 1] + oy, b[j + 2] + oz};
            int lo = 0, hi = P;  // lower_bound
            while (lo < hi) {
                const int mid = (lo + hi) / 2;
                const int* q = pixels + 3 * mid;
                const bool lt = q[2] < t[2] || (q[2] == t[2] && q[1] < t[1]) || (q[2] == t[2] && q[1] == t[1] && q[0] < t[0]);
                if (lt)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            if (lo < P && pixels[3 * lo] == t[0] && pixels[3 * lo + 1] == t[1] && pixels[3 * lo + 2] == t[2]) {
                if (mask_pixels && n < cap) mask_pixels[n] = lo;
                ++n;
            }
        }
        if (n > INT32_MAX) {
            set_error("masks too large");
            return RFBA_ERR_INVALID;
        }
        mask_offsets[k + 1] = (int)n;
    }
    *nnz = n;
    return RFBA_OK;
}

int rfba_3b_gibbs_sample(rfba_ctx* ctx, const rfba_3b_model* m, const double* pixel_intensities, const int* pixels,
                         const double* spots, const int* mask_offsets, const int* mask_pixels, int K, int F, int P,
                         int sweeps, int n_draws, unsigned long long seed, int exclude_spot, uint8_t* states,
                         double* sample_intensities, int ptr_flags, void* stream) {
    int s;
    if ((s = gibbs_check(ctx, m, K, F, P, ptr_flags))) return s;
    if (!pixel_intensities || !pixels || (K > 0 && (!spots || !mask_pixels)) || !mask_offsets || sweeps < 1 ||
        n_draws < 1 || exclude_spot >= K || exclude_spot < -1) {
        set_error("null argument, or sweeps / n_draws < 1, or exclude_spot outside [-1, K)");
        return RFBA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if ((s = order_streams(ctx, st))) return s;
    std::vector<int> hoff, hidx;
    if ((s = gibbs_masks(mask_offsets, mask_pixels, K, P, ptr_flags, st, &hoff, &hidx))) return s;
    GibbsCall c;
    c.K = K;
    c.F = F;
    c.P = P;
    c.sweeps = sweeps;
    c.n_draws = n_draws;
    c.seed = seed;
    c.exclude = exclude_spot;
    c.want_state = states != nullptr;
    c.want_int = sample_intensities != nullptr;
    if ((s = gibbs_run(ctx, m, pixel_intensities, pixels, spots, hoff, hidx, c, ptr_flags, st))) return s;
    copy_out(states, ctx->gb_ostate.p, (size_t)n_draws * K * F, ptr_flags, st, &s);
    copy_out(sample_intensities, ctx->gb_oint.p, (size_t)n_draws * F * P * 8, ptr_flags, st, &s);
    if (s) return s;
    RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    return RFBA_OK;
}

// Seed of spot `s`'s draws in pass `pass` of rfba_3b_optimise_pass: SplitMix64
// (Steele, Lea, Flood, OOPSLA 2014) of the caller's seed mixed with both.
static unsigned long long pass_seed(unsigned long long seed, int pass, int s) {
    unsigned long long z = seed ^ ((unsigned long long)(unsigned)pass << 32) ^ (unsigned long long)(unsigned)s;
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

unsigned long long rfba_3b_pass_seed(unsigned long long seed, int pass, int s) { return pass_seed(seed, pass, s); }

// One pass of FitSpots::optimize_each_spot_in_turn_for_several_passes
// (multispot5.cc:1511-1690).
int rfba_3b_optimise_pass(rfba_ctx* ctx, const rfba_3b_model* m, const double* pixel_intensities, const int* pixels,
                          int F, int P, double* spots, int* nspots, int pass, int main_samples, int sweeps,
                          int cg_max_iterations, const double limit[5], double position_extra_radius,
                          unsigned long long seed, int* evaluations) {
    int s;
    if (!nspots || !spots || !limit || !pixel_intensities || !pixels) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    int K = *nspots;
    if ((s = gibbs_check(ctx, m, K, F, P, RFBA_HOST_PTRS))) return s;
    if (main_samples < 1 || sweeps < 1 || cg_max_iterations < 0) {
        set_error("main_samples and sweeps must be >= 1, cg_max_iterations >= 0");
        return RFBA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    if ((s = order_streams(ctx, st))) return s;
    // masks of every spot (multispot5.cc:1518-1521)
    std::vector<int> off((size_t)K + 1);
    long long nnz = 0;
    if ((s = rfba_3b_spot_masks(pixels, P, spots, K, off.data(), nullptr, 0, &nnz))) return s;
    std::vector<int> idx((size_t)nnz);
    if ((s = rfba_3b_spot_masks(pixels, P, spots, K, off.data(), idx.data(), nnz, &nnz))) return s;
    std::vector<std::vector<int> > masks((size_t)K);
    for (int k = 0; k < K; ++k) masks[k].assign(idx.begin() + off[k], idx.begin() + off[k + 1]);
    // allowed area: the pixels dilated by getBall(extra_radius) (multispot5.cc:1280-1290)
    std::set<long long> allowed;
    auto key = [](int x, int y, int z) {
        return ((long long)(x + (1 << 20)) << 42) | ((long long)(y + (1 << 20)) << 21) | (long long)(z + (1 << 20));
    };
    const bool use_prior = position_extra_radius >= 0;
    if (use_prior) {
        const std::vector<int> b = ball((float)position_extra_radius);
        for (int p = 0; p < P; ++p)
            for (size_t j = 0; j < b.size(); j += 3)
                allowed.insert(key(pixels[3 * p] + b[j], pixels[3 * p + 1] + b[j + 1], pixels[3 * p + 2] + b[j + 2]));
    }
    // the sweep order (multispot5.cc:1541-1560): by x or y position, ascending
    // or descending; the reference's third branch repeats `% 4 == 1` and is never
    // taken, so passes 2 and 3 both sort by descending y
    std::vector<int> order((size_t)K);
    for (int k = 0; k < K; ++k) order[k] = k;
    std::vector<std::array<double, 5> > sp((size_t)K);
    for (int k = 0; k < K; ++k)
        for (int n = 0; n < 5; ++n) sp[k][n] = spots[5 * k + n];
    const int mode = pass % 4 == 0 ? 0 : pass % 4 == 1 ? 1 : 2;
    const int first = mode == 2 ? 3 : 2, second = first == 2 ? 3 : 2;
    std::sort(order.begin(), order.end(), [&](int a, int b) {
        const double fa = sp[a][first], fb = sp[b][first];
        const bool desc = mode != 0;
        if (desc ? fa > fb : fa < fb) return true;
        if (fa == fb) return desc ? sp[a][second] > sp[b][second] : sp[a][second] < sp[b][second];
        return false;
    });
    {
        std::vector<std::array<double, 5> > t((size_t)K);
        for (int k = 0; k < K; ++k) t[k] = sp[order[k]];
        sp.swap(t);
        // masks stay where they were: the reference swaps tmp_spot_pixels[i]
        // with spot_pixels[i], not spot_pixels[index[i]] (multispot5.cc:1570), so
        // a spot's mask is the one at its new position until it is optimised
    }
    // data on the device once
    const size_t FP = (size_t)F * P;
    if ((s = ctx->gb_pix.ensure(FP * 8, "3B data")) || (s = ctx->gb_pixels.ensure((size_t)P * 12, "3B pixels")) ||
        (s = ctx->gb_spots.ensure((size_t)K * 40 + 8, "3B spots")))
        return s;
    RFBA_CUDA(cudaMemcpyAsync(ctx->gb_pix.p, pixel_intensities, FP * 8, cudaMemcpyHostToDevice, st), "data copy");
    RFBA_CUDA(cudaMemcpyAsync(ctx->gb_pixels.p, pixels, (size_t)P * 12, cudaMemcpyHostToDevice, st), "pixels copy");
    int evals = 0;
    for (int k = 0; k < K; ++k) {
        // a fresh sampler for this spot: main_samples draws, the spot taken off
        // them (multispot5.cc:1591-1608)
        std::vector<int> hoff((size_t)K + 1, 0), hidx;
        for (int j = 0; j < K; ++j) {
            hidx.insert(hidx.end(), masks[j].begin(), masks[j].end());
            hoff[j + 1] = (int)hidx.size();
        }
        std::vector<double> flat((size_t)K * 5);
        for (int j = 0; j < K; ++j)
            for (int n = 0; n < 5; ++n) flat[5 * j + n] = sp[j][n];
        RFBA_CUDA(cudaMemcpyAsync(ctx->gb_spots.p, flat.data(), flat.size() * 8, cudaMemcpyHostToDevice, st),
                  "spots copy");
        GibbsCall c;
        c.K = K;
        c.F = F;
        c.P = P;
        c.sweeps = sweeps;
        c.n_draws = main_samples;
        c.seed = pass_seed(seed, pass, k);
        c.exclude = k;
        c.want_int = true;
        if ((s = gibbs_run(ctx, m, static_cast<const double*>(ctx->gb_pix.p), static_cast<const int*>(ctx->gb_pixels.p),
                           static_cast<const double*>(ctx->gb_spots.p), hoff, hidx, c, RFBA_DEVICE_PTRS, st)))
            return s;
        // optimise the spot on those samples (multispot5.cc:1611-1636)
        ThreeBData d;
        if ((s = threeb_stage(ctx, static_cast<const double*>(ctx->gb_oint.p), static_cast<const double*>(ctx->gb_pix.p),
                              static_cast<const int*>(ctx->gb_pixels.p), main_samples, F, P, RFBA_DEVICE_PTRS, st, &d)))
            return s;
        auto grad = [&](const double* x, double* g) -> int {
            if (x[0] <= 0 || x[1] <= 0) {
                for (int n = 0; n < 5; ++n) g[n] = std::numeric_limits<double>::quiet_NaN();
                return RFBA_OK;
            }
            return threeb_eval(ctx, m, d, x, g, nullptr, st);
        };
        CgOnly5 cg;
        if ((s = cg.start(sp[k].data(), limit, grad))) return s;
        cg.max_iterations = cg_max_iterations;
        if ((s = cg.run(grad))) return s;
        evals += cg.evaluations;
        for (int n = 0; n < 5; ++n) sp[k][n] = cg.x[n];
        // new mask; eject the spot if it has no pixels or left the allowed area
        // (multispot5.cc:1651-1674)
        int o2[2];
        long long n2 = 0;
        if ((s = rfba_3b_spot_masks(pixels, P, sp[k].data(), 1, o2, nullptr, 0, &n2))) return s;
        masks[k].assign((size_t)n2, 0);
        if (n2 && (s = rfba_3b_spot_masks(pixels, P, sp[k].data(), 1, o2, masks[k].data(), n2, &n2))) return s;
        const bool zero_prior =
            use_prior && !allowed.count(key(round_away(sp[k][2]), round_away(sp[k][3]), round_away(sp[k][4])));
        if (masks[k].empty() || zero_prior) {
            sp.erase(sp.begin() + k);
            masks.erase(masks.begin() + k);
            --K;
            --k;
        }
    }
    for (int k = 0; k < K; ++k)
        for (int n = 0; n < 5; ++n) spots[5 * k + n] = sp[k][n];
    *nspots = K;
    if (evaluations) *evaluations = evals;
    return RFBA_OK;
}

int rfba_3b_gibbs_trace(rfba_ctx* ctx, const rfba_3b_model* m, const double* pixel_intensities, const int* pixels,
                        const double* spots, const int* mask_offsets, const int* mask_pixels, int K, int F, int P,
                        unsigned long long seed, uint8_t* states, double* log_prob, double* filtered, int ptr_flags,
                        void* stream) {
    int s;
    if ((s = gibbs_check(ctx, m, K, F, P, ptr_flags))) return s;
    if (!pixel_intensities || !pixels || (K > 0 && (!spots || !mask_pixels)) || !mask_offsets) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if ((s = order_streams(ctx, st))) return s;
    std::vector<int> hoff, hidx;
    if ((s = gibbs_masks(mask_offsets, mask_pixels, K, P, ptr_flags, st, &hoff, &hidx))) return s;
    GibbsCall c;
    c.K = K;
    c.F = F;
    c.P = P;
    c.seed = seed;
    c.want_state = true;
    c.trace = true;
    if ((s = gibbs_run(ctx, m, pixel_intensities, pixels, spots, hoff, hidx, c, ptr_flags, st))) return s;
    copy_out(states, ctx->gb_ostate.p, (size_t)K * F, ptr_flags, st, &s);
    copy_out(log_prob, ctx->gb_lp.p, (size_t)K * F * 16, ptr_flags, st, &s);
    copy_out(filtered, ctx->gb_filt.p, (size_t)K * F * 24, ptr_flags, st, &s);
    if (s) return s;
    RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    return RFBA_OK;
}

int rfba_3b_free_energy(rfba_ctx* ctx, const rfba_3b_model* m, const double* pixel_intensities, const int* pixels,
                        const double* spots, const int* mask_offsets, const int* mask_pixels, int K, int F, int P,
                        int samples, int sweeps, unsigned long long seed, double* value, double* residuals,
                        int ptr_flags, void* stream) {
    int s;
    if ((s = gibbs_check(ctx, m, K, F, P, ptr_flags))) return s;
    if (!pixel_intensities || !pixels || (K > 0 && (!spots || !mask_pixels)) || !mask_offsets || !value ||
        samples < 1 || sweeps < 1) {
        set_error("null argument, or samples / sweeps < 1");
        return RFBA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if ((s = order_streams(ctx, st))) return s;
    std::vector<int> hoff, hidx;
    if ((s = gibbs_masks(mask_offsets, mask_pixels, K, P, ptr_flags, st, &hoff, &hidx))) return s;
    // the spots on the host, for the priors
    std::vector<double> hsp((size_t)K * 5);
    if (K) {
        if (ptr_flags == RFBA_HOST_PTRS)
            std::memcpy(hsp.data(), spots, hsp.size() * 8);
        else {
            RFBA_CUDA(cudaMemcpyAsync(hsp.data(), spots, hsp.size() * 8, cudaMemcpyDeviceToHost, st), "spots read-back");
            RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
        }
    }
    // NegativeFreeEnergy::compute_with_mask (multispot5.cc:335-405): slow-growth
    // thermodynamic integration over `samples` draws, draw i taken at the
    // variance of step i - 1 and differentiated by a five-point stencil
    const double base_sigma = std::sqrt(m->variance);
    const double scale_pow = 100.0;
    std::vector<double> var2((size_t)samples);
    for (int i = 0; i < samples; ++i) var2[i] = variance_from_sample(i - 1, samples, base_sigma, scale_pow);
    GibbsCall c;
    c.K = K;
    c.F = F;
    c.P = P;
    c.sweeps = sweeps;
    c.n_draws = samples;
    c.seed = seed;
    c.var_draw = var2.data();
    c.want_err = true;
    if ((s = gibbs_run(ctx, m, pixel_intensities, pixels, spots, hoff, hidx, c, ptr_flags, st))) return s;
    std::vector<double> err((size_t)samples * F);
    RFBA_CUDA(cudaMemcpyAsync(err.data(), ctx->gb_oerr.p, err.size() * 8, cudaMemcpyDeviceToHost, st),
              "residual read-back");
    RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    const unsigned int npixels = (unsigned int)P, nframes = (unsigned int)F;
    double sum = 0;
    for (int sample = 0; sample < samples; sample++) {
        const double var1 = variance_from_sample(sample - 2, samples, base_sigma, scale_pow);
        const double var2s = variance_from_sample(sample - 1, samples, base_sigma, scale_pow);
        const double var3 = variance_from_sample(sample + 1, samples, base_sigma, scale_pow);
        const double var4 = variance_from_sample(sample + 2, samples, base_sigma, scale_pow);
        double err_sum = 0;
        for (int f = 0; f < F; ++f) err_sum -= err[(size_t)sample * F + f];
        if (residuals) residuals[sample] = -err_sum;
        const double e1 = err_sum / (2 * var1) - npixels * nframes * ::log(2 * M_PI * var1) / 2;
        const double e2 = err_sum / (2 * var2s) - npixels * nframes * ::log(2 * M_PI * var2s) / 2;
        const double e3 = err_sum / (2 * var3) - npixels * nframes * ::log(2 * M_PI * var3) / 2;
        const double e4 = err_sum / (2 * var4) - npixels * nframes * ::log(2 * M_PI * var4) / 2;
        sum += (-e1 + 8 * e2 - 8 * e3 + e4) / 12;
    }
    const double log_final =
        (::log(variance_from_sample(samples, samples, base_sigma, scale_pow) * 2 * M_PI) / 2) * npixels * nframes;
    double priors = 0;
    for (int i = 0; i < K; i++) {
        priors += log_log_normal(hsp[i * 5 + 0], m->mu_brightness, m->sigma_brightness);
        priors += log_log_normal(hsp[i * 5 + 1], m->mu_blur, m->sigma_blur);
    }
    *value = -(sum + priors - log_final);
    return RFBA_OK;
}

}  // extern "C"

namespace rfba {

}  // namespace rfba

using namespace rfba;

extern "C" {

int rfba_srrf_forward_shifted(rfba_ctx* ctx, const rfba_srrf_config* cfg, const float* in, const float* shifts,
                              const int dims[4], float* out, void* stream) {
    if (!ctx) {
        set_error("null context");
        return RFBA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL = legacy default stream
    return forward_shifted_locked(ctx, cfg, in, shifts, dims, out, st);
}

int rfba_srrf_backward(rfba_ctx* ctx, const rfba_srrf_config* cfg, const float* in, const float* shifts,
                       const int dims[4], const float* dL_dmap, float* dL_din, float* dL_dshift, void* stream) {
    if (!ctx) {
        set_error("null context");
        return RFBA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL = legacy default stream
    return backward_locked(ctx, cfg, in, shifts, dims, dL_dmap, dL_din, dL_dshift, st);
}

// SpotNegProbabilityDiffWithSampledBackground::operator() (multispot5.cc:616-664)
int rfba_3b_spot_gradient(rfba_ctx* ctx, const rfba_3b_model* m, const double* sample_bg,
                          const double* pixel_intensities, const int* pixels, int S, int F, int P, const double spot[5],
                          double out[5], double* log_prob, int ptr_flags, void* stream) {
    if (!ctx || !m || !sample_bg || !pixel_intensities || !pixels || !spot || !out) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    int s;
    if ((s = threeb_validate(m, S, F, P, ptr_flags))) return s;
    if (spot[0] <= 0 || spot[1] <= 0) {  // multispot5.cc:618-619
        for (int n = 0; n < 5; ++n) out[n] = std::numeric_limits<double>::quiet_NaN();
        return RFBA_OK;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if ((s = order_streams(ctx, st))) return s;
    ThreeBData d;
    if ((s = threeb_stage(ctx, sample_bg, pixel_intensities, pixels, S, F, P, ptr_flags, st, &d))) return s;
    return threeb_eval(ctx, m, d, spot, out, log_prob, st);
}

// The spot optimisation of multispot5.cc:1614-1636: ConjugateGradientOnly<5>
// (conjugate_gradient_only.h) from `spot` with motion limits `limit`, its
// gradient the spot-gradient evaluation above on data staged once.
int rfba_3b_optimise_spot(rfba_ctx* ctx, const rfba_3b_model* m, const double* sample_bg,
                          const double* pixel_intensities, const int* pixels, int S, int F, int P, const double spot[5],
                          const double limit[5], int max_iterations, double spot_out[5], int* iterations,
                          int* evaluations, int ptr_flags, void* stream) {
    if (!ctx || !m || !sample_bg || !pixel_intensities || !pixels || !spot || !limit || !spot_out) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    int s;
    if ((s = threeb_validate(m, S, F, P, ptr_flags))) return s;
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if ((s = order_streams(ctx, st))) return s;
    ThreeBData d;
    if ((s = threeb_stage(ctx, sample_bg, pixel_intensities, pixels, S, F, P, ptr_flags, st, &d))) return s;
    auto grad = [&](const double* x, double* g) -> int {
        if (x[0] <= 0 || x[1] <= 0) {  // multispot5.cc:618-619
            for (int n = 0; n < 5; ++n) g[n] = std::numeric_limits<double>::quiet_NaN();
            return RFBA_OK;
        }
        return threeb_eval(ctx, m, d, x, g, nullptr, st);
    };
    CgOnly5 cg;
    if ((s = cg.start(spot, limit, grad))) return s;
    cg.max_iterations = max_iterations;
    if ((s = cg.run(grad))) return s;
    for (int n = 0; n < 5; ++n) spot_out[n] = cg.x[n];
    if (iterations) *iterations = cg.iterations;
    if (evaluations) *evaluations = cg.evaluations;
    return RFBA_OK;
}

// The same optimiser on the host with a caller-supplied gradient (no device
// work).
int rfba_cg_only_run(const double start[5], const double limit[5], int max_iterations, rfba_grad5_fn grad,
                     void* user, double x_out[5], int* iterations, int* evaluations) {
    if (!start || !limit || !grad || !x_out) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    auto g = [&](const double* x, double* out) -> int { return grad(x, out, user); };
    CgOnly5 cg;
    int s;
    if ((s = cg.start(start, limit, g))) return s;
    cg.max_iterations = max_iterations;
    if ((s = cg.run(g))) return s;
    for (int n = 0; n < 5; ++n) x_out[n] = cg.x[n];
    if (iterations) *iterations = cg.iterations;
    if (evaluations) *evaluations = cg.evaluations;
    return RFBA_OK;
}

int rfba_probe_fp32_fma_peak(int device, double* tflops) {
    if (!tflops) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    *tflops = 0.0;
    const int e = probe_fp32_fma(device, tflops);
    if (e) return cuda_fail((cudaError_t)e, "FP32 probe");
    return RFBA_OK;
}

int rfba_ctx_check(rfba_ctx* c) {
    if (!c) {
        set_error("null context");
        return RFBA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(c->mu);
    RFBA_CUDA(cudaSetDevice(c->device), "cudaSetDevice");
    return device_status(c, c->have_last ? c->last_stream : c->stream, "device work");
}

int rfba_srrf_forward_shifted_region(rfba_ctx* ctx, const rfba_srrf_config* cfg, const float* in,
                                     const float* shifts, const int dims[4], const int lo[3], const int hi[3],
                                     float* out, void* stream) {
    if (!ctx || !lo || !hi) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    return forward_shifted_locked(ctx, cfg, in, shifts, dims, out, static_cast<cudaStream_t>(stream), lo, hi);
}

int rfba_srrf_backward_region(rfba_ctx* ctx, const rfba_srrf_config* cfg, const float* in, const float* shifts,
                              const int dims[4], const int lo[3], const int hi[3], const float* dL_dregion,
                              float* dL_din, float* dL_dshift, void* stream) {
    if (!ctx || !lo || !hi) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    return backward_locked(ctx, cfg, in, shifts, dims, dL_dregion, dL_din, dL_dshift,
                           static_cast<cudaStream_t>(stream), lo, hi);
}

int rfba_ctx_last_backward_ms(rfba_ctx* c, double* ms) {
    if (!c || !ms) return RFBA_ERR_INVALID;
    *ms = c->last_backward_ms;
    return RFBA_OK;
}

const char* rfba_last_error(void) { return g_last_error.c_str(); }
const char* rfba_version(void) { return "rfba_srrf 0.1 (sm_103a)"; }

int rfba_ctx_create(int device, size_t budget, rfba_ctx** out) {
    if (!out) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    rfba_ctx* c = new rfba_ctx();
    int s = ctx_init(c, device, budget);
    if (s) {
        delete c;
        return s;
    }
    *out = c;
    return RFBA_OK;
}

int rfba_ctx_destroy(rfba_ctx* c) {
    if (!c) return RFBA_OK;
    {
        std::lock_guard<std::mutex> lk(g_default_mu);
        if (c == g_default) g_default = nullptr;
    }
    cudaSetDevice(c->device);
    for (DevBuf* b : {&c->in, &c->out, &c->rad, &c->inten, &c->blocks, &c->tiles, &c->tables, &c->counter, &c->prefix,
                      &c->shifted, &c->tmp1, &c->tmp2, &c->gS, &c->gI, &c->gin, &c->dshift, &c->ablocks, &c->atiles,
                      &c->acounter, &c->errw, &c->tb_val, &c->tb_der, &c->tb_em, &c->tb_res, &c->tb_par, &c->tb_bg,
                      &c->tb_pix, &c->tb_pixels, &c->seed_w, &c->seed_sums, &c->seed_carry, &c->seed_map, &c->seed_vox,
                      &c->seed_xyz, &c->gb_pix, &c->gb_pixels, &c->gb_spots, &c->gb_si, &c->gb_moff, &c->gb_midx,
                      &c->gb_state, &c->gb_cur, &c->gb_em, &c->gb_bar, &c->gb_var, &c->gb_ostate, &c->gb_oint,
                      &c->gb_oerr, &c->gb_lp, &c->gb_filt})
        b->release();
    for (auto& e : c->ev)
        if (e) cudaEventDestroy(e);
    c->graphs.clear();
    for (cudaEvent_t e : c->pev) cudaEventDestroy(e);
    if (c->cap) cudaStreamDestroy(c->cap);
    if (c->xev) cudaEventDestroy(c->xev);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return RFBA_OK;
}

// Measurement hooks used by bench.py: CUDA-event times of the last call's
// kernels (on the stream they were launched on) and the kernel launch count.
int rfba_ctx_set_timing(rfba_ctx* c, int enable) {
    if (!c) return RFBA_ERR_INVALID;
    c->timing = enable != 0;
    return RFBA_OK;
}
int rfba_ctx_last_timing(rfba_ctx* c, double* rad_ms, double* temporal_ms, long long* launches) {
    if (!c) return RFBA_ERR_INVALID;
    if (rad_ms) *rad_ms = c->last_rad_ms;
    if (temporal_ms) *temporal_ms = c->last_temporal_ms;
    if (launches) *launches = c->launches;
    return RFBA_OK;
}
int rfba_srrf_seed_spots(rfba_ctx* ctx, const float* map, const int map_dims[3], int mag, const int* voxels,
                         int nvoxels, int num_spots, unsigned long long seed, float* xyz, int ptr_flags, void* stream) {
    if (!ctx || !map || !map_dims || !voxels || !xyz || mag < 1 || nvoxels < 1 || num_spots < 0) {
        set_error("null argument or bad size");
        return RFBA_ERR_INVALID;
    }
    if (map_dims[0] < 1 || map_dims[1] < 1 || map_dims[2] < 1) {
        set_error("bad map dims");
        return RFBA_ERR_INVALID;
    }
    const long long ncand = (long long)nvoxels * mag * mag * mag;
    const long long n1 = (ncand + 511) / 512, n2 = (n1 + 511) / 512;
    if (n2 > 512) {
        set_error("too many candidate subvoxels (at most 512^3)");
        return RFBA_ERR_UNSUPPORTED;
    }
    if (num_spots == 0) return RFBA_OK;
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL = legacy default stream
    int s;
    if ((s = order_streams(ctx, st))) return s;
    if ((s = ctx->seed_w.ensure((size_t)ncand * 8, "seeding weights")) ||
        (s = ctx->seed_sums.ensure((size_t)n1 * 8, "seeding scan")) ||
        (s = ctx->seed_carry.ensure((size_t)(n2 + 1) * 8, "seeding scan")) || (s = ctx->errw.ensure(256, "check word")))
        return s;
    const float* dmap = map;
    const int* dvox = voxels;
    float* dxyz = xyz;
    const size_t map_bytes = (size_t)map_dims[0] * map_dims[1] * map_dims[2] * 4;
    if (ptr_flags == RFBA_HOST_PTRS) {
        if ((s = ctx->seed_map.ensure(map_bytes, "seeding map")) ||
            (s = ctx->seed_vox.ensure((size_t)nvoxels * 12, "seeding voxels")) ||
            (s = ctx->seed_xyz.ensure((size_t)num_spots * 12, "seeding spots")))
            return s;
        RFBA_CUDA(cudaMemcpyAsync(ctx->seed_map.p, map, map_bytes, cudaMemcpyHostToDevice, st), "map copy");
        RFBA_CUDA(cudaMemcpyAsync(ctx->seed_vox.p, voxels, (size_t)nvoxels * 12, cudaMemcpyHostToDevice, st),
                  "voxel copy");
        dmap = static_cast<const float*>(ctx->seed_map.p);
        dvox = static_cast<const int*>(ctx->seed_vox.p);
        dxyz = static_cast<float*>(ctx->seed_xyz.p);
    }
    RFBA_CUDA(cudaMemsetAsync(ctx->errw.p, 0, 8, st), "check word clear");
    int e = launch_seed_spots(dmap, map_dims, mag, dvox, nvoxels, num_spots, seed, dxyz,
                              static_cast<double*>(ctx->seed_w.p), static_cast<double*>(ctx->seed_sums.p),
                              static_cast<double*>(ctx->seed_carry.p),
                              static_cast<unsigned long long*>(ctx->errw.p), st);
    if (e) return cuda_fail((cudaError_t)e, "seeding launch");
    ctx->launches += 3;
    unsigned long long ew = 0;
    RFBA_CUDA(cudaMemcpyAsync(&ew, ctx->errw.p, 8, cudaMemcpyDeviceToHost, st), "check word read");
    if (ptr_flags == RFBA_HOST_PTRS)
        RFBA_CUDA(cudaMemcpyAsync(xyz, dxyz, (size_t)num_spots * 12, cudaMemcpyDeviceToHost, st), "spots copy");
    RFBA_CUDA(cudaStreamSynchronize(st), "synchronize");
    if (ew) {
        // reported here, so cleared: the status word carries unreported failures only
        RFBA_CUDA(cudaMemsetAsync(ctx->errw.p, 0, 8, st), "check word clear");
        set_error("a candidate voxel lies outside the map (magnified voxel index " +
                  std::to_string((long long)(ew & 0x00ffffffffffffffull)) + ")");
        return RFBA_ERR_INVALID;
    }
    return RFBA_OK;
}

int rfba_combine_render(rfba_ctx* ctx, const double* spots, long long nspots, const int img_dims[3], int zoom,
                        const uint16_t* psf, const int psf_dims[3], int noise_r, int noise_rz, int noise_threshold,
                        uint16_t* out, long long* dropped) {
    if (!ctx || (nspots > 0 && !spots) || !img_dims || !psf || !psf_dims || !out || zoom < 1 || noise_r < 0 ||
        noise_rz < 0 || nspots < 0) {
        set_error("null argument or bad size");
        return RFBA_ERR_INVALID;
    }
    const long long Xp = (long long)img_dims[0] * zoom, Yp = (long long)img_dims[1] * zoom,
                    Zp = (long long)img_dims[2] * zoom;
    const long long nk = (long long)psf_dims[0] * psf_dims[1] * psf_dims[2];
    if (Xp < 1 || Yp < 1 || Zp < 1 || Xp > (1 << 30) || Yp > (1 << 30) || nk < 1 || nk * 2 > 200 * 1024 ||
        2 * noise_r + 1 > 255) {
        set_error("bad image, PSF or noise-window size");
        return RFBA_ERR_INVALID;
    }
    const long long nvox = Xp * Yp * Zp;
    std::lock_guard<std::mutex> lk(ctx->mu);
    RFBA_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    int s;
    if ((s = order_streams(ctx, st))) return s;
    DevBuf hist, L, S, o64, o16, idx, val, sp, ps, cnt;
    auto release = [&]() {
        for (DevBuf* b : {&hist, &L, &S, &o64, &o16, &idx, &val, &sp, &ps, &cnt}) b->release();
    };
    const unsigned long long cap = (unsigned long long)std::max<long long>(nspots, 1);
    if ((s = hist.ensure((size_t)nvox * 4, "histogram")) || (s = L.ensure((size_t)nvox, "box sums")) ||
        (s = S.ensure((size_t)nvox * 2, "box sums")) || (s = o64.ensure((size_t)nvox * 8, "convolution")) ||
        (s = o16.ensure((size_t)nvox * 2, "output")) || (s = idx.ensure(cap * 8, "nonzeros")) ||
        (s = val.ensure(cap * 4, "nonzeros")) || (s = sp.ensure((size_t)cap * 40, "spots")) ||
        (s = ps.ensure((size_t)nk * 2, "psf")) || (s = cnt.ensure(64, "counters"))) {
        release();
        return s;
    }
    cudaError_t ce = cudaSuccess;
    if (nspots > 0) ce = cudaMemcpyAsync(sp.p, spots, (size_t)nspots * 40, cudaMemcpyHostToDevice, st);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(ps.p, psf, (size_t)nk * 2, cudaMemcpyHostToDevice, st);
    int e = ce == cudaSuccess ? launch_combine(static_cast<const double*>(sp.p), nspots, zoom, (int)Xp, (int)Yp,
                                               (int)Zp, noise_r, noise_rz, noise_threshold,
                                               static_cast<const uint16_t*>(ps.p), psf_dims[0], psf_dims[1],
                                               psf_dims[2], static_cast<unsigned int*>(hist.p),
                                               static_cast<unsigned char*>(L.p), static_cast<unsigned short*>(S.p),
                                               static_cast<unsigned long long*>(idx.p),
                                               static_cast<unsigned int*>(val.p), cap,
                                               static_cast<unsigned long long*>(cnt.p),
                                               static_cast<unsigned long long*>(o64.p),
                                               static_cast<uint16_t*>(o16.p), st)
                              : (int)ce;
    unsigned long long counters[3] = {0, 0, 0};
    if (!e) e = (int)cudaMemcpyAsync(out, o16.p, (size_t)nvox * 2, cudaMemcpyDeviceToHost, st);
    if (!e) e = (int)cudaMemcpyAsync(counters, cnt.p, sizeof counters, cudaMemcpyDeviceToHost, st);
    if (!e) e = (int)cudaStreamSynchronize(st);
    release();
    if (e) return cuda_fail((cudaError_t)e, "combine");
    ctx->launches += 7;
    if (dropped) *dropped = (long long)counters[0];
    return RFBA_OK;
}

int rfba_ctx_last_schedule(rfba_ctx* c, int* tile_rows, int* tile_order, int* graph, int* tuned) {
    if (!c) return RFBA_ERR_INVALID;
    if (tile_rows) *tile_rows = c->last_ty;
    if (tile_order) *tile_order = c->last_order;
    if (graph) *graph = c->last_graph;
    if (tuned) *tuned = c->last_tuned;
    return RFBA_OK;
}
int rfba_ctx_set_launch(rfba_ctx* c, int grid, int t_chunk) {
    if (!c) return RFBA_ERR_INVALID;
    c->grid_override = grid;
    c->chunk_override = t_chunk;
    return RFBA_OK;
}

int rfba_srrf_plan_info(const rfba_srrf_config* cfg, int* npoints, int* npairs, int* nxvalues, int* nraw) {
    if (!cfg) return RFBA_ERR_INVALID;
    std::string err;
    if (!config_validate(*cfg, &err)) {
        set_error(err);
        return RFBA_ERR_INVALID;
    }
    RingPlan rp;
    if (!build_ring_plan(*cfg, &rp, &err)) {
        set_error(err);
        return RFBA_ERR_UNSUPPORTED;
    }
    if (npoints) *npoints = (int)rp.pt_zval.size();
    if (npairs) *npairs = (int)rp.pair_yval.size();
    if (nxvalues) *nxvalues = (int)rp.grp_xval.size();
    if (nraw) *nraw = rp.npoints_raw;
    return RFBA_OK;
}

int rfba_srrf_config_default(rfba_srrf_config* cfg) {
    if (!cfg) return RFBA_ERR_INVALID;
    config_default(cfg);
    return RFBA_OK;
}

int rfba_srrf_config_load_ini(const char* path, rfba_srrf_config* cfg) {
    if (!cfg || !path) return RFBA_ERR_INVALID;
    config_load_ini(path, cfg);  // a missing file gives the defaults, as GetPrivateProfile* does
    return RFBA_OK;
}

int rfba_srrf_config_from_legacy(const SRRFConf* c, rfba_srrf_config* cfg) {
    if (!c || !cfg) return RFBA_ERR_INVALID;
    cfg->ring_radius = c->RingRadius;
    cfg->mag[0] = cfg->mag[1] = cfg->mag[2] = c->Magnification;
    cfg->axes_in_ring = c->AxesinRing;
    cfg->main_range = c->MainRange;
    cfg->x_range = c->XRange;
    cfg->y_range = c->YRange;
    cfg->z_range = c->ZRange;
    cfg->method = c->Method;
    cfg->itc = c->ITC;
    cfg->trac_order = c->TRACOrder;
    cfg->remove_con = c->RemoveCon;
    cfg->renormalize = c->Renormalize;
    cfg->gradient_smooth = c->GradientSmooth;
    cfg->intensity_w = c->IntensityW;
    cfg->block_size[0] = c->blockSizeX;
    cfg->block_size[1] = c->blockSizeY;
    cfg->block_size[2] = c->blockSizeZ;
    return RFBA_OK;
}

int rfba_blocks_gradientcalc(const rfba_srrf_config* cfg, const int dims[4], rfba_block* blocks, int cap) {
    if (!cfg || !dims) return RFBA_ERR_INVALID;
    std::string err;
    int n = blocks_gradientcalc(*cfg, dims, blocks, blocks ? cap : 0, &err);
    if (n < 0) set_error(err);
    return n;
}

int rfba_blocks_dosplit(const rfba_srrf_config* cfg, const int dims[4], const int max_size[3], int border,
                        rfba_block* blocks, int cap, int64_t* out_elems) {
    if (!cfg || !dims || !max_size) return RFBA_ERR_INVALID;
    std::string err;
    long long oe = 0;
    int n = blocks_dosplit(*cfg, dims, max_size, border, blocks, blocks ? cap : 0, &oe, &err);
    if (n < 0) set_error(err);
    if (out_elems) *out_elems = oe;
    return n;
}

int rfba_srrf_forward_blocks(rfba_ctx* ctx, const rfba_srrf_config* cfg, const void* in, rfba_dtype dtype,
                             const int dims[4], const rfba_block* blocks, int nblocks, float* out, int64_t out_elems,
                             int ptr_flags, void* stream) {
    if (!ctx) {
        set_error("null context");
        return RFBA_ERR_INVALID;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL = legacy default stream
    return forward_blocks_impl(ctx, cfg, in, dtype, dims, blocks, nblocks, out, out_elems, ptr_flags, st, false,
                               true);
}

int rfba_srrf_forward(rfba_ctx* ctx, const rfba_srrf_config* cfg, const void* in, rfba_dtype dtype, const int dims[4],
                      float* out, int ptr_flags, void* stream) {
    if (!ctx || !cfg || !dims) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    rfba_block b;
    std::memset(&b, 0, sizeof b);
    for (int a = 0; a < 3; ++a) {
        b.size[a] = dims[a];
        b.hi[a] = dims[a] * cfg->mag[a];
    }
    b.out_stride[0] = 1;
    b.out_stride[1] = b.hi[0];
    b.out_stride[2] = (int64_t)b.hi[0] * b.hi[1];
    const int64_t n = (int64_t)b.hi[0] * b.hi[1] * b.hi[2];
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL = legacy default stream
    return forward_blocks_impl(ctx, cfg, in, dtype, dims, &b, 1, out, n, ptr_flags, st, false, true);
}

int rfba_srrf_forward_blocks_plain(rfba_ctx* ctx, const rfba_srrf_config* cfg, const void* in, rfba_dtype dtype,
                                   const int dims[4], const rfba_block* blocks, int nblocks, float* out,
                                   int64_t out_elems) {
    // One block at a time: copy the block's input sub-volume to the device,
    // launch, copy its output region back (GradientCalc.cpp:144-160 with
    // kernel.cu:560-657 per block).
    if (!ctx || !cfg || !in || !dims || !out || (nblocks > 0 && !blocks)) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    const size_t es = elem_size(dtype);
    for (int i = 0; i < nblocks; ++i) {
        const rfba_block& b = blocks[i];
        for (int a = 0; a < 3; ++a)
            if (b.size[a] < 1 || b.origin[a] < 0 || b.origin[a] + b.size[a] > dims[a]) {
                set_error("block outside the input volume");
                return RFBA_ERR_INVALID;
            }
        const int bd[4] = {b.size[0], b.size[1], b.size[2], dims[3]};
        std::vector<unsigned char> sub((size_t)bd[0] * bd[1] * bd[2] * bd[3] * es);
        const unsigned char* src = static_cast<const unsigned char*>(in);
        for (int t = 0; t < bd[3]; ++t)
            for (int z = 0; z < bd[2]; ++z)
                for (int y = 0; y < bd[1]; ++y) {
                    const size_t so = ((((size_t)t * dims[2] + b.origin[2] + z) * dims[1] + b.origin[1] + y) * dims[0] +
                                       b.origin[0]) * es;
                    const size_t dof = ((((size_t)t * bd[2] + z) * bd[1] + y) * bd[0]) * es;
                    std::memcpy(sub.data() + dof, src + so, (size_t)bd[0] * es);
                }
        rfba_block lb = b;
        lb.origin[0] = lb.origin[1] = lb.origin[2] = 0;
        const int nx = b.hi[0] - b.lo[0], ny = b.hi[1] - b.lo[1], nz = b.hi[2] - b.lo[2];
        if (nx <= 0 || ny <= 0 || nz <= 0) continue;
        lb.out_offset = 0;
        lb.out_stride[0] = 1;
        lb.out_stride[1] = nx;
        lb.out_stride[2] = (int64_t)nx * ny;
        std::vector<float> o((size_t)nx * ny * nz);
        int s = forward_blocks_impl(ctx, cfg, sub.data(), dtype, bd, &lb, 1, o.data(), (int64_t)o.size(),
                                    RFBA_HOST_PTRS, ctx->stream, false);
        if (s) return s;
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; ++y)
                for (int x = 0; x < nx; ++x) {
                    const int64_t oi = b.out_offset + x * b.out_stride[0] + y * b.out_stride[1] + z * b.out_stride[2];
                    if (oi < 0 || oi >= out_elems) {
                        set_error("block output outside the output array");
                        return RFBA_ERR_INVALID;
                    }
                    out[oi] = o[((size_t)z * ny + y) * nx + x];
                }
    }
    return RFBA_OK;
}

// ---- reference-compatible exports ------------------------------------------

int SRRFGetMag(void) {
    rfba_srrf_config c;
    config_load_ini("SRRF.ini", &c);
    return c.mag[0];
}

int SRRFGradientCalcGPU(float* inImage, int* imageDim, float* outImage, SRRFConf* conf) {
    if (!inImage || !imageDim || !outImage || !conf) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    rfba_ctx* ctx = nullptr;
    int s = default_ctx(&ctx);
    if (s) return s;
    rfba_srrf_config cfg;
    rfba_srrf_config_from_legacy(conf, &cfg);
    return rfba_srrf_forward(ctx, &cfg, inImage, RFBA_F32, imageDim, outImage, RFBA_HOST_PTRS, nullptr);
}

int SRRFGradientCalc(float* inImage, int* imageDim, float* outImage) {
    if (!inImage || !imageDim || !outImage) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    rfba_srrf_config cfg;
    config_load_ini("SRRF.ini", &cfg);  // GradientCalc.cpp:17, re-read on every call
    if (verbose()) std::fprintf(stderr, "rfba: SRRF Method: %d\n", cfg.method);
    rfba_ctx* ctx = nullptr;
    int s = default_ctx(&ctx);
    if (s) return s;
    std::string err;
    int n = blocks_gradientcalc(cfg, imageDim, nullptr, 0, &err);
    if (n < 0) {
        set_error(err);
        return n;
    }
    std::vector<rfba_block> bl(std::max(n, 1));
    blocks_gradientcalc(cfg, imageDim, bl.data(), n, &err);
    const int64_t out_elems = (int64_t)imageDim[0] * imageDim[1] * imageDim[2] * cfg.mag[0] * cfg.mag[0] * cfg.mag[0];
    return forward_blocks_impl(ctx, &cfg, inImage, RFBA_F32, imageDim, bl.data(), n, outImage, out_elems,
                               RFBA_HOST_PTRS, ctx->stream, true);
}

// Targets of the C++-linkage aliases in compat_cxx.cpp.
int rfba_compat_gradientcalc(float* in, int* dims, float* out) { return SRRFGradientCalc(in, dims, out); }
int rfba_compat_getmag(void) { return SRRFGetMag(); }

}  // extern "C"

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

#include "context.h"

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

bool verbose() {
    static int v = -1;
    if (v < 0) {
        const char* e = std::getenv("RFBA_VERBOSE");
        v = (e && *e && *e != '0') ? 1 : 0;
    }
    return v == 1;
}

int cuda_fail(cudaError_t e, const char* what) {
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? RFBA_ERR_NOMEM : RFBA_ERR_CUDA;
}


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
int order_streams(rfba_ctx* ctx, cudaStream_t st) {
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
                       int nblocks, std::vector<BlockDev>* outb, int ty = 0, int tb = 0, int fields = 0) {
    const RingPlan& rp = ctx->plan.ring;
    const int T = dims[3];
    const int FZ = fz_for(cfg.mag[2]);
    outb->clear();
    // bytes per subvoxel: the stacks of the volumes held at once plus the
    // carried temporal state when the series runs in time batches
    const size_t per_vox = (size_t)(tb > 0 ? tb : T) * 2 * sizeof(float) + (size_t)fields * sizeof(float);
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
    // volumes the stacks hold at once, and the carried state of time batches
    const int stack_t = tune.tb > 0 ? std::min(tune.tb, T) : T;
    ps->tb = tune.tb > 0 ? stack_t : 0;
    ps->fields = ps->tb > 0 ? temporal_stream_fields(cfg.method, cfg.trac_order) : 0;
    ps->nbatch = (T + stack_t - 1) / stack_t;
    const size_t per_vox = (size_t)stack_t * 2 * sizeof(float) + (size_t)ps->fields * sizeof(float);
    ps->blocks.clear();
    ps->tiles.clear();
    ps->prefix.clear();
    ps->passes.clear();
    ps->max_stack = 0;
    ps->max_vox = 0;
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
            if (i1 > i0 && (size_t)nv * per_vox > ctx->budget) break;
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
            off += d.vox * stack_t;
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
        pp.vox = vox;
        ps->max_vox = std::max(ps->max_vox, vox);
        const long long nt = (long long)(pp.t1 - pp.t0);
        // time chunk: enough work items for ~8 per CTA slot
        int chunk = ctx->chunk_override;
        if (chunk <= 0) {
            const long long want = 8LL * slots;
            long long nch = (want + nt - 1) / nt;
            nch = std::max<long long>(1, std::min<long long>(nch, stack_t));
            chunk = (int)((stack_t + nch - 1) / nch);
        }
        pp.chunk = chunk;
        pp.nchunks = (stack_t + chunk - 1) / chunk;
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

// Input copy windows of a captured host-buffer forward: volumes [t[k], t[k+1])
// are on the device once ready[k] has fired.
struct InputWindows {
    int n = 0;
    int t[3] = {0, 0, 0};
    const cudaEvent_t* ready = nullptr;
};

// Queue the passes on st: counter reset, radiality, temporal per pass. The
// device lists hold ps's concatenated blocks / tiles / prefixes; evs (3 per
// pass) are recorded around the kernels when given. With input windows the
// radiality of a single whole-series pass runs window by window, each launch
// waiting for its window's copy.
static int enqueue_passes(rfba_ctx* ctx, const rfba_srrf_config& cfg, const void* in_dev, rfba_dtype dtype,
                          const int dims[4], const PassSet& ps, const BlockDev* dblocks, const TileDesc* dtiles,
                          const long long* dprefix, unsigned int* dcounters, float* out_dev, cudaStream_t st,
                          const cudaEvent_t* evs, bool capturing = false, const InputWindows* win = nullptr) {
    // inside a stream capture the events become event-record nodes of the graph
    auto rec = [&](cudaEvent_t e) {
        return capturing ? cudaEventRecordWithFlags(e, st, cudaEventRecordExternal) : cudaEventRecord(e, st);
    };
    const int T = dims[3];
    const int tb = ps.tb > 0 ? ps.tb : T;
    for (size_t i = 0; i < ps.passes.size(); ++i) {
        const PassPlan& pp = ps.passes[i];
        unsigned int* counter = dcounters + 64 * i;
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
        StreamParams sp;
        std::memset(&sp, 0, sizeof sp);
        sp.blocks = tp.blocks;
        sp.vox_prefix = tp.vox_prefix;
        sp.nblocks = tp.nblocks;
        sp.total_vox = tp.total_vox;
        sp.T = T;
        sp.method = cfg.method;
        sp.order = cfg.trac_order;
        sp.iw = cfg.intensity_w;
        sp.state = ctx->tstate_ext ? ctx->tstate_ext : static_cast<float*>(ctx->tstate.p);
        sp.state_stride = ctx->tstate_ext ? ctx->tstate_ext_stride : ps.max_vox;
        sp.keep = ctx->keep_tstate ? 1 : 0;
        sp.rad_stack = rp.rad_stack;
        sp.int_stack = rp.int_stack;
        sp.out = out_dev;
        // Time batches: the radiality of volumes [t_lo, t_hi) into the stacks,
        // then that batch folded into the carried state (the map after the
        // last). With the whole series in one batch the stacks hold it all and
        // the one-pass temporal kernel reduces them. The events time the
        // radiality launches (with the carries of all batches but the last)
        // and the last temporal launch.
        if (evs) RFBA_CUDA(rec(evs[3 * i]), "event");
        // input windows (one pass over the whole series only): the radiality of
        // each window's volumes waits for that window's host copy
        const bool windows = win && ps.tb == 0 && ps.passes.size() == 1;
        const int nlaunch = windows ? win->n : ps.nbatch;
        for (int b = 0; b < nlaunch; ++b) {
            RadParams rb = rp;
            if (windows) {
                rb.t_lo = win->t[b];
                rb.t_hi = win->t[b + 1];
                RFBA_CUDA(cudaStreamWaitEvent(st, win->ready[b], 0), "input window wait");
            } else {
                rb.t_lo = b * tb;
                rb.t_hi = std::min(T, rb.t_lo + tb);
            }
            rb.stack_t0 = ps.tb > 0 ? rb.t_lo : 0;
            rb.nchunks = (rb.t_hi - rb.t_lo + pp.chunk - 1) / pp.chunk;
            rb.nitems = (long long)rb.ntiles * rb.nchunks;
            const int grid = (int)std::max<long long>(1, std::min<long long>(pp.grid, rb.nitems));
            RFBA_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned int), st), "counter reset");
            int le = launch_radiality(rb, grid, pp.smem, dtype == RFBA_U16, st);
            if (le != 0) return cuda_fail((cudaError_t)le, "radiality launch");
            if (ps.tb > 0) {
                const bool last = b == ps.nbatch - 1;
                if (last && evs) RFBA_CUDA(rec(evs[3 * i + 1]), "event");
                sp.t_lo = rb.t_lo;
                sp.t_hi = rb.t_hi;
                sp.last = last ? 1 : 0;
                le = launch_temporal_stream(sp, st);
                if (le != 0) return cuda_fail((cudaError_t)le, "temporal launch");
            }
        }
        if (ps.tb == 0) {
            if (evs) RFBA_CUDA(rec(evs[3 * i + 1]), "event");
            const int le = launch_temporal(tp, st);
            if (le != 0) return cuda_fail((cudaError_t)le, "temporal launch");
        }
        if (evs) RFBA_CUDA(rec(evs[3 * i + 2]), "event");
        if (verbose())
            std::fprintf(stderr,
                         "rfba: pass blocks=%zu tiles=%d ty=%d chunk=%d items=%lld grid=%d smem=%zu batches=%d of %d\n",
                         pp.b1 - pp.b0, rp.ntiles, ps.ty, pp.chunk, pp.nitems, pp.grid, pp.smem, ps.nbatch, tb);
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
    ctx->launches += (long long)ps.passes.size() * (ps.nwin > 0 ? ps.nwin + 1 : 2 * ps.nbatch);
    ctx->last_time_batch = ps.tb;
    ctx->last_batches = ps.tb > 0 ? ps.nbatch : 0;
    ctx->last_flop_units = 0;
    for (const PassPlan& pp : ps.passes) ctx->last_flop_units += pp.units;
}

// Run the device pipeline for all blocks now (no graph). in_dev / out_dev are
// device pointers.
static int run_device(rfba_ctx* ctx, const rfba_srrf_config& cfg, const void* in_dev, rfba_dtype dtype,
                      const int dims[4], const std::vector<BlockDev>& all, float* out_dev, cudaStream_t st,
                      const Tuning& tune = Tuning()) {
    ctx->train.valid = false;
    if (!ctx->tstate_ext) ctx->trainb.valid = false;
    PassSet ps;
    int s;
    if ((s = ctx->errw.ensure(256, "check word"))) return s;
    if ((s = plan_passes(ctx, cfg, dtype, dims, all, tune, &ps))) return s;
    const size_t np = ps.passes.size();
    if ((s = ctx->rad.ensure((size_t)ps.max_stack * 4, "radiality stack"))) return s;
    if ((s = ctx->inten.ensure((size_t)ps.max_stack * 4, "intensity stack"))) return s;
    if (ps.tb > 0 && !ctx->tstate_ext &&
        (s = ctx->tstate.ensure((size_t)ps.fields * ps.max_vox * 4, "temporal state")))
        return s;
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

// Volumes per time batch for a forward (0: the whole series at once). A
// series whose stacks fit the budget runs whole; a longer one runs in batches
// of kTimeBatch volumes with the temporal reduction carried between them, so
// the map is cut into fewer z slices (none when the carried state and one
// batch's stacks fit). TRAC with ITC 1 bins the whole series and slices
// instead. rfba_ctx_set_time_batch overrides the choice.
static constexpr int kTimeBatch = 25;
static int choose_time_batch(const rfba_ctx* ctx, const rfba_srrf_config& cfg, const int dims[4],
                             const rfba_block* blocks, int nblocks) {
    const int T = dims[3];
    if (cfg.method == 3 && cfg.itc == 1) return 0;
    if (ctx->time_batch < 0) return 0;
    if (ctx->time_batch > 0) return ctx->time_batch < T ? ctx->time_batch : 0;
    double vox = 0.0;
    for (int i = 0; i < nblocks; ++i) {
        double v = 1.0;
        for (int a = 0; a < 3; ++a) v *= std::max(blocks[i].hi[a] - blocks[i].lo[a], 0);
        vox += v;
    }
    if (vox * T * 2 * sizeof(float) <= (double)ctx->budget) return 0;
    return T > kTimeBatch ? kTimeBatch : 0;
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
    const int tb = choose_time_batch(ctx, *cfg, dims, blocks, nblocks);
    const int tfields = tb > 0 ? temporal_stream_fields(cfg->method, cfg->trac_order) : 0;
    std::vector<BlockDev> all;
    if ((s = make_blocks(ctx, *cfg, dims, blocks, nblocks, &all, 0, tb, tfields))) return s;
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
            (s = make_blocks(ctx, *cfg, dims, blocks, nblocks, &all, tune.ty, tb, tfields)))
            return s;
        tune.tb = tb;
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
            key_put(&gkey, &tb, 1);
            const int overlap = env_on("RFBA_OVERLAP", true) ? 1 : 0;
            key_put(&gkey, &overlap, 1);
            key_put(&gkey, blocks, (size_t)nblocks);
            const bool host = flags == RFBA_HOST_PTRS;
            auto deps_now = [&]() {
                return std::vector<const void*>{ctx->rad.p,   ctx->inten.p, ctx->tables.p,
                                                ctx->errw.p,  ctx->tstate.p,
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
                // Host input over one whole-series pass: the first tenth of the
                // volumes is copied first and the rest on a second stream while
                // the radiality of the first window runs
                const int T = dims[3];
                const bool windowed = overlap && host && g->ps.tb == 0 && g->ps.passes.size() == 1 && T >= 2;
                g->ps.nwin = windowed ? 2 : 0;
                const PassSet& ps = g->ps;
                const size_t np = ps.passes.size();
                if ((s = ctx->rad.ensure((size_t)ps.max_stack * 4, "radiality stack"))) return s;
                if ((s = ctx->inten.ensure((size_t)ps.max_stack * 4, "intensity stack"))) return s;
                if (ps.tb > 0 &&
                    (s = ctx->tstate.ensure((size_t)ps.fields * ps.max_vox * 4, "temporal state")))
                    return s;
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
                InputWindows win;
                if (windowed) {
                    if (!ctx->cap2) RFBA_CUDA(cudaStreamCreateWithFlags(&ctx->cap2, cudaStreamNonBlocking), "stream");
                    while (g->copy_evs.size() < 3) {
                        cudaEvent_t e;
                        RFBA_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
                        g->copy_evs.push_back(e);
                    }
                    win.n = 2;
                    win.t[0] = 0;
                    win.t[1] = std::max(1, T / 10);
                    win.t[2] = T;
                    win.ready = g->copy_evs.data() + 1;
                }
                const void* gin = host ? ctx->in.p : in;
                float* gout = host ? static_cast<float*>(ctx->out.p) : out;
                RFBA_CUDA(cudaStreamBeginCapture(ctx->cap, cudaStreamCaptureModeThreadLocal), "graph capture");
                int cs = RFBA_OK;
                cudaError_t ce = cudaSuccess;
                if (host && windowed) {
                    // fork: the copy stream takes the input windows, each followed by
                    // the event its radiality launch waits for (the last wait joins it)
                    const size_t vol = in_bytes / (size_t)T;
                    const size_t b0 = vol * (size_t)win.t[1];
                    ce = cudaEventRecord(g->copy_evs[0], ctx->cap);
                    if (ce == cudaSuccess) ce = cudaStreamWaitEvent(ctx->cap2, g->copy_evs[0], 0);
                    if (ce == cudaSuccess) ce = cudaMemcpyAsync(ctx->in.p, in, b0, cudaMemcpyHostToDevice, ctx->cap2);
                    if (ce == cudaSuccess) ce = cudaEventRecord(g->copy_evs[1], ctx->cap2);
                    if (ce == cudaSuccess)
                        ce = cudaMemcpyAsync(static_cast<char*>(ctx->in.p) + b0, static_cast<const char*>(in) + b0,
                                             in_bytes - b0, cudaMemcpyHostToDevice, ctx->cap2);
                    if (ce == cudaSuccess) ce = cudaEventRecord(g->copy_evs[2], ctx->cap2);
                    if (ce == cudaSuccess) ce = cudaMemsetAsync(gout, 0, (size_t)out_elems * 4, ctx->cap);
                } else if (host) {
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
                                        true, windowed ? &win : nullptr);
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
            ctx->trainb.valid = false;
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
    Tuning plain;
    plain.tb = tb;
    if ((s = run_device(ctx, *cfg, in_dev, dtype, dims, all, out_dev, st, plain))) return s;
    if (flags == RFBA_HOST_PTRS) {
        RFBA_CUDA(cudaMemcpyAsync(out, out_dev, (size_t)out_elems * 4, cudaMemcpyDeviceToHost, st), "output copy");
        return device_status(ctx, st, "forward");
    }
    return RFBA_OK;
}

// ---------------------------------------------------------------------------
// Differentiable path

// Volumes per batch of a drift-corrected forward that keeps its carried state
// for the backward, and of that backward (0: z slices). TRA and TRAC with ITC 0
// carry; a forced size (rfba_ctx_set_time_batch > 0) applies to both. The
// automatic choice batches TRAC with ITC 0 when the whole series' stacks
// exceed the budget: its forward keeps every slice's state, so the backward
// needs no extra forward pass and holds a fifth of the scratch of z slices.
static int drift_time_batch(const rfba_ctx* ctx, const rfba_srrf_config& cfg, int T, double vox) {
    if (!(cfg.method == 1 || (cfg.method == 3 && cfg.itc == 0))) return 0;
    if (ctx->time_batch < 0) return 0;
    if (ctx->time_batch > 0) return ctx->time_batch < T ? ctx->time_batch : 0;
    if (cfg.method == 3 && T > kTimeBatch && vox * T * 2 * sizeof(float) > (double)ctx->budget) return kTimeBatch;
    return 0;
}

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
    ctx->trainb.valid = false;
    const int T = dims[3];
    const double rvox = (double)(b.hi[0] - b.lo[0]) * (b.hi[1] - b.lo[1]) * (b.hi[2] - b.lo[2]);
    const int tbb = (!rlo && cfg->method == 3 && cfg->itc == 0) ? drift_time_batch(ctx, *cfg, T, rvox) : 0;
    if (tbb > 0) {
        // TRAC in forced time batches: the map in the z slices the backward
        // will use, every slice's final carried state kept (slice i at off[i],
        // stride total) so that the backward needs no state pass of its own
        if ((s = ensure_plan(ctx, *cfg, st))) return s;
        const int fields = temporal_stream_fields(3, cfg->trac_order);
        const int wl = std::min(T, tbb + 2 * (cfg->trac_order - 1));
        std::vector<BlockDev> all;
        if ((s = make_blocks(ctx, *cfg, dims, &b, 1, &all, 0, wl + tbb, fields))) return s;
        std::vector<long long> off;
        long long total = 0;
        for (const BlockDev& sl : all) {
            off.push_back(total);
            total += sl.vox;
        }
        if ((s = ctx->tstate.ensure((size_t)fields * (size_t)total * 4, "temporal state"))) return s;
        Tuning tt;
        tt.tb = tbb;
        for (size_t i = 0; i < all.size(); ++i) {
            std::vector<BlockDev> one(1, all[i]);
            ctx->tstate_ext = static_cast<float*>(ctx->tstate.p) + off[i];
            ctx->tstate_ext_stride = total;
            ctx->keep_tstate = true;
            s = run_device(ctx, *cfg, ip, RFBA_F32, dims, one, out, st, tt);
            ctx->tstate_ext = nullptr;
            ctx->keep_tstate = false;
            if (s) return s;
        }
        ctx->last_passes = (int)all.size();
        ctx->trainb.valid = true;
        ctx->trainb.cfg = *cfg;
        for (int a = 0; a < 4; ++a) ctx->trainb.dims[a] = dims[a];
        ctx->trainb.in = in;
        ctx->trainb.shifts = shifts;
        ctx->trainb.tb = tbb;
        ctx->trainb.slabs = all;
        ctx->trainb.off = off;
        ctx->trainb.total = total;
        return read_checks(ctx, st, "forward_shifted");
    }
    if ((s = forward_blocks_locked(ctx, cfg, ip, RFBA_F32, dims, &b, 1, out, n, RFBA_DEVICE_PTRS, st, false)))
        return s;
    // the backward can reuse this forward's stacks when they are all resident
    // (one spatial pass over the whole series at once: a forward in time batches
    // keeps only its last batch) and the temporal reduction left them intact
    // (ITC 1 bins the series in place)
    if (!rlo && ctx->last_passes == 1 && ctx->last_time_batch == 0 && !(cfg->method == 3 && cfg->itc == 1)) {
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
                        BlockDev blk, const float* gmap, long long ngmap, cudaStream_t st, int t_lo = 0,
                        int t_hi = 0) {
    // t_hi > 0: only the volumes [t_lo, t_hi), whose dL/dS and dL/dI the caller
    // has put in ctx->gS / ctx->gI from row 0 on (no temporal adjoint here)
    int s;
    const int T = dims[3];
    const bool window = t_hi > 0;
    const int TW = window ? t_hi - t_lo : T;
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
    if ((s = ctx->gS.ensure((size_t)V * TW * 4, "adjoint stack")) || (s = ctx->gI.ensure((size_t)V * TW * 4, "adjoint stack")) ||
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
    int e = 0;
    if (!window) {
        e = launch_temporal_adjoint(dblk, V, static_cast<const float*>(ctx->rad.p),
                                    static_cast<const float*>(ctx->inten.p), gmap, T, cfg->method, cfg->itc,
                                    cfg->trac_order, cfg->intensity_w, cfg->renormalize == 1, cfg->remove_con == 1,
                                    gS, gI, ngmap, err, st);
        if (e) return cuda_fail((cudaError_t)e, "temporal adjoint launch");
    }
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
    nch = std::max<long long>(1, std::min<long long>(nch, TW));
    rp.t_chunk = (int)((TW + nch - 1) / nch);
    rp.nchunks = (TW + rp.t_chunk - 1) / rp.t_chunk;
    rp.nitems = (long long)rp.ntiles * rp.nchunks;
    rp.t_lo = window ? t_lo : 0;
    rp.t_hi = window ? t_hi : T;
    rp.stack_t0 = rp.t_lo;
    const int grid = (int)std::max<long long>(1, std::min<long long>(slots, rp.nitems));
    AdjParams ap{gS, gI, static_cast<float*>(ctx->gin.p), (long long)nin, (long long)V * TW, err};
    e = launch_radiality_adjoint(rp, ap, grid, smem, st);
    if (e) return cuda_fail((cudaError_t)e, "radiality adjoint launch");
    ctx->launches += window ? 1 : 2;
    return RFBA_OK;
}

// Backward in time batches (TRA, TRAC with ITC 0), used when the context
// forces a time batch size: per z slice of the map, a state pass (the
// radiality of every batch folded into the carried temporal state, kept after
// the last batch), then per batch the radiality of the batch and of the k - 1
// volumes on either side that TRAC's lagged products reach, the batch's
// temporal adjoint from the state, and the radiality adjoint of its volumes
// into dL/dI'. Scratch per subvoxel: the window's stacks, the batch's adjoint
// stacks and the state, instead of the whole series' four stacks.
static int backward_batched(rfba_ctx* ctx, const rfba_srrf_config* cfg, const float* ip, const int dims[4],
                            const rfba_block& b, int tb, const float* gmap, long long nreg, cudaStream_t st,
                            bool kept) {
    // kept: the forward before this call ran in these batches and kept every
    // slice's final state (ctx->trainb): no state pass
    int s;
    const int T = dims[3];
    const bool trac = cfg->method == 3;
    const int h = trac ? cfg->trac_order - 1 : 0;
    // TRA's state pass runs TRAC-2's carry: its sum of y is finite exactly when
    // every radiality value of the series is
    rfba_srrf_config scfg = *cfg;
    if (!trac) {
        scfg.method = 3;
        scfg.itc = 0;
        scfg.trac_order = 2;
    }
    const int fields = temporal_stream_fields(3, scfg.trac_order);
    const int wl = std::min(T, tb + 2 * h);
    std::vector<BlockDev> all;
    if (kept)
        all = ctx->trainb.slabs;
    else if ((s = make_blocks(ctx, scfg, dims, &b, 1, &all, 0, wl + tb, fields)))
        return s;
    unsigned long long* err = static_cast<unsigned long long*>(ctx->errw.p);
    for (size_t si = 0; si < all.size(); ++si) {
        const BlockDev& slab = all[si];
        std::vector<BlockDev> one(1, slab);
        const float* state = static_cast<const float*>(ctx->tstate.p);
        long long sstride = slab.vox;
        if (kept) {
            state += ctx->trainb.off[si];
            sstride = ctx->trainb.total;
        } else {
            Tuning ts;
            ts.tb = tb;
            ctx->keep_tstate = true;
            s = run_device(ctx, scfg, ip, RFBA_F32, dims, one, static_cast<float*>(ctx->out.p), st, ts);
            ctx->keep_tstate = false;
            if (s) return s;
        }
        // the window plan: the same slab with wl volumes of stacks
        PassSet ps;
        Tuning tw;
        tw.tb = wl;
        if ((s = plan_passes(ctx, scfg, RFBA_F32, dims, one, tw, &ps))) return s;
        if (ps.passes.size() != 1) {
            set_error("time-batched backward: a slice does not fit one pass");
            return RFBA_ERR_UNSUPPORTED;
        }
        const PassPlan& pp = ps.passes[0];
        const long long V = slab.vox;
        if ((s = ctx->rad.ensure((size_t)V * wl * 4, "radiality stack")) ||
            (s = ctx->inten.ensure((size_t)V * wl * 4, "intensity stack")) ||
            (s = ctx->gS.ensure((size_t)V * tb * 4, "adjoint stack")) ||
            (s = ctx->gI.ensure((size_t)V * tb * 4, "adjoint stack")) ||
            (s = ctx->blocks.ensure(ps.blocks.size() * sizeof(BlockDev), "blocks")) ||
            (s = ctx->tiles.ensure(ps.tiles.size() * sizeof(TileDesc), "tiles")) ||
            (s = ctx->counter.ensure(256, "counter")))
            return s;
        RFBA_CUDA(cudaMemcpyAsync(ctx->blocks.p, ps.blocks.data(), ps.blocks.size() * sizeof(BlockDev),
                                  cudaMemcpyHostToDevice, st), "blocks upload");
        RFBA_CUDA(cudaMemcpyAsync(ctx->tiles.p, ps.tiles.data(), ps.tiles.size() * sizeof(TileDesc),
                                  cudaMemcpyHostToDevice, st), "tiles upload");
        const BlockDev* dblk = static_cast<const BlockDev*>(ctx->blocks.p);
        RadParams rp = fill_rad_params(ctx, scfg, ip, dims, cz_for_mag(scfg.mag[2]), ps.ty);
        rp.tma_bx = radiality_tma_box_x(rp, 0);
        rp.err = err;
        rp.blocks = dblk;
        rp.tiles = static_cast<const TileDesc*>(ctx->tiles.p);
        rp.ntiles = (int)(pp.t1 - pp.t0);
        rp.rad_stack = static_cast<float*>(ctx->rad.p);
        rp.int_stack = static_cast<float*>(ctx->inten.p);
        rp.work_counter = static_cast<unsigned int*>(ctx->counter.p);
        rp.t_chunk = pp.chunk;
        BlockDev blk = slab;
        blk.stack_off = 0;
        for (int t_lo = 0; t_lo < T; t_lo += tb) {
            const int t_hi = std::min(T, t_lo + tb);
            RadParams rb = rp;
            rb.t_lo = std::max(0, t_lo - h);
            rb.t_hi = std::min(T, t_hi + h);
            rb.stack_t0 = rb.t_lo;
            rb.nchunks = (rb.t_hi - rb.t_lo + pp.chunk - 1) / pp.chunk;
            rb.nitems = (long long)rb.ntiles * rb.nchunks;
            const int grid = (int)std::max<long long>(1, std::min<long long>(pp.grid, rb.nitems));
            RFBA_CUDA(cudaMemsetAsync(ctx->counter.p, 0, sizeof(unsigned int), st), "counter reset");
            int e = launch_radiality(rb, grid, pp.smem, 0, st);
            if (e) return cuda_fail((cudaError_t)e, "radiality launch");
            StreamAdjParams ap;
            std::memset(&ap, 0, sizeof ap);
            ap.block = dblk;
            ap.T = T;
            ap.t_lo = t_lo;
            ap.t_hi = t_hi;
            ap.w_lo = rb.t_lo;
            ap.w_hi = rb.t_hi;
            ap.method = cfg->method;
            ap.order = scfg.trac_order;
            ap.iw = cfg->intensity_w;
            ap.renorm = cfg->renormalize == 1;
            ap.poscon = cfg->remove_con == 1;
            ap.state = state;
            ap.state_stride = sstride;
            ap.rad = static_cast<const float*>(ctx->rad.p);
            ap.inten = static_cast<const float*>(ctx->inten.p);
            ap.gmap = gmap;
            ap.nmap = nreg;
            ap.gS = static_cast<float*>(ctx->gS.p);
            ap.gI = static_cast<float*>(ctx->gI.p);
            ap.err = err;
            e = launch_temporal_stream_adjoint(ap, V, st);
            if (e) return cuda_fail((cudaError_t)e, "temporal adjoint launch");
            ctx->launches += 2;
            if ((s = adjoint_slab(ctx, cfg, ip, dims, blk, gmap, nreg, st, t_lo, t_hi))) return s;
        }
    }
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
        RFBA_CUDA(cudaMemsetAsync(ctx->gin.p, 0, nin * 4, st), "adjoint clear");
        // batches when forced, or when the forward before this call ran in batches
        // and kept its state for these arguments (the automatic case)
        const bool kept_ok = !rlo && ctx->trainb.valid && same_cfg(ctx->trainb.cfg, *cfg) &&
                             ctx->trainb.in == in && ctx->trainb.shifts == shifts && ctx->trainb.dims[0] == dims[0] &&
                             ctx->trainb.dims[1] == dims[1] && ctx->trainb.dims[2] == dims[2] &&
                             ctx->trainb.dims[3] == dims[3];
        int btb = (cfg->method == 1 || (cfg->method == 3 && cfg->itc == 0)) && ctx->time_batch > 0 &&
                          ctx->time_batch < T
                      ? ctx->time_batch
                      : 0;
        if (btb == 0 && ctx->time_batch == 0 && kept_ok) btb = ctx->trainb.tb;
        const bool kept = btb > 0 && kept_ok && ctx->trainb.tb == btb;
        if (btb > 0) {
            if ((s = backward_batched(ctx, cfg, ip, dims, b, btb, gmap, nreg, st, kept))) return s;
        }
        std::vector<BlockDev> all;
        if (btb == 0 && (s = make_blocks(ctx, *cfg, dims, &b, 1, &all))) return s;
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
                      &c->tb_pix, &c->tb_pixels, &c->tb_dfd, &c->tb_vdf, &c->seed_w, &c->seed_sums, &c->seed_carry, &c->seed_map, &c->seed_vox,
                      &c->seed_xyz, &c->gb_pix, &c->gb_pixels, &c->gb_par, &c->hs_tab, &c->hs_part, &c->hs_gg, &c->hs_phi,
                      &c->hs_frame, &c->hs_out, &c->tstate})
        b->release();
    for (auto& g : c->gb) g.release();
    for (auto& e : c->ev)
        if (e) cudaEventDestroy(e);
    c->graphs.clear();
    for (cudaEvent_t e : c->pev) cudaEventDestroy(e);
    if (c->cap) cudaStreamDestroy(c->cap);
    if (c->cap2) cudaStreamDestroy(c->cap2);
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
    return seed_spots_locked(ctx, map, map_dims, mag, voxels, nvoxels, num_spots, seed, xyz, ptr_flags, st);
}

}  // extern "C"

namespace rfba {

// The seeding draw with the context already held and its stream ordered.
int seed_spots_locked(rfba_ctx* ctx, const float* map, const int map_dims[3], int mag, const int* voxels, int nvoxels,
                      int num_spots, unsigned long long seed, float* xyz, int ptr_flags, cudaStream_t st) {
    int s;
    const long long ncand = (long long)nvoxels * mag * mag * mag;
    const long long n1 = (ncand + 511) / 512, n2 = (n1 + 511) / 512;
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

}  // namespace rfba

extern "C" {

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
int rfba_ctx_set_time_batch(rfba_ctx* c, int volumes) {
    if (!c) return RFBA_ERR_INVALID;
    std::lock_guard<std::mutex> lk(c->mu);
    c->time_batch = volumes;
    return RFBA_OK;
}
int rfba_ctx_last_time_batches(rfba_ctx* c, int* volumes, int* batches, int* passes) {
    if (!c) return RFBA_ERR_INVALID;
    if (volumes) *volumes = c->last_time_batch;
    if (batches) *batches = c->last_batches;
    if (passes) *passes = c->last_passes;
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

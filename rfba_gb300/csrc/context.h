// The library context (rfba_ctx) and the host helpers its translation units
// share: the error string, CUDA-error mapping, stream ordering between calls.
// A context owns the device scratch of every entry point (grown on demand and
// kept), the cached ring plan and weight tables, autotuned schedules and
// captured graphs; one mutex serialises the calls made on it.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "devbuf.h"
#include "srrf_internal.h"

struct rfba_ctx;

namespace rfba {

void set_error(const std::string& msg);
// Records `what: <CUDA error>`; RFBA_ERR_NOMEM for an allocation failure,
// RFBA_ERR_CUDA otherwise.
int cuda_fail(cudaError_t e, const char* what);
// Makes `st` wait for the previous call's work when that call used another
// stream (calls share the context's scratch).
int order_streams(rfba_ctx* ctx, cudaStream_t st);
// RFBA_VERBOSE=1: per-call schedule and timing lines on stderr.
bool verbose();
// rfba_srrf_seed_spots with the context held and `st` ordered.
int seed_spots_locked(rfba_ctx* ctx, const float* map, const int map_dims[3], int mag, const int* voxels, int nvoxels,
                      int num_spots, unsigned long long seed, float* xyz, int ptr_flags, cudaStream_t st);

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
    int tb = 0;     // time batch (volumes per batch; 0 = the whole series at once)
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
    long long vox = 0;  // region subvoxels of the pass
};
struct PassSet {
    std::vector<BlockDev> blocks;
    std::vector<TileDesc> tiles;
    std::vector<long long> prefix;
    std::vector<PassPlan> passes;
    long long max_stack = 0;
    long long max_vox = 0;
    int ty = 0;
    // time batches: the stacks hold tb volumes and the temporal reduction is
    // carried across batches in `fields` floats per subvoxel (tb 0: the whole
    // series at once)
    int tb = 0, fields = 0, nbatch = 1;
    int nwin = 0;  // radiality launches per pass when the input copy is windowed (0: not)
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
    // fork of the copy stream and the end of each input copy window
    std::vector<cudaEvent_t> copy_evs;
    ~GraphPlan() {
        if (exec) cudaGraphExecDestroy(exec);
        for (cudaEvent_t e : evs) cudaEventDestroy(e);
        for (cudaEvent_t e : copy_evs) cudaEventDestroy(e);
        blocks.release();
        tiles.release();
        prefix.release();
        counters.release();
    }
};


// The device scratch of one Gibbs chain: its spots, spot intensities, masks,
// states, current sample, emission buffers, barrier counter and outputs.
struct GibbsScratch {
    DevBuf spots, si, moff, midx, state, cur, em, bar, var, ostate, oint, oerr, lp, filt;
    void release() {
        for (DevBuf* b : {&spots, &si, &moff, &midx, &state, &cur, &em, &bar, &var, &ostate, &oint, &oerr, &lp, &filt})
            b->release();
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
    // time batches of a forward (0 = automatic: batches of kTimeBatch volumes when
    // the whole series' stacks do not fit the budget, < 0 = never, > 0 = always,
    // this many volumes), what the last forward used, and the carried state
    int time_batch = 0;
    int last_time_batch = 0, last_batches = 0;
    rfba::DevBuf tstate;
    bool keep_tstate = false;  // a time-batched forward stores its final state (for the backward)
    // when set, the carried state lives here ([field][tstate_ext_stride]) instead of tstate
    float* tstate_ext = nullptr;
    long long tstate_ext_stride = 0;
    // a drift-corrected forward in time batches whose slices' final states are
    // kept in tstate (slice i at off[i], stride total) for the backward
    struct TrainBatched {
        bool valid = false;
        rfba_srrf_config cfg;
        int dims[4] = {0, 0, 0, 0};
        const void* in = nullptr;
        const void* shifts = nullptr;
        int tb = 0;
        std::vector<rfba::BlockDev> slabs;
        std::vector<long long> off;
        long long total = 0;
    } trainb;
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
    cudaStream_t cap = nullptr;   // stream the graphs are captured on
    cudaStream_t cap2 = nullptr;  // the captured input copies' stream
    std::map<std::string, std::pair<int, int>> tunes;  // schedule key -> (tile rows, tile order)
    std::vector<std::unique_ptr<rfba::GraphPlan>> graphs;  // most recent first
    // spot seeding scratch
    rfba::DevBuf seed_w, seed_sums, seed_carry, seed_map, seed_vox, seed_xyz;
    // 3B spot-gradient scratch
    rfba::DevBuf tb_val, tb_der, tb_em, tb_res, tb_par, tb_bg, tb_pix, tb_pixels, tb_dfd, tb_vdf;
    // 3B Gibbs sampler scratch
    rfba::DevBuf gb_pix, gb_pixels, gb_par;
    rfba::GibbsScratch gb[2];  // one set per chain run side by side
    // 3B sampled-background Hessian scratch
    rfba::DevBuf hs_tab, hs_part, hs_gg, hs_phi, hs_frame, hs_out;
    int last_ty = 0, last_order = 0, last_graph = 0, last_tuned = 0;
};

// Forward pass that allocates no device memory.
//
// Some callers cannot call cudaMalloc at the point where they need an SRRF map:
// acquisition loops that must not stall on cudaMalloc's device-wide
// synchronisation, hosts whose device memory is owned entirely by their own
// pool allocator, and plugin environments that forbid device allocation.
// rfba_srrf_forward_static_scratch serves them: the caller passes device input
// and output buffers, and every temporary (weight tables, block and tile
// descriptors, the work counter, the radiality and intensity stacks) lives in
// one file-scope device array of fixed size (kStaticScratchBytes). Each GPU
// that loads the library holds that array until the process exits.
//
// The array's address is looked up with cudaGetSymbolAddress once per device,
// on the first call made with that device current; that first call should come
// before any stream capture. Every call uses the same array and leaves its
// contents behind, so calls whose work overlaps on the GPU (different streams,
// or different host threads) race; serialise them. The work counter that must
// start at zero is cleared by each call on its stream.
//
// Nothing is copied from host memory: the block descriptor, the tile list, the
// voxel prefix and the weight tables reach the scratch through small set-up
// kernels that carry them in their launch parameters, so the call never reads
// a host buffer after it has returned and never waits on a pageable copy.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "srrf_internal.h"

namespace rfba {
bool config_validate(const rfba_srrf_config& c, std::string* err);
int ring_zero_pair(const RingPlan& rp);
}  // namespace rfba

namespace {

constexpr size_t kStaticScratchBytes = size_t(128) << 20;  // 128 MiB

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_setup_mu;
std::vector<void*> g_scratch_addr;  // per device ordinal, nullptr until set up

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

int fail(int status, const std::string& msg) {
    rfba::set_error(msg);
    return status;
}

// Address of g_static_scratch on the current device (looked up once).
int scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(RFBA_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if ((int)g_scratch_addr.size() <= dev) g_scratch_addr.resize(dev + 1, nullptr);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p)
            return fail(RFBA_ERR_CUDA, std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e));
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return RFBA_OK;
}

// Device memory of device `dev` (the current one), or managed memory, which
// every device can address. Memory of another GPU is refused: without peer
// access the kernels would fault on it, with peer access they would read and
// write across the link.
bool is_device_ptr(const void* p, int dev) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

using rfba::BlockDev;
using rfba::TileDesc;

// Set-up kernels: descriptors and tables travel in the launch parameters.
struct SetupArgs {
    BlockDev block;
    long long prefix[2];
    int ntile[3];
    int ntiles;
};

__global__ void static_setup_kernel(const SetupArgs a, BlockDev* blk, TileDesc* tiles, long long* prefix,
                                    unsigned int* counter) {
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (i0 == 0) {
        *blk = a.block;
        prefix[0] = a.prefix[0];
        prefix[1] = a.prefix[1];
    }
    if (i0 < 64) counter[i0] = 0u;
    // tile order: x fastest, then y, then z
    for (int i = i0; i < a.ntiles; i += gridDim.x * blockDim.x) {
        TileDesc d;
        d.block = 0;
        d.tx = i % a.ntile[0];
        d.ty = (i / a.ntile[0]) % a.ntile[1];
        d.tz = i / (a.ntile[0] * a.ntile[1]);
        tiles[i] = d;
    }
}

constexpr int kChunkWords = 960;  // 3.8 KB of parameters per launch
struct TableChunk {
    int n;
    float w[kChunkWords];
};

__global__ void static_tables_kernel(const TableChunk c, float* dst) {
    for (int i = threadIdx.x; i < c.n; i += blockDim.x) dst[i] = c.w[i];
}

}  // namespace

using namespace rfba;

extern "C" int rfba_srrf_forward_static_scratch(const rfba_srrf_config* cfg, const void* in, rfba_dtype dtype,
                                                const int dims[4], float* out, void* stream) {
    if (!cfg || !in || !dims || !out) return fail(RFBA_ERR_INVALID, "null argument");
    std::string err;
    if (!config_validate(*cfg, &err)) return fail(RFBA_ERR_INVALID, err);
    if (dtype != RFBA_F32 && dtype != RFBA_U16) return fail(RFBA_ERR_INVALID, "dtype must be RFBA_F32 or RFBA_U16");
    for (int a = 0; a < 4; ++a)
        if (dims[a] < 1) return fail(RFBA_ERR_INVALID, "dims must be positive");
    // sizes in 64 bits; the fixed scratch is checked before any host work
    const long long plane = (long long)dims[0] * dims[1] * dims[2];
    if (plane * dims[3] > (1LL << 40)) return fail(RFBA_ERR_INVALID, "input too large");
    long long nreg64[3];
    for (int a = 0; a < 3; ++a) nreg64[a] = (long long)dims[a] * cfg->mag[a];
    const long long vox64 = nreg64[0] * nreg64[1] * nreg64[2];
    const long long stack64 = vox64 * dims[3] * (long long)sizeof(float);
    // the two stacks alone (the tables, descriptors and tiles come on top)
    if (2 * stack64 > (long long)kStaticScratchBytes || nreg64[0] > INT32_MAX / 2 || nreg64[1] > INT32_MAX / 2 ||
        nreg64[2] > INT32_MAX / 2) {
        char buf[256];
        std::snprintf(buf, sizeof buf,
                      "volume needs at least %lld bytes of scratch; the static scratch holds %zu bytes "
                      "(use rfba_srrf_forward for this size)",
                      2 * stack64, kStaticScratchBytes);
        return fail(RFBA_ERR_UNSUPPORTED, buf);
    }
    int cur_dev = 0;
    {
        const cudaError_t e = cudaGetDevice(&cur_dev);
        if (e != cudaSuccess) return fail(RFBA_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    }
    if (!is_device_ptr(in, cur_dev) || !is_device_ptr(out, cur_dev))
        return fail(RFBA_ERR_INVALID,
                    "the static-scratch forward takes device pointers of the current device for input and output");
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // ring plan and tables
    RingPlan ring;
    std::vector<float> words;
    TableLayout tl;
    if (!build_ring_plan(*cfg, &ring, &err) || !build_tables(*cfg, ring, &words, &tl, &err))
        return fail(RFBA_ERR_UNSUPPORTED, err);
    const int zero_pair = ring_zero_pair(ring);
    if (zero_pair < 0) return fail(RFBA_ERR_UNSUPPORTED, "ring has no (0, 0) pair");

    // the whole volume as one block
    const int T = dims[3];
    const int mz = cfg->mag[2];
    const int FZ = mz * cz_for_mag(mz);
    const int TY = tile_rows_for_mag(cfg->mag[1]);
    BlockDev b;
    std::memset(&b, 0, sizeof b);
    for (int a = 0; a < 3; ++a) {
        b.size[a] = dims[a];
        b.lo[a] = 0;
        b.hi[a] = dims[a] * cfg->mag[a];
        b.nreg[a] = b.hi[a];
        const std::vector<float>& rc = a == 0 ? ring.rx : (a == 1 ? ring.ry : ring.rz);
        window_range(cfg->ring_radius, rc, cfg->mag[a], dims[a], &b.rad_lo[a], &b.rad_hi[a]);
        fine_window_int(cfg->mag[a], dims[a], &b.int_lo[a], &b.int_hi[a]);
    }
    b.zbase = 0;
    b.ntile[0] = (b.nreg[0] + kTileX - 1) / kTileX;
    b.ntile[1] = (b.nreg[1] + TY - 1) / TY;
    b.ntile[2] = (b.hi[2] + FZ - 1) / FZ;
    b.vox = (long long)b.nreg[0] * b.nreg[1] * b.nreg[2];
    b.stack_off = 0;
    b.out_offset = 0;
    b.out_stride[0] = 1;
    b.out_stride[1] = b.hi[0];
    b.out_stride[2] = (long long)b.hi[0] * b.hi[1];
    const long long ntiles64 = (long long)b.ntile[0] * b.ntile[1] * b.ntile[2];
    const long long prefix[2] = {0, b.vox};

    // scratch layout: tables | block | tiles | prefix | counter | radiality | intensity
    const size_t o_tab = 0;
    const size_t o_blk = align256(o_tab + words.size() * sizeof(float));
    const size_t o_til = align256(o_blk + sizeof(BlockDev));
    const size_t o_pre = align256(o_til + (size_t)ntiles64 * sizeof(TileDesc));
    const size_t o_cnt = align256(o_pre + sizeof(prefix));
    const size_t o_rad = align256(o_cnt + 256);
    const size_t stack_bytes = (size_t)b.vox * (size_t)T * sizeof(float);
    const size_t o_int = align256(o_rad + stack_bytes);
    const size_t need = o_int + stack_bytes;
    if (need > kStaticScratchBytes) {
        char buf[256];
        std::snprintf(buf, sizeof buf,
                      "volume needs %zu bytes of scratch; the static scratch holds %zu bytes "
                      "(use rfba_srrf_forward for this size)",
                      need, kStaticScratchBytes);
        return fail(RFBA_ERR_UNSUPPORTED, buf);
    }
    void* base = nullptr;
    int s = scratch_address(&base);
    if (s) return s;
    unsigned char* sc = static_cast<unsigned char*>(base);

    auto cuda_ok = [&](cudaError_t e, const char* what) -> int {
        if (e == cudaSuccess) return RFBA_OK;
        return fail(RFBA_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    };
    // tables, descriptors, tile list and the cleared work counter, written by
    // kernels from their launch parameters
    for (size_t w0 = 0; w0 < words.size(); w0 += kChunkWords) {
        TableChunk c;
        c.n = (int)std::min<size_t>(kChunkWords, words.size() - w0);
        std::memcpy(c.w, words.data() + w0, (size_t)c.n * sizeof(float));
        static_tables_kernel<<<1, 256, 0, st>>>(c, reinterpret_cast<float*>(sc + o_tab) + w0);
        if ((s = cuda_ok(cudaGetLastError(), "tables set-up"))) return s;
    }
    {
        SetupArgs a;
        std::memset(&a, 0, sizeof a);
        a.block = b;
        a.prefix[0] = prefix[0];
        a.prefix[1] = prefix[1];
        for (int k = 0; k < 3; ++k) a.ntile[k] = b.ntile[k];
        a.ntiles = (int)ntiles64;
        const int nb = (int)std::min<long long>(64, std::max<long long>(1, (ntiles64 + 255) / 256));
        static_setup_kernel<<<nb, 256, 0, st>>>(a, reinterpret_cast<BlockDev*>(sc + o_blk),
                                                reinterpret_cast<TileDesc*>(sc + o_til),
                                                reinterpret_cast<long long*>(sc + o_pre),
                                                reinterpret_cast<unsigned int*>(sc + o_cnt));
        if ((s = cuda_ok(cudaGetLastError(), "descriptor set-up"))) return s;
    }

    RadParams rp;
    std::memset(&rp, 0, sizeof rp);
    rp.in = in;
    rp.W = dims[0];
    rp.H = dims[1];
    rp.D = dims[2];
    rp.T = T;
    for (int a = 0; a < 3; ++a) rp.mag[a] = cfg->mag[a];
    rp.nxv = (int)ring.xv.size();
    rp.nyv = (int)ring.yv.size();
    rp.nzv = (int)ring.zv.size();
    rp.ngroups = (int)ring.grp_xval.size();
    rp.npairs = (int)ring.pair_yval.size();
    rp.npoints = (int)ring.pt_zval.size();
    rp.zero_pair = zero_pair;
    if (cfg->gradient_smooth == 0) {
        rp.gr[0] = 1;
        rp.gr[1] = rp.gr[2] = rp.gr[3] = 0;
    } else {
        rp.gr[0] = cfg->main_range;
        rp.gr[1] = cfg->x_range;
        rp.gr[2] = cfg->y_range;
        rp.gr[3] = cfg->z_range;
    }
    rp.R = std::max(std::max(rp.gr[0], rp.gr[1]), std::max(rp.gr[2], rp.gr[3]));
    rp.grad_mode = (rp.gr[0] == 1 && rp.gr[1] == 1 && rp.gr[2] == 1 && rp.gr[3] == 1)   ? 1
                   : (rp.gr[0] == 1 && rp.gr[1] == 0 && rp.gr[2] == 0 && rp.gr[3] == 0) ? 2
                                                                                       : 0;
    rp.TY = TY;
    rp.NU = (kTileX - 1) / cfg->mag[0] + 2 + 4;
    rp.NV = (TY - 1) / cfg->mag[1] + 2 + 4;
    rp.NW = cz_for_mag(mz) + 4;
    rp.NIX = rp.NU + 2 * rp.R;
    rp.NIY = rp.NV + 2 * rp.R;
    rp.NIZ = rp.NW + 2 * rp.R;
    rp.renorm = cfg->renormalize == 1;
    rp.poscon = cfg->remove_con == 1;
    rp.tables = reinterpret_cast<const float*>(sc + o_tab);
    rp.tl = tl;
    rp.smem_table_words = tl.words;
    rp.blocks = reinterpret_cast<const BlockDev*>(sc + o_blk);
    rp.tiles = reinterpret_cast<const TileDesc*>(sc + o_til);
    rp.ntiles = (int)ntiles64;
    rp.rad_stack = reinterpret_cast<float*>(sc + o_rad);
    rp.int_stack = reinterpret_cast<float*>(sc + o_int);
    rp.work_counter = reinterpret_cast<unsigned int*>(sc + o_cnt);
    const size_t smem = radiality_smem_bytes(rp);
    if (smem > 227 * 1024) return fail(RFBA_ERR_UNSUPPORTED, "shared memory tile too large for this configuration");
    int per_sm = 0, dev = 0, sms = 0;
    if ((s = cuda_ok((cudaError_t)radiality_max_ctas_per_sm(rp, dtype == RFBA_U16, &per_sm), "occupancy"))) return s;
    if ((s = cuda_ok(cudaGetDevice(&dev), "cudaGetDevice"))) return s;
    if ((s = cuda_ok(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count"))) return s;
    if (per_sm < 1) return fail(RFBA_ERR_UNSUPPORTED, "radiality kernel does not fit on an SM");
    const int slots = per_sm * sms;
    long long nch = (8LL * slots + rp.ntiles - 1) / rp.ntiles;
    nch = std::max<long long>(1, std::min<long long>(nch, T));
    rp.t_chunk = (int)((T + nch - 1) / nch);
    rp.nchunks = (T + rp.t_chunk - 1) / rp.t_chunk;
    rp.nitems = (long long)rp.ntiles * rp.nchunks;
    const int grid = (int)std::max<long long>(1, std::min<long long>(slots, rp.nitems));

    TemporalParams tp;
    std::memset(&tp, 0, sizeof tp);
    tp.blocks = rp.blocks;
    tp.vox_prefix = reinterpret_cast<const long long*>(sc + o_pre);
    tp.nblocks = 1;
    tp.total_vox = b.vox;
    tp.T = T;
    tp.method = cfg->method;
    tp.itc = cfg->itc;
    tp.order = cfg->trac_order;
    tp.iw = cfg->intensity_w;
    tp.rad_stack = rp.rad_stack;
    tp.int_stack = rp.int_stack;
    tp.out = out;

    if ((s = cuda_ok((cudaError_t)launch_radiality(rp, grid, smem, dtype == RFBA_U16, st), "radiality launch")))
        return s;
    if ((s = cuda_ok((cudaError_t)launch_temporal(tp, st), "temporal launch"))) return s;
    return RFBA_OK;
}

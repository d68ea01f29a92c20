// rfba-srrf: the `--srrf_only 1` step of RFBA.bat (first line written by
// GenerateBlock.m:91) on librfba_srrf.so.
//
//   rfba-srrf [--srrf_only 1] [--save_spots F] [--log_ratios F] [--info] cell1.tif cell2.tif ...
//
// Each TIFF file is one volume (one page per z slice, 8- or 16-bit grey,
// uncompressed strips, either byte order), the files in order are the time
// points — the per-volume files GenerateBlock.m:27-52 writes. As the reference
// does with the shipped multispot5.cfg (preprocess.skip=1,
// preprocess.fixed_scaling=0), every voxel is divided by the standard deviation
// over all voxels of all volumes (storm_imagery.cc:358-416 with the double sums
// of storm_imagery_no_load.cc:87-108), the series is packed [t][z][y][x]
// (multispot5_place_methods.cc:236-249), SRRFGetMag / SRRFGradientCalc run with
// ./SRRF.ini, NaN and negative values become 0 (multispot5_place_methods.cc:260-
// 269) and the map is written raw, float32 little-endian, x fastest, to
// ./SRRF.raw (multispot5_place_methods.cc:272-274). --save_spots and
// --log_ratios belong to the later 3B steps and are accepted and ignored.
// --info prints each file's size and a checksum and stops (no GPU needed).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/rfba_srrf.h"

namespace {

struct Volume {
    int w = 0, h = 0, d = 0, bits = 0;
    std::vector<float> v;  // [z][y][x]
};

struct Reader {
    std::vector<unsigned char> b;
    bool be = false;
    bool ok(size_t off, size_t n) const { return off <= b.size() && n <= b.size() - off; }
    uint32_t u16(size_t o) const {
        return be ? (uint32_t)(b[o] << 8 | b[o + 1]) : (uint32_t)(b[o] | b[o + 1] << 8);
    }
    uint32_t u32(size_t o) const {
        return be ? ((uint32_t)b[o] << 24 | (uint32_t)b[o + 1] << 16 | (uint32_t)b[o + 2] << 8 | b[o + 3])
                  : ((uint32_t)b[o] | (uint32_t)b[o + 1] << 8 | (uint32_t)b[o + 2] << 16 | (uint32_t)b[o + 3] << 24);
    }
    // value i of a SHORT or LONG tag entry at e
    bool value(size_t e, uint32_t i, uint32_t* out) const {
        const uint32_t type = u16(e + 2), cnt = u32(e + 4);
        if (i >= cnt) return false;
        const size_t sz = type == 3 ? 2 : (type == 4 ? 4 : 0);
        if (!sz) return false;
        size_t at = (size_t)cnt * sz <= 4 ? e + 8 : u32(e + 8);
        at += (size_t)i * sz;
        if (!ok(at, sz)) return false;
        *out = sz == 2 ? u16(at) : u32(at);
        return true;
    }
};

bool load_tiff(const char* path, Volume* vol, std::string* err) {
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        *err = "cannot open";
        return false;
    }
    Reader r;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    r.b.resize(n > 0 ? (size_t)n : 0);
    const size_t got = r.b.empty() ? 0 : std::fread(r.b.data(), 1, r.b.size(), f);
    std::fclose(f);
    if (got != r.b.size() || r.b.size() < 8) {
        *err = "short file";
        return false;
    }
    if (r.b[0] == 'M' && r.b[1] == 'M')
        r.be = true;
    else if (!(r.b[0] == 'I' && r.b[1] == 'I')) {
        *err = "not a TIFF";
        return false;
    }
    if (r.u16(2) != 42) {
        *err = "not a classic TIFF";
        return false;
    }
    size_t ifd = r.u32(4);
    int pages = 0;
    while (ifd) {
        if (!r.ok(ifd, 2)) {
            *err = "bad directory offset";
            return false;
        }
        const uint32_t ne = r.u16(ifd);
        if (!r.ok(ifd + 2, (size_t)ne * 12 + 4)) {
            *err = "bad directory";
            return false;
        }
        uint32_t w = 0, h = 0, bits = 1, comp = 1, spp = 1;
        size_t e_off = 0, e_cnt = 0;
        for (uint32_t k = 0; k < ne; ++k) {
            const size_t e = ifd + 2 + (size_t)k * 12;
            const uint32_t tag = r.u16(e);
            switch (tag) {
                case 256: r.value(e, 0, &w); break;
                case 257: r.value(e, 0, &h); break;
                case 258: r.value(e, 0, &bits); break;
                case 259: r.value(e, 0, &comp); break;
                case 277: r.value(e, 0, &spp); break;
                case 273: e_off = e; break;
                case 279: e_cnt = e; break;
                default: break;
            }
        }
        if (comp != 1 || spp != 1 || (bits != 8 && bits != 16) || !w || !h || !e_off || !e_cnt) {
            *err = "unsupported page (needs uncompressed 8/16-bit grey strips)";
            return false;
        }
        if (pages == 0) {
            vol->w = (int)w;
            vol->h = (int)h;
            vol->bits = (int)bits;
        } else if ((int)w != vol->w || (int)h != vol->h || (int)bits != vol->bits) {
            *err = "pages differ in size or depth";
            return false;
        }
        const size_t bps = bits / 8;
        const size_t plane = (size_t)w * h;
        const size_t base = vol->v.size();
        vol->v.resize(base + plane);
        size_t filled = 0;
        const uint32_t nstrips = r.u32(e_off + 4);
        for (uint32_t sidx = 0; sidx < nstrips && filled < plane; ++sidx) {
            uint32_t so = 0, sc = 0;
            if (!r.value(e_off, sidx, &so) || !r.value(e_cnt, sidx, &sc) || !r.ok(so, sc)) {
                *err = "bad strip";
                return false;
            }
            const size_t px = std::min<size_t>(sc / bps, plane - filled);
            for (size_t i = 0; i < px; ++i) {
                const size_t at = so + i * bps;
                vol->v[base + filled + i] = bps == 1 ? (float)r.b[at] : (float)r.u16(at);
            }
            filled += px;
        }
        if (filled != plane) {
            *err = "strips shorter than the page";
            return false;
        }
        ++pages;
        ifd = r.u32(ifd + 2 + (size_t)ne * 12);
    }
    vol->d = pages;
    return pages > 0;
}

}  // namespace

int main(int argc, char** argv) {
    std::vector<std::string> files;
    bool info = false;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "--info") {
            info = true;
        } else if (a == "--srrf_only" || a == "--save_spots" || a == "--log_ratios") {
            ++i;  // value belongs to the option
        } else if (a.size() > 2 && a[0] == '-' && a[1] == '-') {
            std::fprintf(stderr, "rfba-srrf: unknown option %s\n", a.c_str());
            return 2;
        } else {
            files.push_back(a);
        }
    }
    if (files.empty()) {
        std::fprintf(stderr, "usage: rfba-srrf [--srrf_only 1] [--info] cell1.tif cell2.tif ...\n");
        return 2;
    }
    std::vector<Volume> vols(files.size());
    for (size_t i = 0; i < files.size(); ++i) {
        std::string err;
        if (!load_tiff(files[i].c_str(), &vols[i], &err)) {
            std::fprintf(stderr, "rfba-srrf: %s: %s\n", files[i].c_str(), err.c_str());
            return 1;
        }
        if (vols[i].w != vols[0].w || vols[i].h != vols[0].h || vols[i].d != vols[0].d) {
            std::fprintf(stderr, "rfba-srrf: %s: all images must be the same size\n", files[i].c_str());
            return 1;
        }
        if (info) {
            double sum = 0.0;
            for (float x : vols[i].v) sum += x;
            std::printf("%s %d %d %d %d %.17g\n", files[i].c_str(), vols[i].w, vols[i].h, vols[i].d, vols[i].bits, sum);
        }
    }
    if (info) return 0;
    // global mean and variance, volume by volume: double sums of the voxels and of
    // their float squares (utility.h:48 sq(float)), storm_imagery_no_load.cc:87-108,
    // returned as floats; then every voxel divided by sqrt(variance)
    // (storm_imagery.cc:400-405)
    double sum = 0.0, sum2 = 0.0, area = 0.0;
    for (const Volume& v : vols) {
        area += (double)v.v.size();
        for (float x : v.v) {
            const float sq = x * x;
            sum += x;
            sum2 += sq;
        }
    }
    sum /= area;
    sum2 /= area;
    const double variance = (double)(float)(sum2 - sum * sum);
    const double sd = std::sqrt(variance);
    int dims[4] = {vols[0].w, vols[0].h, vols[0].d, (int)vols.size()};
    const size_t nv = (size_t)dims[0] * dims[1] * dims[2];
    std::vector<float> in(nv * dims[3]);
    for (int t = 0; t < dims[3]; ++t)
        for (size_t j = 0; j < nv; ++j) in[(size_t)t * nv + j] = (float)(vols[t].v[j] / sd);
    const int mag = SRRFGetMag();
    if (mag < 1) {
        std::fprintf(stderr, "rfba-srrf: bad magnification in SRRF.ini\n");
        return 1;
    }
    const size_t nout = nv * (size_t)mag * mag * mag;
    std::vector<float> out(nout);
    const int st = SRRFGradientCalc(in.data(), dims, out.data());
    if (st != 0) {
        std::fprintf(stderr, "rfba-srrf: SRRFGradientCalc failed (%d): %s\n", st, rfba_last_error());
        return 1;
    }
    for (float& x : out)
        if (std::isnan(x) || x < 0.f) x = 0.f;
    FILE* fp = std::fopen("SRRF.raw", "wb");
    if (!fp || std::fwrite(out.data(), sizeof(float), nout, fp) != nout) {
        std::fprintf(stderr, "rfba-srrf: cannot write SRRF.raw\n");
        if (fp) std::fclose(fp);
        return 1;
    }
    std::fclose(fp);
    return 0;
}

// CombineBlock: the reconstruction after 3B (Matlab Scripts/CombineBlock.m with
// genpsf.m and loadResult.m), host side: the PSF table, the result-file parser
// and the C-ABI of the GPU renderer (combine.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "srrf_internal.h"

namespace rfba {

void set_error(const std::string& msg);

namespace {

// fspecial('gaussian', [rows cols], sigma): exp(-(x^2 + y^2) / (2 sigma^2)) on
// the grid centred at (size - 1) / 2, values below eps * max set to 0, then
// normalised to unit sum (column-major accumulation order).
std::vector<double> gaussian2d(int rows, int cols, double sigma) {
    std::vector<double> h((size_t)rows * cols);
    const double cr = (rows - 1) / 2.0, cc = (cols - 1) / 2.0;
    double mx = 0.0;
    for (int j = 0; j < cols; ++j)
        for (int i = 0; i < rows; ++i) {
            const double x = j - cc, y = i - cr;
            const double v = std::exp(-(x * x + y * y) / (2.0 * sigma * sigma));
            h[(size_t)j * rows + i] = v;  // column-major, as the reference's arrays
            mx = std::max(mx, v);
        }
    const double eps = 2.220446049250313e-16;
    double sum = 0.0;
    for (double& v : h) {
        if (v < eps * mx) v = 0.0;
        sum += v;
    }
    if (sum != 0.0)
        for (double& v : h) v /= sum;
    return h;
}

// MATLAB uint16(): round half away from zero, saturate, NaN -> 0
uint16_t to_u16(double v) {
    if (!(v == v)) return 0;
    if (v <= 0.0) return 0;
    if (v >= 65535.0) return 65535;
    return (uint16_t)std::floor(v + 0.5);
}

}  // namespace

// genpsf.m: separable Gaussian (generation size 100, sigma in xy and z), scaled
// to 65535 at its maximum, rounded to uint16 and cropped symmetrically where the
// middle slice's rows / columns and the slices stay at or below the threshold.
// Output [z][row][col] (row = the first array dimension, y in CombineBlock).
bool genpsf(double sigma, double thr, std::vector<uint16_t>* out, int* nrow, int* ncol, int* nz, std::string* err) {
    const int g = 100;
    std::vector<double> xy = gaussian2d(g, g, sigma);
    double mxy = 0.0;
    for (double v : xy) mxy = std::max(mxy, v);
    for (double& v : xy) v *= 65535.0 / mxy;
    std::vector<double> zl = gaussian2d(1, g, sigma);
    double mz = 0.0;
    for (double v : zl) mz = std::max(mz, v);
    for (double& v : zl) v *= 65535.0 / mz;
    // h(:, :, k) = xy * z(k), then scaled so that max(h) = 65535
    double mh = 0.0;
    for (int k = 0; k < g; ++k)
        for (size_t i = 0; i < xy.size(); ++i) mh = std::max(mh, xy[i] * zl[k]);
    std::vector<uint16_t> psf((size_t)g * g * g);  // column-major (row, col, slice)
    for (int k = 0; k < g; ++k)
        for (size_t i = 0; i < xy.size(); ++i) psf[(size_t)k * g * g + i] = to_u16(xy[i] * zl[k] * (65535.0 / mh));
    auto P = [&](int r, int c, int k) -> int { return psf[(size_t)k * g * g + (size_t)c * g + r]; };  // 0-based
    const int half = (int)std::lround(g / 2.0);  // round(sz/2) = 50 (1-based)
    const int mid = half - 1;                     // 0-based middle slice
    auto rowmax = [&](int r) {
        int m = 0;
        for (int c = 0; c < g; ++c) m = std::max(m, P(r, c, mid));
        return m;
    };
    auto colmax = [&](int c) {
        int m = 0;
        for (int r = 0; r < g; ++r) m = std::max(m, P(r, c, mid));
        return m;
    };
    // rows (genpsf's "x" crop), 1-based indices as in the script
    int x1 = 0;
    for (int i = 1; i <= half; ++i)
        if (rowmax(i - 1) <= thr) x1 = i;
    x1 += 1;
    int x2 = g;
    for (int i = half; i <= g; ++i)
        if (rowmax(i - 1) > thr) x2 = i;
    x1 = std::min(x1, g - x2 + 1);
    x2 = g - x1 + 1;
    int y1 = 0;
    for (int i = 1; i <= half; ++i)
        if (colmax(i - 1) <= thr) y1 = i;
    y1 += 1;
    int y2 = g;
    for (int i = half; i <= g; ++i)
        if (colmax(i - 1) > thr) y2 = i;
    y1 = std::min(y1, g - y2 + 1);
    y2 = g - y1 + 1;
    auto slicemax = [&](int k) {
        int m = 0;
        for (int c = y1 - 1; c < y2; ++c)
            for (int r = x1 - 1; r < x2; ++r) m = std::max(m, P(r, c, k));
        return m;
    };
    int z1 = 0;
    for (int i = 1; i <= half; ++i)
        if (slicemax(i - 1) <= thr) z1 = i;
    z1 += 1;
    int z2 = -1;
    for (int i = half; i <= g; ++i)
        if (slicemax(i - 1) > thr) z2 = i;
    if (z2 < 0) {
        *err = "no PSF slice above the crop threshold";
        return false;
    }
    z1 = std::min(z1, g - z2 + 1);
    z2 = g - z1 + 1;
    *nrow = x2 - x1 + 1;
    *ncol = y2 - y1 + 1;
    *nz = z2 - z1 + 1;
    out->assign((size_t)(*nrow) * (*ncol) * (*nz), 0);
    for (int k = 0; k < *nz; ++k)
        for (int r = 0; r < *nrow; ++r)
            for (int c = 0; c < *ncol; ++c)
                (*out)[((size_t)k * (*nrow) + r) * (*ncol) + c] = (uint16_t)P(x1 - 1 + r, y1 - 1 + c, z1 - 1 + k);
    return true;
}

// loadResult.m: every "PASS..." line's numbers after ": " are spots of 5 values
// (intensity, blur, x, y, z); a spot is kept when its position relative to the
// block (x - start + 1, start 1-based) lies strictly inside (border, size - border)
// on all three axes.
bool load_result(const char* path, int border, const int start[3], const int size[3], std::vector<double>* spots,
                 std::string* err) {
    std::ifstream f(path);
    if (!f) {
        *err = std::string("cannot open ") + path;
        return false;
    }
    std::string line;
    while (std::getline(f, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        if (line.size() <= 5 || line.compare(0, 4, "PASS") != 0) continue;
        const size_t colon = line.find(':');
        const size_t from = colon == std::string::npos ? 6 : colon + 2;
        if (from > line.size()) continue;
        std::istringstream is(line.substr(from));
        std::vector<double> v;
        double d;
        while (is >> d) v.push_back(d);
        for (size_t i = 0; i + 5 <= v.size(); i += 5) {
            const double x = v[i + 2] - start[0] + 1, y = v[i + 3] - start[1] + 1, z = v[i + 4] - start[2] + 1;
            if (x > border && x < size[0] - border && y > border && y < size[1] - border && z > border &&
                z < size[2] - border)
                spots->insert(spots->end(), v.begin() + i, v.begin() + i + 5);
        }
    }
    return true;
}

}  // namespace rfba

using namespace rfba;

extern "C" {

int rfba_combine_psf(double sigma, double crop_threshold, uint16_t* psf, long long cap, int psf_dims[3]) {
    if (!psf_dims || sigma <= 0.0) {
        set_error("bad PSF arguments");
        return RFBA_ERR_INVALID;
    }
    std::vector<uint16_t> p;
    int nr, nc, nz;
    std::string err;
    if (!genpsf(sigma, crop_threshold, &p, &nr, &nc, &nz, &err)) {
        set_error(err);
        return RFBA_ERR_INVALID;
    }
    psf_dims[0] = nc;  // x (columns)
    psf_dims[1] = nr;  // y (rows)
    psf_dims[2] = nz;
    if (psf && cap >= (long long)p.size()) std::memcpy(psf, p.data(), p.size() * 2);
    return (int)p.size();
}

int rfba_combine_load_result(const char* path, int border, const int block_start[3], const int block_size[3],
                             double* spots, long long cap, long long* nspots) {
    if (!path || !block_start || !block_size || !nspots) {
        set_error("null argument");
        return RFBA_ERR_INVALID;
    }
    std::vector<double> v;
    std::string err;
    if (!load_result(path, border, block_start, block_size, &v, &err)) {
        set_error(err);
        return RFBA_ERR_IO;
    }
    *nspots = (long long)(v.size() / 5);
    if (spots && cap >= *nspots) std::memcpy(spots, v.data(), v.size() * sizeof(double));
    return RFBA_OK;
}

}  // extern "C"

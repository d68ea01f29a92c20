// Host planning for the radiality kernels: configuration (INI), ring
// deduplication and per-axis factorisation, separable Catmull-Rom weight
// tables, interpolation windows and block lists.
#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "srrf_internal.h"

namespace rfba {

// ---------------------------------------------------------------------------
// Configuration

// GradientCalc.cpp:19-41 defaults.
void config_default(rfba_srrf_config* c) {
    c->ring_radius = 0.5f;
    c->mag[0] = c->mag[1] = c->mag[2] = 5;
    c->axes_in_ring = 6;
    c->main_range = 1;
    c->x_range = c->y_range = c->z_range = 0;
    c->method = 1;
    c->itc = 1;
    c->trac_order = 2;
    c->remove_con = 0;
    c->renormalize = 0;
    c->gradient_smooth = 0;
    c->intensity_w = 1;
    c->block_size[0] = c->block_size[1] = c->block_size[2] = 16;
}

namespace {
std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}
bool ieq(const std::string& a, const std::string& b) {
    if (a.size() != b.size()) return false;
    for (size_t i = 0; i < a.size(); ++i)
        if (std::tolower((unsigned char)a[i]) != std::tolower((unsigned char)b[i])) return false;
    return true;
}
}  // namespace

// Profile-file reader with the lookup rules the reference relies on
// (GetPrivateProfileString/Int, GradientCalc.cpp:15-42): section and key
// names are case-insensitive, the first matching key wins, a missing file,
// section or key gives the default, integers parse like atoi.
struct Ini {
    std::vector<std::tuple<std::string, std::string, std::string>> kv;
    bool load(const char* path) {
        FILE* f = std::fopen(path, "r");
        if (!f) return false;
        char line[2048];
        std::string sec;
        while (std::fgets(line, sizeof line, f)) {
            std::string l = trim(line);
            if (l.empty() || l[0] == ';') continue;
            if (l[0] == '[') {
                size_t e = l.find(']');
                sec = trim(l.substr(1, e == std::string::npos ? std::string::npos : e - 1));
                continue;
            }
            size_t eq = l.find('=');
            if (eq == std::string::npos) continue;
            std::string v = trim(l.substr(eq + 1));
            if (v.size() >= 2 && v.front() == '"' && v.back() == '"') v = v.substr(1, v.size() - 2);
            kv.emplace_back(sec, trim(l.substr(0, eq)), v);
        }
        std::fclose(f);
        return true;
    }
    const std::string* find(const char* sec, const char* key) const {
        for (auto& e : kv)
            if (ieq(std::get<0>(e), sec) && ieq(std::get<1>(e), key)) return &std::get<2>(e);
        return nullptr;
    }
    int geti(const char* sec, const char* key, int def) const {
        const std::string* v = find(sec, key);
        return v ? std::atoi(v->c_str()) : def;
    }
    float getf(const char* sec, const char* key, float def) const {
        const std::string* v = find(sec, key);
        return v ? (float)std::atof(v->c_str()) : def;
    }
};

bool config_load_ini(const char* path, rfba_srrf_config* c) {
    config_default(c);
    Ini ini;
    bool ok = ini.load(path);
    c->ring_radius = ini.getf("SRRF", "RingRadius", 0.5f);
    int m = ini.geti("SRRF", "Magnification", 5);
    c->mag[0] = c->mag[1] = c->mag[2] = m;
    c->axes_in_ring = ini.geti("SRRF", "AxesinRing", 6);
    c->main_range = ini.geti("SRRF", "MainRange", 1);
    c->x_range = ini.geti("SRRF", "XRange", 0);
    c->y_range = ini.geti("SRRF", "YRange", 0);
    c->z_range = ini.geti("SRRF", "ZRange", 0);
    c->method = ini.geti("Temproal", "Method", 1);
    c->itc = ini.geti("Temproal", "Integrate_Temporal_Correlations", 1);
    c->trac_order = ini.geti("Temproal", "TRAC_ORDER", 2);
    c->remove_con = ini.geti("Radiality", "Remove_Positivity_Constraint", 0);
    c->renormalize = ini.geti("Radiality", "Renormalize", 0);
    c->gradient_smooth = ini.geti("Radiality", "Gradient_Smoothing", 0);
    c->intensity_w = ini.geti("Weighting", "Intensity_Weighting", 1);
    c->block_size[0] = ini.geti("Split", "BlockSizeX", 16);
    c->block_size[1] = ini.geti("Split", "BlockSizeY", 16);
    c->block_size[2] = ini.geti("Split", "BlockSizeZ", 16);
    return ok;
}

bool config_validate(const rfba_srrf_config& c, std::string* err) {
    char buf[256];
    for (int a = 0; a < 3; ++a)
        if (c.mag[a] < 1 || c.mag[a] > kMaxMag) {
            std::snprintf(buf, sizeof buf, "magnification %d on axis %d outside [1, %d]", c.mag[a], a, kMaxMag);
            *err = buf;
            return false;
        }
    if (!(c.ring_radius > 0.f) || !std::isfinite(c.ring_radius)) {
        *err = "ring radius must be a positive number";
        return false;
    }
    if (c.axes_in_ring < 1 || c.axes_in_ring > 32) {
        *err = "AxesinRing must be in [1, 32]";
        return false;
    }
    const int rs[4] = {c.main_range, c.x_range, c.y_range, c.z_range};
    for (int r : rs)
        if (r < 0 || r > kMaxGradRange) {
            std::snprintf(buf, sizeof buf, "gradient ranges must be in [0, %d]", kMaxGradRange);
            *err = buf;
            return false;
        }
    if (c.method < 0 || c.method > 3) {
        *err = "Method must be 0 (TRM), 1 (TRA), 2 (TRPPM) or 3 (TRAC)";
        return false;
    }
    if (c.method == 3 && (c.trac_order < 2 || c.trac_order > 4)) {
        *err = "TRAC_ORDER must be 2, 3 or 4";
        return false;
    }
    return true;
}

// ---------------------------------------------------------------------------
// Ring

// kernel.cu:17 and :23-33: float angle step (PI = 3.141592654f), float sin/cos,
// (r * sin) * cos association.
static void raw_ring(float r, int n, std::vector<float>& x, std::vector<float>& y, std::vector<float>& z) {
    x.resize(n * n);
    y.resize(n * n);
    z.resize(n * n);
    const float step = (3.141592654f * 2.0f) / (float)n;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            const int k = i * n + j;
            x[k] = r * std::sin(step * (float)i) * std::cos(step * (float)j);
            y[k] = r * std::sin(step * (float)i) * std::sin(step * (float)j);
            z[k] = r * std::cos(step * (float)i);
        }
}

static int value_index(std::vector<float>& vals, float v, float tol) {
    for (size_t i = 0; i < vals.size(); ++i)
        if (std::fabs(vals[i] - v) <= tol) return (int)i;
    vals.push_back(v);
    return (int)vals.size() - 1;
}

bool build_ring_plan(const rfba_srrf_config& c, RingPlan* rp, std::string* err) {
    const int n = 2 * c.axes_in_ring;
    const float r = c.ring_radius;
    rp->n = n;
    raw_ring(r, n, rp->rx, rp->ry, rp->rz);
    rp->npoints_raw = n * n;
    // Points that coincide up to float rounding of sin/cos (|d| <= 1e-6 r) are
    // one point with a multiplicity; coordinates within 1e-6 r of 0 are 0.
    const float tol = 1e-6f * r;
    auto snap = [&](float v) { return std::fabs(v) <= tol ? 0.f : v; };
    std::vector<std::array<float, 3>> reps;
    std::vector<int> mult;
    for (int i = 0; i < n * n; ++i) {
        const float px = snap(rp->rx[i]), py = snap(rp->ry[i]), pz = snap(rp->rz[i]);
        int found = -1;
        for (size_t k = 0; k < reps.size(); ++k)
            if (std::fabs(reps[k][0] - px) <= tol && std::fabs(reps[k][1] - py) <= tol &&
                std::fabs(reps[k][2] - pz) <= tol) {
                found = (int)k;
                break;
            }
        if (found < 0) {
            reps.push_back({px, py, pz});
            mult.push_back(1);
        } else
            mult[found]++;
    }
    // distinct axis values, sorted
    std::vector<float> xv, yv, zv;
    for (auto& p : reps) {
        value_index(xv, p[0], tol);
        value_index(yv, p[1], tol);
        value_index(zv, p[2], tol);
    }
    std::sort(xv.begin(), xv.end());
    std::sort(yv.begin(), yv.end());
    std::sort(zv.begin(), zv.end());
    struct P {
        int a, b, c, m;
        float x, y, z;
    };
    std::vector<P> pts;
    for (size_t k = 0; k < reps.size(); ++k) {
        P p;
        p.a = value_index(xv, reps[k][0], tol);
        p.b = value_index(yv, reps[k][1], tol);
        p.c = value_index(zv, reps[k][2], tol);
        p.m = mult[k];
        p.x = reps[k][0];
        p.y = reps[k][1];
        p.z = reps[k][2];
        pts.push_back(p);
    }
    std::sort(pts.begin(), pts.end(), [](const P& u, const P& v) {
        return std::tie(u.a, u.b, u.c) < std::tie(v.a, v.b, v.c);
    });
    rp->xv = xv;
    rp->yv = yv;
    rp->zv = zv;
    rp->grp_xval.clear();
    rp->grp.clear();
    rp->pair_yval.clear();
    rp->pair_pt.clear();
    rp->pt_zval.clear();
    rp->pt_vec.clear();
    rp->pair_rot.clear();
    rp->zero_x = rp->zero_y = -1;
    for (size_t i = 0; i < xv.size(); ++i)
        if (xv[i] == 0.f) rp->zero_x = (int)i;
    for (size_t i = 0; i < yv.size(); ++i)
        if (yv[i] == 0.f) rp->zero_y = (int)i;
    if (rp->zero_x < 0 || rp->zero_y < 0) {
        *err = "ring has no point on the z axis";
        return false;
    }
    int last_a = -1, last_b = -1;
    for (size_t k = 0; k < pts.size(); ++k) {
        const P& p = pts[k];
        if (p.a != last_a) {
            rp->grp_xval.push_back(p.a);
            rp->grp.push_back((int)rp->pair_yval.size());
            last_a = p.a;
            last_b = -1;
        }
        const double ux = (double)p.x / r, uy = (double)p.y / r, uz = (double)p.z / r;
        const double hxy = std::sqrt(ux * ux + uy * uy);
        const double un = std::sqrt(ux * ux + uy * uy + uz * uz);
        if (p.b != last_b) {
            rp->pair_yval.push_back(p.b);
            rp->pair_pt.push_back((int)k);
            last_b = p.b;
            rp->pair_rot.push_back(hxy > 0 ? (float)(ux / hxy) : 1.f);
            rp->pair_rot.push_back(hxy > 0 ? (float)(uy / hxy) : 0.f);
        }
        rp->pt_zval.push_back(p.c);
        rp->pt_vec.push_back((float)(hxy / un));
        rp->pt_vec.push_back((float)(uz / un));
        rp->pt_vec.push_back((float)p.m / (float)n);  // kernel.cu:244 divides by n, not n^2
        rp->pt_vec.push_back((float)(-un));
    }
    rp->grp.push_back((int)rp->pair_yval.size());
    rp->pair_pt.push_back((int)pts.size());
    return true;
}

int ring_zero_pair(const RingPlan& rp) {
    for (size_t g = 0; g + 1 < rp.grp.size(); ++g) {
        if (rp.grp_xval[g] != rp.zero_x) continue;
        for (int p = rp.grp[g]; p < rp.grp[g + 1]; ++p)
            if (rp.pair_yval[p] == rp.zero_y) return p;
    }
    return -1;
}

// ---------------------------------------------------------------------------
// Weight tables

// Catmull-Rom kernel, a = 0.5 (kernel.cu:128-138), evaluated in double.
static double cubic(double xx) {
    const double a = 0.5;
    double x = std::fabs(xx);
    if (x < 1.0) return x * x * (x * (-a + 2.0) + (a - 3.0)) + 1.0;
    if (x < 2.0) return -a * x * x * x + 5.0 * a * x * x - 8.0 * a * x + 4.0 * a;
    return 0.0;
}

// For fine index X = mag*xi + ph and ring offset rho, the sample sits at
// q = xi + f with f = (ph + 0.5 + rho) / mag; the reference's taps are
// u0-1..u0+2 with u0 = floor(q - 0.5) (kernel.cu:149-166). With f in
// [-0.5, 1.5) the taps lie in xi-2..xi+2: 4 of them start at xi-2+off,
// off = floor(f - 0.5) + 1.
static bool tap4(int ph, double rho, int mag, float w[4], int* off) {
    const double f = (ph + 0.5 + rho) / mag;
    if (!(f >= -0.5 && f < 1.5)) return false;
    const int u0 = (int)std::floor(f - 0.5);
    *off = u0 + 1;
    for (int k = 0; k < 4; ++k) w[k] = (float)cubic(f - ((u0 - 1 + k) + 0.5));
    return true;
}
static bool tap5(int ph, double rho, int mag, float w[5]) {
    const double f = (ph + 0.5 + rho) / mag;
    if (!(f >= -0.5 && f < 1.5)) return false;
    for (int m = 0; m < 5; ++m) w[m] = (float)cubic(f - ((m - 2) + 0.5));
    return true;
}

bool build_tables(const rfba_srrf_config& c, const RingPlan& rp, std::vector<float>* words, TableLayout* tl,
                  std::string* err) {
    const int mx = c.mag[0], my = c.mag[1], mz = c.mag[2];
    const int na = (int)rp.xv.size(), nb = (int)rp.yv.size(), nc = (int)rp.zv.size();
    std::vector<float>& W = *words;
    W.clear();
    auto align4 = [&]() {
        while (W.size() % 4) W.push_back(0.f);
    };
    auto push_int = [&](int v) {
        float f;
        std::memcpy(&f, &v, 4);
        W.push_back(f);
    };
    align4();
    tl->wx = (int)W.size();
    std::vector<int> ox(na * mx), oy(nb * my);
    for (int a = 0; a < na; ++a)
        for (int ph = 0; ph < mx; ++ph) {
            float w[4];
            int off;
            if (!tap4(ph, rp.xv[a], mx, w, &off)) {
                *err = "ring radius too large for the x magnification (needs ring_radius < (1 + mag)/2)";
                return false;
            }
            for (int k = 0; k < 4; ++k) W.push_back(w[k]);
            ox[a * mx + ph] = off;
        }
    tl->offx = (int)W.size();
    for (int v : ox) push_int(v);
    align4();
    tl->wy = (int)W.size();
    for (int b = 0; b < nb; ++b)
        for (int ph = 0; ph < my; ++ph) {
            float w[4];
            int off;
            if (!tap4(ph, rp.yv[b], my, w, &off)) {
                *err = "ring radius too large for the y magnification (needs ring_radius < (1 + mag)/2)";
                return false;
            }
            for (int k = 0; k < 4; ++k) W.push_back(w[k]);
            oy[b * my + ph] = off;
        }
    tl->offy = (int)W.size();
    for (int v : oy) push_int(v);
    tl->wz = (int)W.size();
    std::vector<int> oz(nc, 0);
    for (int cc = 0; cc < nc; ++cc)
        for (int ph = 0; ph < mz; ++ph) {
            float w[4];
            int off;
            if (!tap4(ph, rp.zv[cc], mz, w, &off)) {
                *err = "ring radius too large for the z magnification (needs ring_radius < (1 + mag)/2)";
                return false;
            }
            for (int m = 0; m < 4; ++m) W.push_back(w[m]);
            oz[cc] |= off << ph;  // bit ph: taps start one coarse cell later
        }
    tl->offz = (int)W.size();
    for (int v : oz) push_int(v);
    tl->wzi = (int)W.size();
    for (int ph = 0; ph < mz; ++ph) {
        float w[5];
        tap5(ph, 0.0, mz, w);
        for (int m = 0; m < 5; ++m) W.push_back(w[m]);
    }
    tl->grp_xval = (int)W.size();
    for (int v : rp.grp_xval) push_int(v);
    tl->grp = (int)W.size();
    for (int v : rp.grp) push_int(v);
    tl->pair_yval = (int)W.size();
    for (int v : rp.pair_yval) push_int(v);
    tl->pair_pt = (int)W.size();
    for (int v : rp.pair_pt) push_int(v);
    tl->pt_zval = (int)W.size();
    for (int v : rp.pt_zval) push_int(v);
    align4();
    tl->pt_vec = (int)W.size();
    for (float v : rp.pt_vec) W.push_back(v);
    tl->pair_rot = (int)W.size();
    for (float v : rp.pair_rot) W.push_back(v);
    align4();
    tl->words = (int)W.size();
    return true;
}

// ---------------------------------------------------------------------------
// Windows

// The reference's sample window (kernel.cu:143-147 / 260-265) in float.
static inline bool window_ok(float x0f, int mag, int dim) {
    const float q = x0f / (float)mag;
    return !(q < 1.5f || q > (float)dim - 1.5f);
}

// Fine indices X in [0, dim*mag) whose ring samples on this axis all pass the
// window. Float addition and division are monotone, so testing the smallest and
// largest ring coordinate is exact. Returns lo > hi when none passes.
bool window_range(float, const std::vector<float>& rc, int mag, int dim, int* lo, int* hi) {
    float rmin = rc[0], rmax = rc[0];
    for (float v : rc) {
        rmin = std::min(rmin, v);
        rmax = std::max(rmax, v);
    }
    *lo = 1;
    *hi = 0;
    bool any = false;
    for (int X = 0; X < dim * mag; ++X) {
        const float xc = (float)X + 0.5f;
        if (window_ok(xc + rmin, mag, dim) && window_ok(xc + rmax, mag, dim)) {
            if (!any) *lo = X;
            *hi = X;
            any = true;
        }
    }
    return any;
}

// Fine indices whose centre passes the window (interpolateIntensity).
int fine_window_int(int mag, int dim, int* lo, int* hi) {
    *lo = 1;
    *hi = 0;
    bool any = false;
    for (int X = 0; X < dim * mag; ++X)
        if (window_ok((float)X + 0.5f, mag, dim)) {
            if (!any) *lo = X;
            *hi = X;
            any = true;
        }
    return any ? 1 : 0;
}

// ---------------------------------------------------------------------------
// Block lists

// GradientCalc.cpp:47-116 with border 2. Each block computes only the part of
// its interior that the reference's put-back leaves in the output (later
// blocks overwrite the overlap of earlier ones), so every output voxel is
// written once with the value the reference ends up with.
int blocks_gradientcalc(const rfba_srrf_config& c, const int dims[4], rfba_block* out, int cap, std::string* err) {
    const int border = 2;
    // the reference has one magnification; the extended configuration's
    // per-axis factors apply axis by axis (equal factors give the reference's blocks)
    const int* mag = c.mag;
    int split[3];
    for (int a = 0; a < 3; ++a) {
        const int step = c.block_size[a] - 2 * border;
        if (step <= 0) {
            *err = "block size must exceed 4 (GradientCalc border 2 on both sides)";
            return RFBA_ERR_INVALID;
        }
        const int num = dims[a] - 2 * border;
        split[a] = num / step;  // C truncation, as the reference
        if (num % step != 0) split[a] += 1;
        if (split[a] < 0) split[a] = 0;
    }
    const long long W = (long long)dims[0] * mag[0], H = (long long)dims[1] * mag[1];
    int count = 0;
    for (int k = 0; k < split[2]; ++k)
        for (int j = 0; j < split[1]; ++j)
            for (int i = 0; i < split[0]; ++i) {
                const int pos[3] = {i, j, k};
                rfba_block b;
                std::memset(&b, 0, sizeof b);
                bool empty = false;
                for (int a = 0; a < 3; ++a) {
                    const int step = c.block_size[a] - 2 * border;
                    const bool last = pos[a] == split[a] - 1;
                    const int res = last ? dims[a] - (split[a] - 1) * step : c.block_size[a];
                    const int start = pos[a] == 0 ? 0 : pos[a] * step;
                    b.origin[a] = start;
                    b.size[a] = res;
                    b.lo[a] = border * mag[a];
                    b.hi[a] = last ? res * mag[a] : (step + border) * mag[a];
                    if (b.hi[a] > res * mag[a]) b.hi[a] = res * mag[a];
                    if (b.hi[a] <= b.lo[a]) empty = true;
                }
                if (empty) continue;
                b.out_stride[0] = 1;
                b.out_stride[1] = W;
                b.out_stride[2] = W * H;
                b.out_offset = ((long long)b.origin[2] * mag[2] + b.lo[2]) * W * H +
                               ((long long)b.origin[1] * mag[1] + b.lo[1]) * W +
                               ((long long)b.origin[0] * mag[0] + b.lo[0]);
                if (out && count < cap) out[count] = b;
                ++count;
            }
    return count;
}

// Matlab Scripts/doSplit.m:1-19 (1-based positions turned 0-based).
static std::vector<std::pair<int, int>> dosplit_axis(int xall, int maxX, int border) {
    std::vector<std::pair<int, int>> pos;  // (start, size), 1-based start
    if (maxX >= xall) {
        pos.push_back({1, xall});
        return pos;
    }
    pos.push_back({1, maxX});
    while (pos.back().first + maxX <= xall) {
        const int nxt = pos.back().first + pos.back().second - 2 * border;
        pos.push_back({nxt, maxX});
    }
    pos.back().second = xall - pos.back().first + 1;
    return pos;
}

int blocks_dosplit(const rfba_srrf_config& c, const int dims[4], const int max_size[3], int border, rfba_block* out,
                   int cap, long long* out_elems, std::string* err) {
    if (border < 0 || max_size[0] <= 2 * border || max_size[1] <= 2 * border || max_size[2] <= 2 * border) {
        *err = "doSplit needs max size > 2*border";
        return RFBA_ERR_INVALID;
    }
    auto xs = dosplit_axis(dims[0], max_size[0], border);
    auto ys = dosplit_axis(dims[1], max_size[1], border);
    auto zs = dosplit_axis(dims[2], max_size[2], border);
    int count = 0;
    long long off = 0;
    // GenerateBlock.m:118-120 loop order: x outermost, z innermost.
    for (auto& px : xs)
        for (auto& py : ys)
            for (auto& pz : zs) {
                rfba_block b;
                std::memset(&b, 0, sizeof b);
                b.origin[0] = px.first - 1;
                b.origin[1] = py.first - 1;
                b.origin[2] = pz.first - 1;
                b.size[0] = px.second;
                b.size[1] = py.second;
                b.size[2] = pz.second;
                for (int a = 0; a < 3; ++a) {
                    b.lo[a] = 0;
                    b.hi[a] = b.size[a] * c.mag[a];
                }
                b.out_offset = off;
                b.out_stride[0] = 1;
                b.out_stride[1] = b.hi[0];
                b.out_stride[2] = (long long)b.hi[0] * b.hi[1];
                off += (long long)b.hi[0] * b.hi[1] * b.hi[2];
                if (out && count < cap) out[count] = b;
                ++count;
            }
    if (out_elems) *out_elems = off;
    return count;
}

}  // namespace rfba

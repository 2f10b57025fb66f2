// mtg_host.cpp -- host-side seeded synthetic inputs for the C ABI (no GPU use).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <cstdint>
#include <climits>
#include <vector>
#include <algorithm>

#include "../../include/mtcode_gb300.h"

namespace {

// splitmix64 (Steele, Lea, Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014)
struct SplitMix {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
};

}  // namespace

extern "C" {

// Random sequential addition with a cell hash: each candidate is tested against the accepted
// particles of the 27 surrounding cells (side >= min_dist).
mtg_status mtg_random_positions(int n, double box, int periodic, double min_dist, uint64_t seed, double *x) {
    if (n < 0 || box <= 0 || min_dist < 0 || !x) return MTG_ERR_ARG;
    SplitMix rng{seed ^ 0x5DEECE66Dull};
    int nc = min_dist > 0 ? (int)std::floor(box / min_dist) : 1;
    if (nc < 1) nc = 1;
    if (nc > 512) nc = 512;
    const double scale = nc / box;
    std::vector<int> head((size_t)nc * nc * nc, -1), next((size_t)n, -1);
    const double md2 = min_dist * min_dist;
    int placed = 0;
    int64_t attempts = 0, limit = 1000LL * (int64_t)(n > 0 ? n : 1);
    while (placed < n) {
        if (++attempts > limit) return MTG_ERR_ARG;
        double c[3] = {rng.uniform() * box, rng.uniform() * box, rng.uniform() * box};
        int ci[3];
        for (int k = 0; k < 3; k++) {
            ci[k] = (int)(c[k] * scale);
            if (ci[k] >= nc) ci[k] = nc - 1;
        }
        bool ok = true;
        const int lo = nc >= 3 ? -1 : 0, hi = nc >= 2 ? 1 : 0;
        for (int dz = lo; dz <= hi && ok; dz++)
            for (int dy = lo; dy <= hi && ok; dy++)
                for (int dx = lo; dx <= hi && ok; dx++) {
                    int a = ci[0] + dx, b = ci[1] + dy, e = ci[2] + dz;
                    if (!periodic && (a < 0 || a >= nc || b < 0 || b >= nc || e < 0 || e >= nc)) continue;
                    a = (a + nc) % nc; b = (b + nc) % nc; e = (e + nc) % nc;
                    for (int j = head[(size_t)a + nc * ((size_t)b + (size_t)nc * e)]; j >= 0; j = next[j]) {
                        double d2 = 0;
                        for (int k = 0; k < 3; k++) {
                            double d = c[k] - x[3 * (size_t)j + k];
                            if (periodic) d -= box * std::nearbyint(d / box);
                            d2 += d * d;
                        }
                        if (d2 < md2) { ok = false; break; }
                    }
                }
        if (!ok) continue;
        for (int k = 0; k < 3; k++) x[3 * (size_t)placed + k] = c[k];
        size_t cell = (size_t)ci[0] + nc * ((size_t)ci[1] + (size_t)nc * ci[2]);
        next[placed] = head[cell];
        head[cell] = placed;
        placed++;
    }
    return MTG_OK;
}

// Self-avoiding random-walk chains: chain c's bead b goes to row c * beads + b.  The first bead of a chain
// is uniform in the box; each next one is `step` away from its predecessor along a direction drawn
// uniformly on the sphere (rejection from the cube, no trig, so the same bits on every host).  Every
// bead keeps min_dist from all earlier beads (minimum image); walls reject, periodic faces wrap.  A
// chain that gets stuck is removed and restarted.
mtg_status mtg_random_chains(int n_chains, int beads, double box, int periodic, double step, double min_dist,
                             uint64_t seed, double *x) {
    if (n_chains < 0 || beads < 1 || box <= 0 || step <= 0 || min_dist < 0 || min_dist >= step || !x)
        return MTG_ERR_ARG;
    const int64_t n = (int64_t)n_chains * beads;
    if (n > INT32_MAX) return MTG_ERR_ARG;
    SplitMix rng{seed ^ 0x2545F4914F6CDD1Dull};
    int nc = min_dist > 0 ? (int)std::floor(box / min_dist) : 1;
    if (nc < 1) nc = 1;
    if (nc > 1024) nc = 1024;
    const double scale = nc / box;
    std::vector<int> head((size_t)nc * nc * nc, -1), next((size_t)(n > 0 ? n : 1), -1), cell_of((size_t)(n > 0 ? n : 1));
    const double md2 = min_dist * min_dist;
    auto cell_index = [&](const double c[3]) {
        int ci[3];
        for (int k = 0; k < 3; k++) {
            ci[k] = (int)(c[k] * scale);
            if (ci[k] >= nc) ci[k] = nc - 1;
            if (ci[k] < 0) ci[k] = 0;
        }
        return ci[0] + nc * (ci[1] + nc * ci[2]);
    };
    auto is_free = [&](const double c[3]) {
        const int cc = cell_index(c);
        const int ci[3] = {cc % nc, (cc / nc) % nc, cc / (nc * nc)};
        const int lo = nc >= 3 ? -1 : 0, hi = nc >= 2 ? 1 : 0;
        for (int dz = lo; dz <= hi; dz++)
            for (int dy = lo; dy <= hi; dy++)
                for (int dx = lo; dx <= hi; dx++) {
                    int a = ci[0] + dx, b = ci[1] + dy, e = ci[2] + dz;
                    if (!periodic && (a < 0 || a >= nc || b < 0 || b >= nc || e < 0 || e >= nc)) continue;
                    a = (a + nc) % nc; b = (b + nc) % nc; e = (e + nc) % nc;
                    for (int j = head[(size_t)a + nc * ((size_t)b + (size_t)nc * e)]; j >= 0; j = next[j]) {
                        double d2 = 0;
                        for (int k = 0; k < 3; k++) {
                            double d = c[k] - x[3 * (size_t)j + k];
                            if (periodic) d -= box * std::nearbyint(d / box);
                            d2 += d * d;
                        }
                        if (d2 < md2) return false;
                    }
                }
        return true;
    };
    auto place = [&](int i, const double c[3]) {
        for (int k = 0; k < 3; k++) x[3 * (size_t)i + k] = c[k];
        const int cc = cell_index(c);
        cell_of[i] = cc;
        next[i] = head[cc];
        head[cc] = i;
    };
    for (int ch = 0; ch < n_chains; ch++) {
        const int i0 = ch * beads;
        bool done = false;
        for (int restart = 0; restart < 1000 && !done; restart++) {
            int placed = 0;
            for (int tries = 0; tries < 10000 && placed == 0; tries++) {
                double c[3] = {rng.uniform() * box, rng.uniform() * box, rng.uniform() * box};
                if (is_free(c)) { place(i0, c); placed = 1; }
            }
            if (!placed) return MTG_ERR_ARG;
            while (placed < beads) {
                bool ok = false;
                for (int tries = 0; tries < 200 && !ok; tries++) {
                    double v[3], r2 = 0;
                    do {
                        r2 = 0;
                        for (int k = 0; k < 3; k++) { v[k] = 2.0 * rng.uniform() - 1.0; r2 += v[k] * v[k]; }
                    } while (r2 > 1.0 || r2 < 1e-6);
                    const double inv = step / std::sqrt(r2);
                    double c[3];
                    bool inside = true;
                    for (int k = 0; k < 3; k++) {
                        c[k] = x[3 * (size_t)(i0 + placed - 1) + k] + v[k] * inv;
                        if (periodic) {
                            if (c[k] < 0) c[k] += box;
                            else if (c[k] >= box) c[k] -= box;
                        } else if (c[k] < 0 || c[k] >= box) {
                            inside = false;
                        }
                    }
                    if (inside && is_free(c)) { place(i0 + placed, c); ok = true; }
                }
                if (!ok) break;
                placed++;
            }
            if (placed == beads) {
                done = true;
            } else {
                // stuck: unlink this chain's beads (the most recent insertions head their cells)
                for (int i = i0 + placed - 1; i >= i0; i--) head[cell_of[i]] = next[i];
            }
        }
        if (!done) return MTG_ERR_ARG;
    }
    return MTG_OK;
}

// Frame files in the reference's format: one row per line, values separated by ',', each value as
// std::ostream prints a double by default (six significant digits, %g), i.e. matrix::operator<<=
// (DataStructures/matrix2.cpp:898-912) as Condensate::run writes pos / orientation frames
// (Condensate/Condensate.cpp:378-418).
mtg_status mtg_csv_write(const char *path, const double *a, int64_t rows, int cols) {
    if (!path || (rows > 0 && !a) || rows < 0 || cols < 1) return MTG_ERR_ARG;
    FILE *f = std::fopen(path, "w");
    if (!f) return MTG_ERR_ARG;
    char buf[64];
    for (int64_t i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++) {
            int n = std::snprintf(buf, sizeof(buf), "%g", a[(size_t)i * cols + j]);
            buf[n++] = j == cols - 1 ? '\n' : ',';
            if (std::fwrite(buf, 1, (size_t)n, f) != (size_t)n) {
                std::fclose(f);
                return MTG_ERR_ARG;
            }
        }
    return std::fclose(f) == 0 ? MTG_OK : MTG_ERR_ARG;
}

// importcsv (DataStructures/matrix2.cpp:1597-1640): every line is a row, cells split at ',' and read
// with atof; the column count is the longest row's and shorter rows are padded with 0.  With a null
// `a` (or too small a capacity) only the shape is returned, and MTG_ERR_CAPACITY when it does not fit.
mtg_status mtg_csv_read(const char *path, double *a, int64_t cap, int64_t *rows, int *cols) {
    if (!path || !rows || !cols) return MTG_ERR_ARG;
    FILE *f = std::fopen(path, "r");
    if (!f) return MTG_ERR_ARG;
    std::vector<std::vector<double>> data;
    std::string line;
    int c;
    bool more = true;
    while (more) {
        line.clear();
        while ((c = std::fgetc(f)) != EOF && c != '\n') line.push_back((char)c);
        if (c == EOF) {
            more = false;
            if (line.empty()) break;  // getline yields no line after a final newline
        }
        std::vector<double> row;
        size_t start = 0;
        while (start < line.size()) {  // getline(cell, ','): no empty cell after a trailing ','
            size_t end = line.find(',', start);
            if (end == std::string::npos) end = line.size();
            row.push_back(std::atof(line.substr(start, end - start).c_str()));
            start = end + 1;
        }
        data.push_back(std::move(row));
    }
    std::fclose(f);
    int nz = 0;
    for (auto &r : data) nz = std::max(nz, (int)r.size());
    *rows = (int64_t)data.size();
    *cols = nz;
    if (!a || cap < (int64_t)data.size() * nz) return a ? MTG_ERR_CAPACITY : MTG_OK;
    for (size_t i = 0; i < data.size(); i++)
        for (int j = 0; j < nz; j++) a[i * nz + j] = j < (int)data[i].size() ? data[i][j] : 0.0;
    return MTG_OK;
}

// Condensate::run's frame file name: kind + strbase + "_i=" + the frame number zero-padded to the
// digits of ceil(runtime / every) + ".csv" (Condensate.cpp:296-300, 383-405).  Returns the length.
int mtg_frame_name(char *out, int cap, const char *kind, const char *strbase, int frame, int runtime, int every) {
    if (!kind || every < 1 || runtime < 0 || frame < 0) return -1;
    int tf = (int)std::ceil((double)runtime / (double)every), digits = 0;
    do {
        ++digits;
        tf /= 10;
    } while (tf);
    return std::snprintf(out, out ? (size_t)cap : 0, "%s%s_i=%0*d.csv", kind, strbase ? strbase : "", digits, frame);
}

// BindingModelSingle(on_rate, off_rate) (Bindings/BindingModelSingle.cpp) in table form: a doublet goes to
// unbound with weight off_rate and to bound with on_rate, whatever it was before; a triplet bound on one edge
// keeps it with on_rate and moves to each other state with off_rate / 3 + 0.001, an unbound triplet binds each
// edge with on_rate / 3 and stays unbound with off_rate.
void mtg_binding_single(mtg_binding_model *m, double on_rate, double off_rate) {
    if (!m) return;
    std::memset(m, 0, sizeof(*m));
    m->species_rule = 0;
    m->np = 1;
    m->drate[0][0] = off_rate;
    m->drate[0][1] = on_rate;
    m->drate[0][2] = off_rate;
    m->drate[0][3] = on_rate;
    const double x = (off_rate / 3.) + 0.001;
    double *t = m->trate[0];
    for (int st = 0; st < 3; st++)
        for (int k = 0; k < 4; k++) t[4 * st + k] = k == st ? on_rate : x;
    t[12] = on_rate / 3.;
    t[13] = on_rate / 3.;
    t[14] = on_rate / 3.;
    t[15] = off_rate;
}

// BindingModelBinary(div) + setup_equilibrium() (Bindings/BindingModelBinary.cpp): every species pair binds
// a doublet for certain; every species triple uses the same triplet table, and the 122 / 222 triplets take
// their rate to none-bound from the 111 table, as the reference's triplet does.
void mtg_binding_binary_equilibrium(mtg_binding_model *m, int div) {
    if (!m) return;
    std::memset(m, 0, sizeof(*m));
    m->species_rule = 1;
    m->div1 = div;
    m->np = 1;
    static const double r2[4] = {0.0, 1.0, 0.0, 1.0};
    static const double t3[16] = {0.998, 0.001, 0.001, 0.000, 0.001, 0.998, 0.001, 0.000,
                                  0.001, 0.001, 0.998, 0.000, 0.33, 0.33, 0.33, 0.01};
    const int pair_rows[3] = {0, 1, 3};        // 11, 12, 22
    const int triple_rows[4] = {0, 1, 3, 6};   // 111, 112, 122, 222
    for (int r : pair_rows) std::memcpy(m->drate[r], r2, sizeof(r2));
    for (int r : triple_rows) std::memcpy(m->trate[r], t3, sizeof(t3));
    for (int r : {3, 6})
        for (int st = 0; st < 4; st++) m->trate[r][4 * st + 3] = m->trate[0][4 * st + 3];
}

void mtg_single_bond_defaults(mtg_single_bond *sb) {
    if (!sb) return;
    std::memset(sb, 0, sizeof(*sb));
    mtg_binding_single(&sb->model, 1.0, 0.0);
    sb->max_ang = std::nan("");
    sb->list_cut = 2.5;
    sb->patch_every = 10;
}

// Arvo, "Fast random rotation matrices" (Graphics Gems III, 1992): M = (2 v v^T - I) Rz(2 pi x1),
// v = (cos(2 pi x2) sqrt(x3), sin(2 pi x2) sqrt(x3), sqrt(1 - x3)) -- the construction of
// LangevinNVTR::initialize (LangevinR.cpp:239-267), driven by splitmix64 instead of rand().
void mtg_random_rotations(int n, uint64_t seed, double *Q) {
    SplitMix rng{seed ^ 0xA0761D6478BD642Full};
    const double two_pi = 6.283185307179586476925286766559;
    for (int i = 0; i < n; i++) {
        double x1 = rng.uniform(), x2 = rng.uniform(), x3 = rng.uniform();
        double v[3] = {std::cos(two_pi * x2) * std::sqrt(x3), std::sin(two_pi * x2) * std::sqrt(x3), std::sqrt(1. - x3)};
        double c = std::cos(two_pi * x1), s = std::sin(two_pi * x1);
        double Rz[3][3] = {{c, s, 0}, {-s, c, 0}, {0, 0, 1}};
        double *q = Q + 9 * (size_t)i;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                double acc = 0;
                for (int k = 0; k < 3; k++) acc += (2 * v[a] * v[k] - (a == k ? 1.0 : 0.0)) * Rz[k][b];
                q[3 * a + b] = acc;
            }
    }
}

}  // extern "C"

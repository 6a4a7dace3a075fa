// C entry points of the oracle restatement, for tests and the CPU-baseline leg of bench.py.
// Test infrastructure only: the product never links this library.
#include "oracle.hpp"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

using namespace orc;

namespace {
struct Ctx {
    Params par;
    Snapshot snap;
    Finder finder;
    std::string summary;
    double t_read = 0, t_tree = 0, t_find = 0;
    uint32_t n_input = 0;
    bool no_ghost = false;
    bool dvs = false;  // --Density_Vs_Scale settings for the tree
};
double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
}  // namespace

extern "C" {

void *orc_open(const char *param_path, int threads, int pow_mode, int no_ghost) {
    Ctx *c = new Ctx();
    if (param_path && *param_path) {
        if (read_param_file(param_path, c->par) != 0) { delete c; return nullptr; }
    }
    c->finder.par = &c->par;
    c->finder.threads = threads > 0 ? threads : (int)(c->par.num_threads ? c->par.num_threads : 1);
    c->finder.pow_mode = pow_mode ? POW_CORRECT : POW_LIBM;
    c->no_ghost = no_ghost != 0;
    return c;
}

void orc_close(void *h) { delete static_cast<Ctx *>(h); }

// --Density_Vs_Scale for the next orc_load: the tree as that analysis builds it (64-point
// leaves, no ghosts, ghost zone as wide as the box; src/analyses.hpp:29-33)
void orc_set_density_vs_scale(void *h) { static_cast<Ctx *>(h)->dvs = true; }

// BasicAnalysesWithTree on the loaded tree: radii and densities; returns the number of radii
int orc_density_vs_scale(void *h, double *radii, double *rho, int cap) {
    Ctx *c = static_cast<Ctx *>(h);
    DensityVsScale dv = density_vs_scale(c->finder.tree, c->par, c->snap.time);
    for (int i = 0; i < (int)dv.radii.size() && i < cap; ++i) {
        radii[i] = dv.radii[i];
        rho[i] = dv.max_rhop[i];
    }
    return (int)dv.radii.size();
}

// The parameters the analysis reads: box_length[3], box_min[3], box_max[3], box_center[3],
// box_half_width[0], max_half_width, cell_length[3], shear_speed, mass_per_particle[0], time
void orc_density_vs_scale_params(void *h, double *out19) {
    Ctx *c = static_cast<Ctx *>(h);
    const Params &p = c->par;
    for (int d = 0; d < 3; ++d) {
        out19[d] = p.box_length[d];
        out19[3 + d] = p.box_min[d];
        out19[6 + d] = p.box_max[d];
        out19[9 + d] = p.box_center[d];
        out19[14 + d] = p.cell_length[d];
    }
    out19[12] = p.box_half_width[0];
    out19[13] = p.max_half_width;
    out19[17] = p.shear_speed;
    out19[18] = p.mass_per_particle.empty() ? 0.0 : p.mass_per_particle[0];
}

// -x/-y/-z user box for the next orc_load (lo <= hi per axis; 0,0 = the box's extent)
void orc_set_user_box(void *h, const double *lo3, const double *hi3) {
    Ctx *c = static_cast<Ctx *>(h);
    c->par.user_box = true;
    for (int d = 0; d < 3; ++d) {
        c->par.user_box_min[d] = lo3[d];
        c->par.user_box_max[d] = hi3[d];
    }
}

// Read one combined .lis file (first file of a run), make ghosts and build the tree.
// lis_paths: one path, or the files of one snapshot separated by newlines (id0 first)
int orc_load(void *h, const char *lis_paths) {
    Ctx *c = static_cast<Ctx *>(h);
    double t0 = now();
    std::vector<std::string> files;
    std::string all(lis_paths);
    for (size_t b = 0; b <= all.size();) {
        size_t e = all.find('\n', b);
        if (e == std::string::npos) e = all.size();
        if (e > b) files.push_back(all.substr(b, e - b));
        b = e + 1;
    }
    if (files.empty()) return 3;
    int rc = read_lis_files(files, c->snap);
    if (rc) return rc;
    finish_read(c->snap, c->par, true);
    if (c->snap.num_particles == 0) return 7;  // the reference has no check and crashes in BuildTree
    if (c->dvs) {
        c->par.max_ghost_zone_width = c->par.max_half_width;
        c->no_ghost = true;
        c->finder.tree.max_leaf_size = 64;
    }
    c->n_input = c->snap.num_particles;
    double t1 = now();
    if (!c->no_ghost) make_ghosts(c->snap, c->par);
    c->finder.time = c->snap.time;
    c->finder.tree.build(c->par, c->snap.parts, true);
    double t2 = now();
    c->t_read = t1 - t0;
    c->t_tree = t2 - t1;
    return 0;
}

int orc_find(void *h) {
    Ctx *c = static_cast<Ctx *>(h);
    double t0 = now();
    try {
        c->summary = c->finder.find(c->n_input);
    } catch (const std::domain_error &e) {
        c->summary = e.what();
        return -7;
    }
    c->t_find = now() - t0;
    return (int)c->finder.num_planetesimals;
}

void orc_timings(void *h, double *out3) {
    Ctx *c = static_cast<Ctx *>(h);
    out3[0] = c->t_read; out3[1] = c->t_tree; out3[2] = c->t_find;
}

const char *orc_summary(void *h) { return static_cast<Ctx *>(h)->summary.c_str(); }
uint32_t orc_num_points(void *h) { return static_cast<Ctx *>(h)->finder.tree.size(); }
uint32_t orc_num_nodes(void *h) { return (uint32_t)static_cast<Ctx *>(h)->finder.tree.nodes.size(); }
uint32_t orc_num_input(void *h) { return static_cast<Ctx *>(h)->n_input; }

// Sorted tree points: pos[3], vel[3], mass, ath_density, new_density (9 doubles per point),
// original ids and sink flags.
void orc_points(void *h, double *out9, uint32_t *orig, uint8_t *sink) {
    auto &t = static_cast<Ctx *>(h)->finder.tree;
    for (uint32_t i = 0; i < t.size(); ++i) {
        const TreePoint &p = t.pts[i];
        double *o = out9 + 9 * (size_t)i;
        for (int d = 0; d < 3; ++d) { o[d] = p.pos[d]; o[3 + d] = p.vel[d]; }
        o[6] = p.mass; o[7] = p.ath_density; o[8] = p.new_density;
        if (orig) orig[i] = p.original_id;
        if (sink) sink[i] = p.sink_flag ? 1 : 0;
    }
}

void orc_keys(void *h, uint32_t *out3) {
    auto &t = static_cast<Ctx *>(h)->finder.tree;
    for (uint32_t i = 0; i < t.size(); ++i) {
        Key k = t.morton(t.pts[i].pos, 0);
        out3[3 * (size_t)i] = (uint32_t)k;
        out3[3 * (size_t)i + 1] = (uint32_t)(k >> 32);
        out3[3 * (size_t)i + 2] = (uint32_t)(k >> 64);
    }
}

// Nodes: center[3], half_width (4 doubles) and begin, end, parent, first_daughter,
// orthant, num_daughters, level (7 u32) per node.
void orc_nodes(void *h, double *f4, uint32_t *u7) {
    auto &t = static_cast<Ctx *>(h)->finder.tree;
    for (size_t i = 0; i < t.nodes.size(); ++i) {
        const Node &n = t.nodes[i];
        for (int d = 0; d < 3; ++d) f4[4 * i + d] = n.center[d];
        f4[4 * i + 3] = n.half_width;
        uint32_t *u = u7 + 7 * i;
        u[0] = n.begin; u[1] = n.end; u[2] = n.parent; u[3] = n.first_daughter;
        u[4] = n.orthant; u[5] = n.num_daughters; u[6] = n.level;
    }
}

void orc_tree_box(void *h, double *out5) {
    auto &t = static_cast<Ctx *>(h)->finder.tree;
    for (int d = 0; d < 3; ++d) out5[d] = t.root_center[d];
    out5[3] = t.half_width;
    out5[4] = t.epsilon;
}

// KNN of an arbitrary position (est = 0 uses the reference's own first radius).
// Returns 0, or 7 when the position has no leaf in the tree (the reference's Key2Leaf
// failure; its KNN is undefined there).
int orc_knn(void *h, const double *pos, unsigned k, double est, uint32_t *idx, double *dr2) {
    auto &t = static_cast<Ctx *>(h)->finder.tree;
    Heap hp;
    if (!t.knn(V3(pos[0], pos[1], pos[2]), k, hp, est)) return 7;
    for (unsigned j = 0; j < k; ++j) { idx[j] = (uint32_t)hp[j].first; dr2[j] = hp[j].second; }
    return 0;
}

void orc_densest(void *h, uint32_t *out) {
    auto &f = static_cast<Ctx *>(h)->finder;
    std::memcpy(out, f.densest.data(), 4 * f.densest.size());
}

void orc_peaks(void *h, uint32_t *out) {
    auto &f = static_cast<Ctx *>(h)->finder;
    std::memcpy(out, f.peak_of.data(), 4 * f.peak_of.size());
}

void orc_thresholds(void *h, double *out4) {
    auto &f = static_cast<Ctx *>(h)->finder;
    out4[0] = f.density_threshold; out4[1] = f.peak_density_threshold;
    out4[2] = f.clump_mass_threshold; out4[3] = f.median_kernel ? 1.0 : 0.0;
}

void orc_stats(void *h, uint64_t *out8) {
    auto &s = static_cast<Ctx *>(h)->finder.stats;
    out8[0] = s.naive_peaks; out8[1] = s.after_merge_a; out8[2] = s.after_merge_b; out8[3] = s.final_clumps;
    out8[4] = s.sweeps_a; out8[5] = s.sweeps_b; out8[6] = s.zero_key_quirk;
    out8[7] = static_cast<Ctx *>(h)->finder.tree.check_outside;
}

// Final clumps in key order: peak, n; M, Hill, com[3], vcom[3], J[3] (11 doubles);
// members (tree indices, `indices` order) concatenated into `members` when non-null.
uint32_t orc_num_clumps(void *h) { return (uint32_t)static_cast<Ctx *>(h)->finder.clumps.size(); }
uint64_t orc_clumps(void *h, uint32_t *peak_n, double *f11, uint32_t *members) {
    auto &f = static_cast<Ctx *>(h)->finder;
    size_t k = 0;
    uint64_t m = 0;
    for (auto &it : f.clumps) {
        const Clump &c = it.second;
        if (peak_n) { peak_n[2 * k] = it.first; peak_n[2 * k + 1] = (uint32_t)c.indices.size(); }
        if (f11) {
            double *o = f11 + 11 * k;
            o[0] = c.total_mass; o[1] = c.Hill_radius;
            for (int d = 0; d < 3; ++d) { o[2 + d] = c.center_of_mass[d]; o[5 + d] = c.vel_com[d]; o[8 + d] = c.J[d]; }
        }
        if (members) for (uint32_t i : c.indices) members[m++] = i;
        else m += c.indices.size();
        ++k;
    }
    return m;
}

// Write peaks_at_<time>.txt next to out_path and append the basic-results line(s) to
// <stem>_planetesimals.txt (header first when `first` is non-zero).
int orc_write_outputs(void *h, const char *out_path, int first) {
    Ctx *c = static_cast<Ctx *>(h);
    std::string op(out_path);
    write_peaks_file(peaks_file_name(op, c->snap.time), c->finder);
    std::string stem = op.substr(0, op.find_last_of('.')) + "_planetesimals.txt";
    FILE *f = std::fopen(stem.c_str(), first ? "w" : "a");
    if (!f) return 3;
    std::string s = (first ? basic_results_header() : std::string()) + basic_results_line(c->finder, c->par, c->snap.time);
    std::fwrite(s.data(), 1, s.size(), f);
    std::fclose(f);
    return 0;
}

// The order std::sort with the reference's comparator (low 96 bits only,
// src/tree.hpp:2269-2273, 2831) gives keys in input order: order[i] = input index of the
// i-th sorted key.
void orc_morton_order(const uint32_t *keys3, uint32_t n, uint32_t *order) {
    typedef unsigned __int128 u128;
    std::vector<u128> m(n);
    for (uint32_t i = 0; i < n; ++i)
        m[i] = ((u128)i << 96) | ((u128)keys3[3 * (size_t)i + 2] << 64) | ((u128)keys3[3 * (size_t)i + 1] << 32) | keys3[3 * (size_t)i];
    std::sort(m.begin(), m.end(), [](u128 x, u128 y) { return (x << 32) < (y << 32); });
    for (uint32_t i = 0; i < n; ++i) order[i] = (uint32_t)(m[i] >> 96);
}

}  // extern "C"

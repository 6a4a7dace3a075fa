// CPU restatement of PLAN's clump-finding path; see oracle.hpp for scope and rules.
#include "oracle.hpp"

#include <algorithm>
#include <chrono>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <limits>
#include <numeric>
#include <sstream>
#include <stdexcept>
#include <sys/stat.h>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

double norm(const V3 &a) { return std::sqrt(norm2(a)); }

// ================================================================ parameters
void Params::derive() {  // src/global.cpp:28-47
    for (int d = 0; d < 3; ++d) box_half_width[d] = box_length[d] / 2.0;
    max_half_width = 0.0;
    for (int d = 0; d < 3; ++d) {
        max_half_width = std::max(max_half_width, box_half_width[d]);
        max_ghost_zone_width = std::max(max_ghost_zone_width, ghost_zone_width[d]);
    }
    for (int d = 0; d < 3; ++d) cell_length[d] = box_length[d] / box_resolution[d];
    cell_volume = 1.0;
    for (int d = 0; d < 3; ++d) cell_volume = cell_volume * cell_length[d];
    mass_total_code_units = std::sqrt(2 * PI) * box_length[0] * box_length[1] * solid_to_gas_ratio;
    G_tilde = four_PI_G / Omega / Omega;
    mass_physical = (G_tilde / 0.1) * 1.3e24;
    grav_constant = four_PI_G / four_PI;
    shear_speed = q * Omega * box_length[0];
    min_trusted_mass = 3 * std::pow(cell_length[0], 3) * Omega * Omega / rho_g0 / grav_constant;
}

static void trim(std::string &s) {
    size_t b = 0, e = s.size();
    while (b < e && std::isspace((unsigned char)s[b])) ++b;
    while (e > b && std::isspace((unsigned char)s[e - 1])) --e;
    s = s.substr(b, e - b);
}

int read_param_file(const std::string &path, Params &p) {  // src/global.cpp:51-225
    std::ifstream in(path);
    if (!in.is_open()) {
        std::fprintf(stderr, "Error: Failed to open file %s\n", path.c_str());
        return 3;
    }
    std::unordered_map<std::string, double> kv;
    std::string line;
    while (in && std::getline(in, line)) {
        if (line.empty() || line[0] == '#' || line[0] == '<') continue;
        line = line.substr(0, line.find_first_of('#'));
        size_t eq = line.find_first_of('=');
        std::string name = line.substr(0, eq), value = line.substr(eq + 1);
        trim(name);
        trim(value);
        if (value.find('/') != std::string::npos) {
            std::istringstream iss(value);
            double v1, v2;
            char c;
            iss >> v1 >> c >> v2;
            kv.emplace(name, v1 / v2);
        } else {
            try {
                kv.emplace(name, std::stod(value));
            } catch (...) {
                std::fprintf(stderr, "Error: cannot parse value of %s\n", name.c_str());
                return 4;
            }
        }
    }
    auto get = [&](const char *k, double &v) {
        auto it = kv.find(k);
        if (it == kv.end()) return false;
        v = it->second;
        return true;
    };
    double v;
    if (get("Z", v)) p.solid_to_gas_ratio = v;
    if (get("Nx1", v)) p.box_resolution[0] = (unsigned)v;
    if (get("Nx2", v)) p.box_resolution[1] = (unsigned)v;
    if (get("Nx3", v)) p.box_resolution[2] = (unsigned)v;
    if (get("four_pi_G_par", v)) p.four_PI_G = v;
    if (get("omp_threads", v)) p.num_threads = (unsigned)v;
    if (get("num_threads", v)) p.num_threads = (unsigned)v;
    if (get("num_peaks", v)) p.num_peaks = (unsigned)v;
    if (get("num_peak", v)) p.num_peaks = (unsigned)v;
    if (get("num_neighbors_in_knn_search", v)) p.knn = (unsigned)v;
    if (get("num_knn", v)) p.knn = (unsigned)v;
    if (get("knn", v)) p.knn = (unsigned)v;
    if (get("num_neighbors_to_hop", v)) { p.hop = (unsigned)v; p.fixed_hop = true; }
    if (get("num_hop", v)) { p.hop = (unsigned)v; p.fixed_hop = true; }
    if (get("hop", v)) { p.hop = (unsigned)v; p.fixed_hop = true; }
    if (get("clump_diffuse_threshold", v)) {
        p.clump_diffuse_threshold = v;
        if (v < 0) return 4;
    }
    if (get("Hill_fraction_for_merge", v)) {
        p.Hill_fraction_for_merge = v;
        if (v < 0) return 4;
    }
    p.derive();
    return 0;
}

// ================================================================ particle input
static bool read_header(std::ifstream &f, Snapshot &s, long &n) {
    float lim[12], fv;
    f.read(reinterpret_cast<char *>(lim), sizeof(lim));
    for (int i = 0; i < 12; ++i) s.coor_lim[i] = (double)lim[i];
    unsigned ntypes = 0;
    f.read(reinterpret_cast<char *>(&ntypes), 4);
    s.type_info.resize(ntypes);
    for (unsigned i = 0; i < ntypes; ++i) {
        f.read(reinterpret_cast<char *>(&fv), 4);
        s.type_info[i] = (double)fv;
    }
    f.read(reinterpret_cast<char *>(&fv), 4);
    s.time = (double)fv;
    f.read(reinterpret_cast<char *>(&fv), 4);
    s.dt = (double)fv;
    f.read(reinterpret_cast<char *>(&n), 8);
    return (bool)f;
}

static void unpack(const char *c, Particle &p) {  // one 44-byte record, src/tree.hpp:1488-1511
    float fv[3], dens;
    std::memcpy(fv, c, 12);
    for (int d = 0; d < 3; ++d) p.pos[d] = (double)fv[d];
    std::memcpy(fv, c + 12, 12);
    for (int d = 0; d < 3; ++d) p.vel[d] = (double)fv[d];
    std::memcpy(&dens, c + 24, 4);
    p.density = (double)dens;
    std::memcpy(&p.property_index, c + 28, 4);
    unsigned long idr;
    std::memcpy(&idr, c + 32, 8);
    p.id_in_run = (uint32_t)idr;
    unsigned cpu;
    std::memcpy(&cpu, c + 40, 4);
    p.cpu_id = (uint16_t)cpu;
}

int read_lis_files(const std::vector<std::string> &files, Snapshot &s) {
    if (files.empty()) return 3;
    long total = 0;
    std::vector<long> counts;
    for (size_t k = 0; k < files.size(); ++k) {
        std::ifstream f(files[k], std::ios::binary);
        if (!f.is_open()) {
            std::fprintf(stderr, "Error: Failed to open file %s\n", files[k].c_str());
            return 3;
        }
        long n = 0;
        if (k == 0) {
            read_header(f, s, n);
        } else {  // later files: only the count (src/tree.hpp:1344-1356)
            f.seekg((14 + s.type_info.size()) * sizeof(float) + sizeof(int), std::ios::beg);
            f.read(reinterpret_cast<char *>(&n), 8);
        }
        counts.push_back(n);
        total += n;
    }
    s.num_particles = (uint32_t)total;
    s.parts.assign(s.num_particles, Particle());
    uint32_t at = 0;
    for (size_t k = 0; k < files.size(); ++k) {
        std::ifstream f(files[k], std::ios::binary);
        f.seekg((14 + s.type_info.size()) * sizeof(float) + sizeof(int), std::ios::beg);
        long n = 0;
        f.read(reinterpret_cast<char *>(&n), 8);
        std::vector<char> body((size_t)n * 44);
        f.read(body.data(), (std::streamsize)body.size());
        for (long i = 0; i < n; ++i) unpack(body.data() + 44 * i, s.parts[at++]);
    }
    return 0;
}

void finish_read(Snapshot &s, Params &p, bool first_file) {  // src/tree.hpp:1551-1583
    std::sort(s.parts.begin(), s.parts.end(), [](const Particle &a, const Particle &b) {
        if (a.cpu_id == b.cpu_id) return a.id_in_run < b.id_in_run;
        return a.cpu_id < b.cpu_id;
    });
    for (uint32_t i = 0; i < s.num_particles; ++i) s.parts[i].id = i;
    if (first_file) {
        p.box_min = V3(s.coor_lim[6], s.coor_lim[8], s.coor_lim[10]);
        p.box_max = V3(s.coor_lim[7], s.coor_lim[9], s.coor_lim[11]);
        p.box_center = div(add(p.box_min, p.box_max), 2.0);
        p.box_length = sub(p.box_max, p.box_min);
        p.derive();
        size_t nt = s.type_info.size();
        p.mass_per_particle.assign(nt, 0);
        p.mass_fraction_per_species.assign(nt, 0);
        double sum = 0;
        for (size_t i = 0; i < nt; ++i) {
            p.mass_fraction_per_species[i] = s.type_info[i];
            sum += s.type_info[i];
        }
        for (size_t i = 0; i < nt; ++i) {
            p.mass_fraction_per_species[i] /= sum;
            p.mass_total_code_units = p.solid_to_gas_ratio * p.box_length[0] * p.box_length[1] * std::sqrt(2. * p.PI);
            p.mass_per_particle[i] = p.mass_fraction_per_species[i] * p.mass_total_code_units / s.num_particles;
        }
    }
    if (p.user_box) {  // src/tree.hpp:1585-1620
        auto in_range = [&](const V3 &v) {
            bool in = true;
            for (int d = 0; d < 3; ++d) in = in && (v[d] >= p.user_box_min[d] && v[d] <= p.user_box_max[d]);
            return in;
        };
        for (int d = 0; d < 3; ++d) {
            if (p.user_box_min[d] == 0 && p.user_box_max[d] == 0) {
                p.user_box_min[d] = p.box_min[d];
                p.user_box_max[d] = p.box_max[d];
            }
        }
        if (!(in_range(p.box_min) && in_range(p.box_max))) {
            std::vector<Particle> kept;
            for (uint32_t i = 0; i < s.num_particles; ++i)
                if (in_range(s.parts[i].pos)) kept.push_back(s.parts[i]);
            s.parts.swap(kept);
            s.num_particles = (uint32_t)s.parts.size();
        }
    }
}

void make_ghosts(Snapshot &s, const Params &p) {  // src/tree.hpp:1626-1754
    V3 w = sub(p.box_half_width, p.ghost_zone_width);
    for (int d = 0; d < 3; ++d) if (w[d] < 0) w[d] = 0;
    V3 lo = sub(p.box_center, w), hi = add(p.box_center, w);
    uint32_t next_id = s.num_particles;
    std::vector<Particle> gx, gy;
    for (uint32_t i = 0; i < s.num_particles; ++i) {
        const Particle &q = s.parts[i];
        if (q.pos[0] > hi[0]) {
            Particle g = q;
            g.id = next_id++;
            g.pos[0] -= p.box_length[0];
            double ny = g.pos[1] + p.shear_speed * s.time;
            g.pos[1] = ny - static_cast<int>((ny - p.box_min[1]) / p.box_length[1]) * p.box_length[1];
            gx.push_back(g);
        }
        if (q.pos[0] < lo[0]) {
            Particle g = q;
            g.id = next_id++;
            g.pos[0] += p.box_length[0];
            double ny = g.pos[1] - p.shear_speed * s.time;
            g.pos[1] = ny + static_cast<int>((p.box_max[1] - ny) / p.box_length[1]) * p.box_length[1];
            gx.push_back(g);
        }
    }
    for (const Particle &q : gx) {
        if (q.pos[1] < lo[1]) { Particle g = q; g.id = next_id++; g.pos[1] += p.box_length[1]; gy.push_back(g); }
        if (q.pos[1] > hi[1]) { Particle g = q; g.id = next_id++; g.pos[1] -= p.box_length[1]; gy.push_back(g); }
    }
    for (uint32_t i = 0; i < s.num_particles; ++i) {
        const Particle &q = s.parts[i];
        if (q.pos[1] < lo[1]) { Particle g = q; g.id = next_id++; g.pos[1] += p.box_length[1]; gy.push_back(g); }
        if (q.pos[1] > hi[1]) { Particle g = q; g.id = next_id++; g.pos[1] -= p.box_length[1]; gy.push_back(g); }
    }
    s.parts.resize(s.num_particles);
    s.parts.insert(s.parts.end(), gx.begin(), gx.end());
    s.parts.insert(s.parts.end(), gy.begin(), gy.end());
}

// ================================================================ Morton keys
static inline uint32_t double2int(double d) {  // src/tree.cpp:106-113
    double t = d * 4294967294.0 + 6755399441055744.0;
    uint64_t bits;
    std::memcpy(&bits, &t, 8);
    return (uint32_t)bits;
}

static inline Key dilate3(uint32_t v) {
    // Spread 32 bits three apart (bit b -> bit 3b). The reference multiplies masks
    // (src/tree.cpp:162-174); a plain loop gives the same 96-bit pattern.
    Key r = 0;
    for (int b = 0; b < 32; ++b) if (v >> b & 1u) r |= (Key)1 << (3 * b);
    return r;
}

Key Tree::morton(const V3 &pos, uint32_t index) const {  // src/tree.hpp:2315-2336
    V3 s = sub(pos, boxmin);
    Key r = (Key)index << 96;
    for (int d = 0; d < 3; ++d) {
        s[d] *= scale[d];
        r |= dilate3(double2int(s[d])) << d;
    }
    return r;
}

static inline int key_digit(Key k, int level) { return (int)((k >> (93 - 3 * (level - 1))) & 7); }
static inline Key low96(Key k) { return k << 32; }

static const int kOrth[8][3] = {{-1, -1, -1}, {1, -1, -1}, {-1, 1, -1}, {1, 1, -1},
                                {-1, -1, 1},  {1, -1, 1},  {-1, 1, 1},  {1, 1, 1}};

// ================================================================ tree build
void Tree::build(Params &p, std::vector<Particle> &parts, bool check_pos) {  // src/tree.hpp:2759
    pts.clear();
    nodes.clear();
    sinks.clear();
    check_outside = 0;
    const uint32_t n0 = (uint32_t)parts.size();
    if (check_pos) {
        V3 mn = parts[0].pos, mx = parts[0].pos;
        for (uint32_t i = 1; i < n0; ++i)
            for (int d = 0; d < 3; ++d) {
                mn[d] = std::min(parts[i].pos[d], mn[d]);
                mx[d] = std::max(parts[i].pos[d], mx[d]);
            }
        double ext = 0.0;
        for (int d = 0; d < 3; ++d) ext = std::max(ext, mx[d] - mn[d]);
        half_width = p.max_half_width + p.max_ghost_zone_width;
        root_center = p.box_center;
        if (ext < half_width) {
            half_width = (std::ceil(ext * 100.) + 1) / 100.;
            for (int d = 0; d < 3; ++d) {
                if (mx[d] - mn[d] < 0.5 * p.box_length[d]) {
                    root_center[d] = (mx[d] + mn[d]) / 2.0;
                    root_center[d] = std::round(root_center[d] * 1000.) / 1000.;
                } else {
                    root_center[d] = p.box_center[d];
                }
            }
        }
    } else if (half_width < 1e-16) {
        half_width = p.max_half_width + p.max_ghost_zone_width;
        root_center = p.box_center;
    }
    std::vector<TreePoint> raw(n0);
    for (uint32_t i = 0; i < n0; ++i) {
        raw[i].pos = parts[i].pos;
        raw[i].vel = parts[i].vel;
        raw[i].mass = p.mass_per_particle[parts[i].property_index];
        raw[i].ath_density = parts[i].density;
        raw[i].original_id = parts[i].id;
    }
    std::vector<Particle>().swap(parts);
    V3 hwv(half_width, half_width, half_width);
    boxmin = sub(root_center, hwv);
    V3 boxmax = add(root_center, hwv);
    for (int d = 0; d < 3; ++d) scale[d] = 1.0 / (boxmax[d] - boxmin[d]);
    epsilon = 2 * half_width / std::pow(2, 31);
    std::vector<Key> keys(n0);
    for (uint32_t i = 0; i < n0; ++i) keys[i] = morton(raw[i].pos, i);
    std::sort(keys.begin(), keys.end(), [](Key a, Key b) { return low96(a) < low96(b); });
    // SortPoints + MakeSinkParticle (src/tree.hpp:2591-2651)
    std::vector<Key> sk;
    sk.reserve(n0);
    for (uint32_t i = 0; i < n0;) {
        uint32_t src = (uint32_t)(keys[i] >> 96);
        if (i + 1 < n0 && low96(keys[i]) == low96(keys[i + 1])) {
            TreePoint t = raw[src];
            t.sink_flag = true;
            auto &members = sinks[(uint32_t)pts.size()];
            members.push_back(raw[src]);
            members.push_back(raw[(uint32_t)(keys[i + 1] >> 96)]);
            uint32_t j = i + 2;
            while (j < n0 && low96(keys[i]) == low96(keys[j])) members.push_back(raw[(uint32_t)(keys[j++] >> 96)]);
            pts.push_back(t);
            sk.push_back(keys[i]);
            i = j;
        } else {
            pts.push_back(raw[src]);
            sk.push_back(keys[i]);
            ++i;
        }
    }
    for (auto &it : sinks) {
        double mass = 0.0;
        V3 vel;
        for (auto &m : it.second) {
            vel = add(vel, mul(m.mass, m.vel));
            mass += m.mass;
        }
        vel = div(vel, mass);
        pts[it.first].mass = mass;
        pts[it.first].vel = vel;
    }
    const uint32_t n = (uint32_t)pts.size();
    // Octree: the reference counts nodes per level, then fills them depth first with node
    // index = level offset + rank within the level (src/tree.hpp:2655-2755, 2848-2886).
    int level_count[32] = {0};
    level_count[0] = 1;
    struct Seg { int level; uint32_t b, e; };
    // counting pass
    std::vector<Seg> stack;
    {
        std::vector<Seg> st{{1, 0, n}};
        while (!st.empty()) {
            Seg s = st.back();
            st.pop_back();
            std::vector<Seg> kids;
            uint32_t b = s.b;
            while (b < s.e) {
                int o = key_digit(sk[b], s.level);
                uint32_t e = b;
                while (e < s.e && key_digit(sk[e], s.level) == o) ++e;
                level_count[s.level]++;
                if (!(e - b <= max_leaf_size || s.level == 31)) kids.push_back({s.level + 1, b, e});
                b = e;
            }
            for (auto it = kids.rbegin(); it != kids.rend(); ++it) st.push_back(*it);
        }
    }
    int total = 0;
    for (int l = 0; l < 32; ++l) total += level_count[l];
    nodes.assign(total, Node());
    int level_ptr[32];
    level_ptr[0] = 0;
    for (int l = 1; l < 32; ++l) level_ptr[l] = level_ptr[l - 1] + level_count[l - 1];
    Node &root = nodes[0];
    root.center = root_center;
    root.half_width = half_width;
    root.begin = 0;
    root.end = n;
    root.level = 1;
    root.parent = std::numeric_limits<uint32_t>::max();
    // fill pass: recursive depth-first, same visiting order as FillTree
    struct Frame { int level; uint32_t b, e, parent; V3 c; double hw; };
    std::vector<Frame> st{{1, 0, n, 0, root_center, 0.5 * half_width}};
    std::vector<Frame> kids;
    while (!st.empty()) {
        Frame f = st.back();
        st.pop_back();
        kids.clear();
        uint32_t b = f.b;
        while (b < f.e) {
            int o = key_digit(sk[b], f.level);
            uint32_t e = b;
            while (e < f.e && key_digit(sk[e], f.level) == o) ++e;
            int d = level_ptr[f.level]++;
            Node &par = nodes[f.parent];
            if (par.first_daughter == 0) { par.first_daughter = d; par.num_daughters = 1; }
            else par.num_daughters++;
            Node &nd = nodes[d];
            nd.level = (uint8_t)(f.level + 1);
            nd.parent = f.parent;
            nd.begin = b;
            nd.end = e;
            nd.half_width = f.hw;
            for (int k = 0; k < 3; ++k) nd.center[k] = f.c[k] + f.hw * kOrth[o][k];
            nd.orthant = (uint16_t)o;
            if (!(e - b <= max_leaf_size || f.level == 31)) kids.push_back({f.level + 1, b, e, (uint32_t)d, nd.center, 0.5 * f.hw});
            b = e;
        }
        // FillTree recurses into each branch before creating the next sibling, so node
        // numbers within a level follow depth-first order; pushing in reverse keeps it.
        for (auto it = kids.rbegin(); it != kids.rend(); ++it) st.push_back(*it);
    }
    // CheckTree (src/tree.hpp:2924-2944): count points outside their node.
    for (size_t k = 0; k < nodes.size(); ++k)
        for (uint32_t i = nodes[k].begin; i < nodes[k].end; ++i)
            if (!within(pts[i].pos, nodes[k].center, nodes[k].half_width)) ++check_outside;
    cell_length = p.cell_length;
    half_cell_length = div(cell_length, 2.);
    cell_length_squared = V3(cell_length[0] * cell_length[0], cell_length[1] * cell_length[1], cell_length[2] * cell_length[2]);
    three_half_cell_length = mul(half_cell_length, 3.);
}

bool Tree::within(const V3 &pos, const V3 &c, double hw) const {  // src/tree.hpp:2912-2919
    for (int d = 0; d < 3; ++d)
        if (!(pos[d] >= c[d] - hw - epsilon && pos[d] <= c[d] + hw + epsilon)) return false;
    return true;
}

uint32_t Tree::pos2node(const V3 &pos) const {  // Pos2Node + Key2Leaf, src/tree.hpp:2968-2997
    Key k = morton(pos, 0);
    uint32_t node = 0;
    int level = 1;
    while (nodes[node].num_daughters != 0) {
        int o = key_digit(k, level);
        uint32_t found = UINT32_MAX;
        for (uint32_t d = nodes[node].first_daughter; d != nodes[node].first_daughter + nodes[node].num_daughters; ++d)
            if (nodes[d].orthant == o) { found = d; break; }
        if (found == UINT32_MAX) return UINT32_MAX;
        node = found;
        ++level;
    }
    return node;
}

bool Tree::sphere_contains(const V3 &c, double r, uint32_t node) const {  // src/tree.hpp:3001-3015
    const Node &nd = nodes[node];
    V3 md = sub(nd.center, c);
    double diag = nd.half_width * std::sqrt(3);
    for (int i = 0; i < 3; ++i) md[i] = std::fabs(md[i]) + diag;
    return norm2(md) < r * r;
}

bool Tree::sphere_intersects(const V3 &c, double r, uint32_t node) const {  // src/tree.hpp:3019-3049
    const Node &nd = nodes[node];
    double c2c = norm2(sub(nd.center, c));
    double t = nd.half_width * std::sqrt(3) + r;
    if (c2c > t * t) return false;
    if (c2c < r || c2c < nd.half_width) return true;
    V3 hw(nd.half_width, nd.half_width, nd.half_width);
    V3 lo = sub(nd.center, hw), hi = add(nd.center, hw);
    double m2 = 0;
    for (int d = 0; d < 3; ++d) {
        if (c[d] < lo[d]) m2 += (c[d] - lo[d]) * (c[d] - lo[d]);
        else if (c[d] > hi[d]) m2 += (c[d] - hi[d]) * (c[d] - hi[d]);
    }
    return m2 <= r * r;
}

namespace {
struct LessSecond {
    bool operator()(const std::pair<int, double> &a, const std::pair<int, double> &b) const { return a.second < b.second; }
};
inline void heap_add(Heap &h, unsigned k, int i, double dr2) {  // Add2Heaps, src/tree.hpp:3063-3075
    if (h.size() < k) {
        h.emplace_back(i, dr2);
        std::push_heap(h.begin(), h.end(), LessSecond());
    } else if (dr2 < h.front().second) {
        std::pop_heap(h.begin(), h.end(), LessSecond());
        h.pop_back();
        h.emplace_back(i, dr2);
        std::push_heap(h.begin(), h.end(), LessSecond());
    }
}
}  // namespace

bool Tree::knn(const V3 &pos, unsigned k, Heap &heap, double est) const {  // src/tree.hpp:3198-3251
    double r;
    if (est == 0) {
        double r2 = 0;
        if (within(pos, root_center, half_width)) {
            uint32_t node = pos2node(pos);
            if (node == UINT32_MAX) {
                heap.clear();
                return false;
            }
            while (nodes[node].end - nodes[node].begin < k / 4) node = nodes[node].parent;
            r2 = nodes[node].half_width * nodes[node].half_width;
        } else {
            for (int d = 0; d < 3; ++d) {
                double dx = std::max(std::max(root_center[d] - half_width - pos[d], 0.0), pos[d] - root_center[d] - half_width);
                r2 += dx * dx;
            }
        }
        r = std::sqrt(r2);
    } else {
        r = est;
    }
    std::vector<uint32_t> st;
    do {
        heap.clear();
        st.assign(1, 0);
        // RecursiveKNN_OpenMP (src/tree.hpp:3177-3193) with an explicit stack; daughters are
        // pushed in reverse so they are visited in ascending order, as the recursion does.
        while (!st.empty()) {
            uint32_t node = st.back();
            st.pop_back();
            const Node &nd = nodes[node];
            if (sphere_contains(pos, r, node)) {
                for (uint32_t q = nd.begin; q != nd.end; ++q) heap_add(heap, k, (int)q, norm2(sub(pos, pts[q].pos)));
            } else if (sphere_intersects(pos, r, node)) {
                if (nd.num_daughters == 0) {
                    for (uint32_t q = nd.begin; q != nd.end; ++q) heap_add(heap, k, (int)q, norm2(sub(pos, pts[q].pos)));
                } else {
                    for (int d = nd.num_daughters - 1; d >= 0; --d) st.push_back(nd.first_daughter + d);
                }
            }
        }
        r *= 2;
    } while (heap.size() < k);
    std::sort_heap(heap.begin(), heap.end(), LessSecond());
    return true;
}

void Tree::ball(const V3 &c, double r, std::vector<uint32_t> &out) const {  // src/tree.hpp:3275-3304
    out.clear();
    std::vector<uint32_t> st{0};
    while (!st.empty()) {
        uint32_t node = st.back();
        st.pop_back();
        const Node &nd = nodes[node];
        if (sphere_contains(c, r, node)) {
            for (uint32_t q = nd.begin; q != nd.end; ++q) out.push_back(q);
        } else if (sphere_intersects(c, r, node)) {
            if (nd.num_daughters == 0) {
                for (uint32_t q = nd.begin; q != nd.end; ++q)
                    if (norm2(sub(c, pts[q].pos)) <= r * r) out.push_back(q);
            } else {
                for (int d = nd.num_daughters - 1; d >= 0; --d) st.push_back(nd.first_daughter + d);
            }
        }
    }
}

uint32_t Tree::ball_count_sheared(const V3 &c, double r, const V3 &max_distance, double shear_distance, const Params &p) const {
    const double diag_f = std::sqrt(3);  // to_diagonal
    uint32_t count = 0;
    std::vector<uint32_t> st{0};
    while (!st.empty()) {
        const uint32_t node = st.back();
        st.pop_back();
        const Node &nd = nodes[node];
        // ShearedCenter2Center (src/tree.hpp:3308-3331): the node's image across the x
        // faces also moves in y by the shear, which the y component then sees
        V3 nc = nd.center, c2c;
        for (int i = 0; i < 3; ++i) {
            c2c[i] = c[i] - nc[i];
            if (std::fabs(c2c[i]) > max_distance[i]) {
                if (c2c[i] > 0) c2c[i] -= p.box_length[i];
                else c2c[i] += p.box_length[i];
                if (i == 0) {
                    if (c[0] < 0) {
                        nc[1] -= shear_distance;
                        nc[1] += static_cast<int>((p.box_max[1] - nc[1]) / p.box_length[1]) * p.box_length[1];
                    } else {
                        nc[1] += shear_distance;
                        nc[1] -= static_cast<int>((nc[1] - p.box_min[1]) / p.box_length[1]) * p.box_length[1];
                    }
                }
            }
        }
        // SphereContainNodeWithShear (src/tree.hpp:3335-3346)
        const double tmp = nd.half_width * diag_f;
        V3 td;
        for (int i = 0; i < 3; ++i) td[i] = std::fabs(c2c[i]) + tmp;
        if (norm2(td) < r * r) {
            count += nd.end - nd.begin;
            continue;
        }
        // SphereNodeIntersectWithShear (src/tree.hpp:3350-3380)
        const double cd = norm2(c2c), tr = tmp + r;
        if (cd > tr * tr) continue;
        bool hit = cd < r || cd < nd.half_width;
        if (!hit) {
            double m2 = 0;
            for (int d = 0; d < 3; ++d) {
                const double lo = (c[d] - c2c[d]) - nd.half_width, hi = (c[d] - c2c[d]) + nd.half_width;
                if (c[d] < lo) m2 += (c[d] - lo) * (c[d] - lo);
                else if (c[d] > hi) m2 += (c[d] - hi) * (c[d] - hi);
            }
            hit = m2 <= r * r;
        }
        if (!hit) continue;
        if (nd.num_daughters == 0) {  // the points themselves are compared without the image
            for (uint32_t q = nd.begin; q != nd.end; ++q)
                if (norm2(sub(c, pts[q].pos)) <= r * r) ++count;
        } else {
            for (int d = nd.num_daughters - 1; d >= 0; --d) st.push_back(nd.first_daughter + d);
        }
    }
    return count;
}

DensityVsScale density_vs_scale(const Tree &t, const Params &p, double time) {
    DensityVsScale out;
    // z range: from the cell centre at the box centre down past the lowest point, up to the
    // highest point (RecursiveFindExtreme finds the extreme values exactly)
    double zlo = t.pts[0].pos[2], zhi = t.pts[0].pos[2];
    for (const auto &q : t.pts) {
        zlo = std::min(zlo, q.pos[2]);
        zhi = std::max(zhi, q.pos[2]);
    }
    double z_min = p.box_center[2] - p.cell_length[2] / 2.0;
    const double z_max = zhi;
    while (z_min - p.cell_length[2] > zlo) z_min -= p.cell_length[2];
    const int num_levels = (int)std::round(std::log10(p.box_half_width[0] * 2 / p.cell_length[0]) / std::log10(2.0)) + 1;
    out.radii.assign(num_levels, p.cell_length[0] / 2.0);
    out.max_rhop.assign(num_levels, 0.0);
    std::vector<V3> maxd(num_levels);
    const double shear = p.shear_speed * time;
    for (int i = 0; i < num_levels; ++i) {
        out.radii[i] *= std::pow(2.0, i);
        for (int d = 0; d < 3; ++d) maxd[i][d] = p.box_length[d] - out.radii[i];
        maxd[i][2] = 100 * p.max_half_width;  // no periodic search in z
    }
    const V3 cmin(p.box_min[0] + 0.5 * p.cell_length[0], p.box_min[1] + 0.5 * p.cell_length[1], p.box_min[2] + 0.5 * p.cell_length[2]);
    const V3 step = p.cell_length, sub1 = div(step, 2.0), sub2 = div(step, 4.0);
    for (double z = z_min; z < z_max; z += step[2]) {
        for (double y = cmin[1]; y < p.box_max[1]; y += step[1]) {
            for (double x = cmin[0]; x < p.box_max[0]; x += step[0]) {
                const V3 c(x, y, z);
                for (int i = 0; i < num_levels; ++i) {
                    double &mx = out.max_rhop[i];
                    uint32_t n = t.ball_count_sheared(c, out.radii[i], maxd[i], shear, p);
                    if (n > mx) mx = n;
                    if (i >= 3) continue;
                    for (int o = 0; o < 8; ++o) {  // the eight sub-centres
                        V3 sc;
                        for (int d = 0; d < 3; ++d) sc[d] = c[d] + sub1[d] * kOrth[o][d];
                        n = t.ball_count_sheared(sc, out.radii[i], maxd[i], shear, p);
                        if (n > mx) mx = n;
                        if (i == 0) {
                            // the reference's inner loop offsets by the outer orthant eight
                            // times (src/analyses.hpp:296-305): one more centre per orthant
                            V3 ss;
                            for (int d = 0; d < 3; ++d) ss[d] = sc[d] + sub2[d] * kOrth[o][d];
                            n = t.ball_count_sheared(ss, out.radii[i], maxd[i], shear, p);
                            if (n > mx) mx = n;
                        }
                    }
                }
            }
        }
    }
    std::ostringstream h, l;
    h << std::setw(15) << std::setfill(' ') << "#time";
    for (double r : out.radii) h << std::setw(15) << std::setfill(' ') << std::scientific << r;
    h << "\n";
    l << std::setw(15) << std::setfill(' ') << std::scientific << time;
    for (int i = 0; i < num_levels; ++i) {
        out.max_rhop[i] *= (p.mass_per_particle[0] / (4.1887902047863910 * std::pow(out.radii[i], 3)));
        l << std::setw(15) << std::setfill(' ') << std::scientific << out.max_rhop[i];
    }
    l << "\n";
    out.header = h.str();
    out.line = l.str();
    return out;
}

uint32_t Tree::ball_count(const V3 &c, double r) const {
    std::vector<uint32_t> v;
    ball(c, r, v);
    return (uint32_t)v.size();
}

// src/tree.hpp:3406-3419. The reference writes std::pow(v, 2.); its optimised build (GCC,
// -O2 and above) turns that call into v * v, the correctly rounded square, so that is what
// it computes (glibc's pow(v, 2.) itself differs from v * v by one unit in the last place on
// about one argument in a thousand).
double Tree::quadratic_spline(V3 dist) const {
    for (int d = 0; d < 3; ++d) dist[d] = std::fabs(dist[d]);
    double w = 1;
    for (int i = 0; i < 3; ++i) {
        if (dist[i] <= half_cell_length[i]) {
            w *= (0.75 - dist[i] * dist[i] / cell_length_squared[i]);
        } else if (dist[i] < three_half_cell_length[i]) {
            const double v = 1.5 - dist[i] / cell_length[i];
            w *= 0.5 * (v * v);
        } else {
            return 0.;
        }
    }
    return w;
}

// ================================================================ correctly rounded powers
double cr_pow15(double x) {
    if (!(x > 0) || std::isinf(x)) return std::pow(x, 1.5);
    double s = std::sqrt(x);
    double r = std::fma(-s, s, x);          // exact residual x - s^2
    double t = r / (2.0 * s);               // sqrt(x) = s + t to ~2^-106
    double p = x * s;
    double e = std::fma(x, s, -p);          // exact low part of x*s
    return p + (e + x * t);
}

double cr_pow_third(double x) {
    if (!(x > 0) || std::isinf(x)) return std::pow(x, 1. / 3.);
    double c0 = std::cbrt(x);
    double c2 = c0 * c0, e2 = std::fma(c0, c0, -c2);
    double c3 = c2 * c0, c3l = std::fma(c2, c0, -c3) + e2 * c0;
    double r = (x - c3) - c3l;
    double clo = r / (3.0 * c2);
    // x^(1/3.) = cbrt(x) * x^(-delta), delta = 1/3 - (double)(1/3.) = 2^-54/3
    const double delta = 1.8503717077085943e-17;
    double L = std::log(x);
    return c0 + (clo - c0 * (delta * L));
}

double Finder::pow15(double x) const { return pow_mode == POW_LIBM ? std::pow(x, 1.5) : cr_pow15(x); }
double Finder::hill_pow(double x) const { return pow_mode == POW_LIBM ? std::pow(x, 1. / 3.) : cr_pow_third(x); }

// ================================================================ density kernels
double Finder::density_kernel(const Heap &h, uint32_t self, unsigned k) const {
    if (median_kernel) {  // MedianSphericalDensityKernel, src/tree.hpp:3473-3491
        int i = (int)k;
        double t = 4 * h[i / 2].second;
        for (i = i - 1; i >= 0; i--) {
            if (h[i].second > t) continue;
            break;
        }
        t = h[i].second;
        double dens = 0;
        for (; i >= 0; i--) dens += tree.pts[h[i].first].mass;
        dens /= par->four_PI_over_three * pow15(t);
        return dens;
    }
    double dens = 0;  // QseudoQuadraticSplinesKernel, src/tree.hpp:3427-3434
    for (unsigned i = 0; i < k; ++i)
        dens += tree.pts[h[i].first].mass / par->cell_volume * tree.quadratic_spline(sub(tree.pts[h[i].first].pos, tree.pts[self].pos));
    return dens;
}

// ================================================================ clump helpers
void Finder::kinematics(Clump &c) const {  // src/tree.hpp:4431-4442
    c.total_mass = 0;
    c.center_of_mass = V3();
    c.vel_com = V3();
    for (uint32_t i : c.indices) {
        const TreePoint &t = tree.pts[i];
        c.total_mass += t.mass;
        c.center_of_mass = add(c.center_of_mass, mul(t.pos, t.mass));
        c.vel_com = add(c.vel_com, mul(t.vel, t.mass));
    }
    c.center_of_mass = div(c.center_of_mass, c.total_mass);
    c.vel_com = div(c.vel_com, c.total_mass);
}

void Finder::one10th(Clump &c) const {  // shared tail of SortParticles / Merge, src/tree.hpp:4461-4511
    const auto &P = c.particles;
    double tenth = tree.pts[c.indices[c.indices.size() / 2]].new_density / 10.;
    size_t a = 0;
    for (; a < P.size(); ++a) if (tree.pts[P[a].first].new_density < tenth) break;
    c.inner_one10th_radius = (a != P.size()) ? P[a].second : P.back().second;
    size_t b = P.size();
    for (; b > 0; --b) if (tree.pts[P[b - 1].first].new_density > tenth) break;
    // when no member exceeds the cut the reference dereferences rend(); b == 0 never
    // happens because the median member itself has density > its tenth when positive
    c.outer_one10th_radius = P[b > 0 ? b - 1 : 0].second;
    c.one10th_radius = (c.inner_one10th_radius + c.outer_one10th_radius) / 2.;
    double m = 0., tenth_mass = c.total_mass * (1.0 - 0.95);
    size_t r = P.size();
    for (; r > 0; --r) {
        m += tree.pts[P[r - 1].first].mass;
        if (m > tenth_mass) break;
    }
    c.two_sigma_mass_radius = P[r > 0 ? r - 1 : 0].second;
    if (c.inner_one10th_radius > 0 && c.outer_one10th_radius / c.inner_one10th_radius > 2.5)
        c.one10th_radius = std::min(c.outer_one10th_radius, c.two_sigma_mass_radius);
    else
        c.one10th_radius = std::min(c.one10th_radius, c.two_sigma_mass_radius);
}

static void sort_by_distance(std::vector<std::pair<uint32_t, double>> &P) {
    std::sort(P.begin(), P.end(), [](const std::pair<uint32_t, double> &a, const std::pair<uint32_t, double> &b) { return a.second < b.second; });
}

void Finder::sort_particles(Clump &c) const {  // src/tree.hpp:4446-4512
    kinematics(c);
    for (uint32_t i : c.indices) c.particles.emplace_back(i, norm(sub(tree.pts[i].pos, c.center_of_mass)));
    sort_by_distance(c.particles);
    for (size_t k = 0; k < c.particles.size(); ++k) c.indices[k] = c.particles[k].first;
    one10th(c);
}

bool Finder::dispersion_too_large(const Clump &c, double tol) const {  // src/tree.hpp:4516-4528
    size_t n = c.particles.size();
    double s = 0.0;
    for (size_t i = 0; i < n; ++i) s = s + c.particles[i].second * c.particles[i].second;
    return s / n > std::pow(tol * c.particles[n - 1].second, 2);
}

void Finder::merge(Clump &a, Clump &b) const {  // MergeAnotherPlanetesimal, src/tree.hpp:4532-4611
    if (tree.pts[a.peak_index].new_density < tree.pts[b.peak_index].new_density) {
        a.potential_subpeak_indices.push_back(a.peak_index);
        a.peak_index = b.peak_index;
    } else {
        a.potential_subpeak_indices.push_back(b.peak_index);
    }
    double M = a.total_mass + b.total_mass;
    a.center_of_mass = div(add(mul(a.center_of_mass, a.total_mass), mul(b.center_of_mass, b.total_mass)), M);
    a.vel_com = div(add(mul(a.vel_com, a.total_mass), mul(b.vel_com, b.total_mass)), M);
    a.total_mass = M;
    a.particles.insert(a.particles.end(), b.particles.begin(), b.particles.end());
    for (auto &q : a.particles) q.second = norm(sub(tree.pts[q.first].pos, a.center_of_mass));
    sort_by_distance(a.particles);
    a.indices.resize(a.particles.size());
    for (size_t k = 0; k < a.particles.size(); ++k) a.indices[k] = a.particles[k].first;
    one10th(a);
}

void Finder::remove_unbound(Clump &c) const {  // src/tree.hpp:4615-4674
    const Params &p = *par;
    size_t i = c.particles.size() - 1;
    while (i != 0) {
        const TreePoint &t = tree.pts[c.particles[i].first];
        double Mr = c.total_mass - t.mass;
        V3 com = div(sub(mul(c.center_of_mass, c.total_mass), mul(t.pos, t.mass)), Mr);
        V3 vcom = div(sub(mul(c.vel_com, c.total_mass), mul(t.vel, t.mass)), Mr);
        V3 dv = sub(sub(vcom, mul(p.shear_vector, com[0] - t.pos[0])), t.vel);
        double e = +0.5 / c.total_mass * norm2(dv) - p.grav_constant / norm(sub(com, t.pos));
        if (e > 0) {
            std::swap(c.indices[i], c.indices.back());
            c.indices.pop_back();
            std::swap(c.particles[i], c.particles.back());
            c.particles.pop_back();
            c.vel_com = vcom;
            c.center_of_mass = com;
            c.total_mass = Mr;
        }
        i--;
    }
    c.particles.clear();
    sort_particles(c);
}

// Replays one call's candidates with the reference's own test and update, in sequence and
// in five ways of stepping through them, and counts the steps of each (a step being what one
// pass of a warp or block does before the state may change):
//   0, 1, 2  first bound: test the next 32, 256 or 1024 candidates against the state, take the
//            first bound one (or none) and continue after it;
//   3        speculative windows of 32: all decided against the window's first state, the
//            state chained through those tentative acceptances, each decision checked against
//            the state before it, the agreeing prefix kept and the first disagreeing candidate
//            decided exactly;
//   4        as 3, but a 256-wide scan first skips to the next candidate bound under the
//            current state, so a stretch without any bound candidate costs one step.
// The speculative results must equal the sequential one.
void Finder::count_windows(const Clump &c, const std::vector<uint32_t> &near) {
    struct St {
        double M;
        V3 com, vcom;
    };
    const Params &p = *par;
    std::vector<uint32_t> E;
    for (uint32_t idx : near)
        if (!tree.pts[idx].in_clump_flag && tree.pts[idx].new_density >= density_threshold) E.push_back(idx);
    auto bound = [&](const St &s, uint32_t idx) {
        const TreePoint &t = tree.pts[idx];
        double M = s.M + t.mass;
        V3 dv = sub(sub(s.vcom, mul(p.shear_vector, s.com[0] - t.pos[0])), t.vel);
        return +0.5 / M * norm2(dv) - p.grav_constant / norm(sub(s.com, t.pos)) < 0;
    };
    auto update = [&](St &s, uint32_t idx) {
        const TreePoint &t = tree.pts[idx];
        s.M = s.M + t.mass;
        s.com = div(add(mul(s.com, s.M), mul(t.mass, t.pos)), s.M);
        s.vcom = div(add(mul(s.M, s.vcom), mul(t.mass, t.vel)), s.M);
    };
    const St s0{c.total_mass, c.center_of_mass, c.vel_com};
    const size_t n = E.size();
    std::vector<size_t> seq;
    St s = s0;
    for (size_t k = 0; k < n; ++k)
        if (bound(s, E[k])) {
            update(s, E[k]);
            seq.push_back(k);
        }
    uint64_t steps[kWindowSchemes] = {0};
    const size_t widths[3] = {32, 256, 1024};
    for (int wi = 0; wi < 3; ++wi) {
        s = s0;
        for (size_t at = 0; at < n; ++steps[wi]) {
            const size_t end = std::min(at + widths[wi], n);
            size_t j = end;
            for (size_t k = at; k < end && j == end; ++k)
                if (bound(s, E[k])) j = k;
            if (j < end) update(s, E[j]);
            at = j < end ? j + 1 : end;
        }
    }
    uint64_t busy = 0;
    // one speculative window from `at` (32 candidates at most); returns the next position
    auto window = [&](St &st, size_t at, std::vector<size_t> &acc, bool count) {
        const int w = (int)(std::min(at + 32, n) - at);
        bool tent[32];
        St chain[33];
        chain[0] = st;
        int nt = 0;
        for (int l = 0; l < w; ++l) {
            tent[l] = bound(st, E[at + l]);
            if (tent[l]) {
                chain[nt + 1] = chain[nt];
                update(chain[nt + 1], E[at + l]);
                ++nt;
            }
        }
        int below = 0, m = -1, kept = 0;
        for (int l = 0; l < w && m < 0; ++l) {
            if (bound(chain[below], E[at + l]) != tent[l]) m = l;
            else if (tent[l]) {
                acc.push_back(at + l);
                ++below;
                ++kept;
            }
        }
        st = chain[below];
        size_t next = at + (size_t)w;
        if (m >= 0) {
            if (count) ++window_stats.mismatch_windows;
            if (!tent[m]) {  // the exact state binds it
                update(st, E[at + m]);
                acc.push_back(at + m);
                ++kept;
            }
            next = at + (size_t)m + 1;
        }
        if (count) {
            ++window_stats.accepted_per_window[kept];
            if (kept) ++busy;
        }
        return next;
    };
    std::vector<size_t> spec3, spec4;
    s = s0;
    for (size_t at = 0; at < n; ++steps[3]) at = window(s, at, spec3, true);
    s = s0;
    for (size_t at = 0; at < n; ++steps[4]) {
        const size_t end = std::min(at + 256, n);
        size_t f = end;
        for (size_t k = at; k < end && f == end; ++k)
            if (bound(s, E[k])) f = k;
        at = f < end ? window(s, f, spec4, false) : end;
    }
    WindowStats &ws = window_stats;
    ws.calls++;
    ws.candidates += n;
    ws.accepted += seq.size();
    auto &pc = ws.per_clump[c.peak_index];
    pc.accepted += seq.size();
    pc.busy_windows += busy;
    pc.call.push_back({(uint64_t)seq.size(), steps[0], steps[3], busy});
    for (int k = 0; k < kWindowSchemes; ++k) {
        ws.steps[k] += steps[k];
        ws.longest_call[k] = std::max(ws.longest_call[k], steps[k]);
        pc.steps[k] += steps[k];
    }
    if (spec3 != seq || spec4 != seq) ws.disagreements++;
}

void Finder::search_bound_in_hill(Clump &c) {  // src/tree.hpp:4678-4711
    std::vector<uint32_t> near;
    tree.ball(c.center_of_mass, c.Hill_radius, near);
    if (window_stats_on) {
        count_windows(c, near);
        auto &pc = window_stats.per_clump[c.peak_index];
        pc.calls++;
        const size_t members_before = c.indices.size();
        search_bound_in_hill_loop(c, near);
        if (c.indices.size() > members_before) pc.grown_members += c.indices.size();
        return;
    }
    search_bound_in_hill_loop(c, near);
}

// The acceptance loop over the ball's points and the final SortParticles (src/tree.hpp:4686-4710).
void Finder::search_bound_in_hill_loop(Clump &c, const std::vector<uint32_t> &near) {
    const Params &p = *par;
    for (uint32_t idx : near) {
        TreePoint &t = tree.pts[idx];
        if (t.in_clump_flag || t.new_density < density_threshold) continue;
        double M = c.total_mass + t.mass;
        V3 dv = sub(sub(c.vel_com, mul(p.shear_vector, c.center_of_mass[0] - t.pos[0])), t.vel);
        double e = +0.5 / M * norm2(dv) - p.grav_constant / norm(sub(c.center_of_mass, t.pos));
        if (e < 0) {
            c.indices.push_back(idx);
            c.total_mass = M;
            c.center_of_mass = div(add(mul(c.center_of_mass, c.total_mass), mul(t.mass, t.pos)), c.total_mass);
            c.vel_com = div(add(mul(c.total_mass, c.vel_com), mul(t.mass, t.vel)), c.total_mass);
            t.in_clump_flag = true;
        }
    }
    if (c.indices.size() > c.particles.size()) {
        c.particles.clear();
        sort_particles(c);
    }
}

void Finder::hill(Clump &c) const {  // src/tree.hpp:4715-4717
    c.Hill_radius = hill_pow(c.total_mass * par->grav_constant / 3. / par->Omega / par->Omega);
}

void Finder::angular_momentum(Clump &c) const {  // src/tree.hpp:4721-4747
    const Params &p = *par;
    double units = c.total_mass * c.Hill_radius * c.Hill_radius * p.Omega;
    V3 shear(0., p.q * p.Omega, 0.);
    for (auto &q : c.particles) {
        const TreePoint &t = tree.pts[q.first];
        V3 dr = sub(t.pos, c.center_of_mass);
        V3 dv = sub(sub(t.vel, mul(shear, t.pos[0])), sub(c.vel_com, mul(shear, c.center_of_mass[0])));
        V3 j(dr[1] * dv[2] - dr[2] * dv[1], dr[2] * dv[0] - dr[0] * dv[2], dr[0] * dv[1] - dr[1] * dv[0]);
        j = add(j, mul(p.Omega, V3(-dr[0] * dr[2], -dr[1] * dr[2], (dr[0] * dr[0] + dr[1] * dr[1]))));
        c.J = add(c.J, mul(t.mass, j));
    }
    c.J = div(c.J, units);
}

bool Finder::bound(const Clump &a, const Clump &b) const {  // src/tree.hpp:4867-4874
    const Params &p = *par;
    double M = a.total_mass + b.total_mass;
    double pg = -p.grav_constant / norm(sub(a.center_of_mass, b.center_of_mass));
    V3 dv = sub(sub(a.vel_com, mul(p.shear_vector, a.center_of_mass[0] - b.center_of_mass[0])), b.vel_com);
    double ek = 0.5 / M * norm2(dv);
    return pg + ek < 0.;
}

bool Finder::saddle_deep(const Clump &a, const Clump &b, bool hill_mode) const {  // src/tree.hpp:4880-4909
    double ra = hill_mode ? a.Hill_radius : a.one10th_radius;
    double rb = hill_mode ? b.Hill_radius : b.one10th_radius;
    V3 r12 = sub(b.center_of_mass, a.center_of_mass);
    double f = ra / (ra + rb);
    for (int d = 0; d < 3; ++d) r12[d] *= f;
    V3 sp = add(a.center_of_mass, r12);
    double est = std::min(ra, rb);
    if (hill_mode) est = est / Hill_fraction_for_merge;
    Heap h;
    tree.knn(sp, par->knn, h, est);
    double dens = density_kernel(h, 0, par->knn);
    return dens < 2.5 * density_threshold;
}

void Finder::remove_small_and_low() {  // src/tree.hpp:3524-3546
    std::vector<uint32_t> del;
    for (auto &it : clumps) {
        if (it.second.total_mass < clump_mass_threshold || tree.pts[it.first].new_density < peak_density_threshold) {
            del.push_back(it.first);
            continue;
        }
        size_t lim = std::min<size_t>(it.second.indices.size(), par->knn);
        double m = 0;
        for (size_t k = 0; k < lim; ++k) m = std::max(m, tree.pts[it.second.indices[k]].ath_density);
        if (m < peak_density_threshold) del.push_back(it.first);
    }
    for (auto k : del) clumps.erase(k);
}

void Finder::build_clump_tree(Tree &ct, double &max_radius, bool hill_mode) {  // src/tree.hpp:5251-5284
    std::vector<Particle> cs;
    for (auto &it : clumps) {
        if (!it.second.mask) continue;
        Particle q;
        q.pos = it.second.center_of_mass;
        q.vel = it.second.vel_com;
        q.id = (uint32_t)cs.size();
        q.density = it.first;
        q.property_index = 0;
        cs.push_back(q);
        double r = hill_mode ? it.second.Hill_radius * Hill_fraction_for_merge : it.second.one10th_radius;
        max_radius = std::max(r, max_radius);
    }
    if (cs.size() != num_planetesimals) stats.zero_key_quirk++;
    ct.root_center = tree.root_center;
    ct.half_width = tree.half_width;
    if (cs.empty()) { ct.pts.clear(); ct.nodes.clear(); return; }
    ct.build(*par, cs, false);
}

// ================================================================ FindPlanetesimals
std::string Finder::find(uint32_t num_in) {
    Params &p = *par;
    num_input_particles = num_in;
    clumps.clear();
    peaks_and_masses.clear();
    stats = Stats();
    const uint32_t T = tree.size();
    // KNN_Search_OpenMP asserts knn <= num_particles (src/tree.hpp:3199). The reference is
    // built with NDEBUG, and then its radius-doubling loop never ends on such a snapshot: the
    // restatement refuses it, as the device path does.
    if (p.knn < 1 || p.hop < 1 || p.knn > T || p.hop > T)
        throw std::domain_error("knn and hop must be at least 1 and not exceed the number of tree points");
    // kernel choice, src/tree.hpp:3576-3611
    uint32_t horiz = p.box_resolution[0] * p.box_resolution[1];
    if (tree.half_width < p.max_half_width + p.max_ghost_zone_width - 1e-16)
        horiz = (uint32_t)std::pow(tree.half_width / p.cell_length[0] * ((tree.half_width - p.max_ghost_zone_width) / tree.half_width), 2.0);
    if (num_in >= 4 * horiz) {
        if (!p.fixed_hop && num_in >= 1.67e7) p.hop = 64;
        enough_particle_resolution = 1;
        median_kernel = true;
    } else {
        enough_particle_resolution = 0;
        median_kernel = false;
    }
    // thresholds, src/tree.hpp:3633-3660
    density_threshold = std::pow(p.Omega, 2.) / p.PI / p.grav_constant * 2.;
    if (p.mass_total_code_units / num_in / p.cell_volume > density_threshold / 4) density_threshold *= 9. / 8.;
    double res_min = std::min(std::min((double)p.box_resolution[0] / p.box_length[0], (double)p.box_resolution[1] / p.box_length[1]), (double)p.box_resolution[2] / p.box_length[2]);
    unsigned hydro = (unsigned)res_min;
    clump_diffuse_threshold = 0.55;
    Hill_fraction_for_merge = 0.25;
    if (hydro <= 1024) { clump_diffuse_threshold = 0.35; Hill_fraction_for_merge = 0.75; }
    else if (hydro <= 1536) { clump_diffuse_threshold = 0.4; Hill_fraction_for_merge = 0.5; }
    else if (hydro <= 2048) { clump_diffuse_threshold = 0.5; Hill_fraction_for_merge = 0.35; }
    if (p.clump_diffuse_threshold > 0) clump_diffuse_threshold = p.clump_diffuse_threshold;
    if (p.Hill_fraction_for_merge > 0) Hill_fraction_for_merge = p.Hill_fraction_for_merge;
    clump_mass_threshold = p.min_trusted_mass;
    peak_density_threshold = 3 * density_threshold;

    // PLAN_ORACLE_TRACE=1 prints the wall time of each phase to stderr
    const bool trace_on = std::getenv("PLAN_ORACLE_TRACE") != nullptr;
    auto t_last = std::chrono::steady_clock::now();
    auto phase_mark = [&](const char *what) {
        if (!trace_on) return;
        auto t = std::chrono::steady_clock::now();
        std::fprintf(stderr, "[oracle] %-16s %9.1f ms\n", what, std::chrono::duration<double, std::milli>(t - t_last).count());
        t_last = t;
    };
    // 1. densities, src/tree.hpp:3667-3689
#pragma omp parallel num_threads(threads)
    {
        Heap h;
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < (int64_t)T; ++i) {
            tree.knn(tree.pts[i].pos, p.knn, h);
            tree.pts[i].new_density = density_kernel(h, (uint32_t)i, p.knn);
        }
    }
    phase_mark("density");
    // 2. densest neighbour, src/tree.hpp:3711-3760
    densest.assign(T, 0);
#pragma omp parallel num_threads(threads)
    {
        Heap h;
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < (int64_t)T; ++i) {
            densest[i] = (uint32_t)i;
            if (tree.pts[i].new_density < density_threshold) continue;
            tree.knn(tree.pts[i].pos, p.hop, h);
            double best = tree.pts[i].new_density;
            for (unsigned j = 0; j < p.hop; ++j) {
                uint32_t q = (uint32_t)h[j].first;
                double dq = tree.pts[q].new_density;
                if (best < dq) { densest[i] = q; best = dq; }
                else if (best == dq && densest[i] > q) densest[i] = q;
            }
        }
    }
    phase_mark("densest");
    // 3. HOP chains, src/tree.hpp:3766-3809
    std::vector<char> open(T, 1);
    peak_of.assign(T, 0);
    std::vector<uint32_t> chain;
    for (uint32_t i = 0; i < T; ++i) {
        if (!open[i]) continue;
        if (tree.pts[i].new_density < density_threshold) {
            open[i] = 0;
            peak_of[i] = T;
            continue;
        }
        chain.assign(1, i);
        open[i] = 0;
        uint32_t c = densest[i];
        while (chain.back() != c) {
            if (!open[c]) break;
            chain.push_back(c);
            open[c] = 0;
            c = densest[c];
        }
        uint32_t root = (chain.back() == c) ? c : peak_of[c];
        for (uint32_t q : chain) peak_of[q] = root;
        auto ins = clumps.emplace(peak_of[i], Clump());
        if (ins.second) ins.first->second.peak_index = peak_of[i];
        auto &ind = ins.first->second.indices;
        ind.insert(ind.end(), chain.begin(), chain.end());
    }
    std::vector<uint32_t> del;
    for (auto &it : clumps) {
        sort_particles(it.second);
        if (clump_diffuse_threshold < 0.525 && dispersion_too_large(it.second, clump_diffuse_threshold)) del.push_back(it.first);
    }
    if (clump_diffuse_threshold < 0.525) for (auto k : del) clumps.erase(k);
    del.clear();
    if (enough_particle_resolution == 0) remove_small_and_low();
    num_planetesimals = (uint32_t)clumps.size();
    stats.naive_peaks = num_planetesimals;

    phase_mark("hop");
    // 4. merge sweeps, src/tree.hpp:3863-4152
    Tree ct;
    for (int sweep_kind = 0; sweep_kind < 2; ++sweep_kind) {
        const bool hill_mode = sweep_kind == 1;
        double max_radius = 0.;
        if (hill_mode) for (auto &it : clumps) hill(it.second);
        std::vector<uint32_t> to_delete(num_planetesimals, 0);
        uint32_t delete_count = 0;
        bool merged = true;
        while (merged) {
            build_clump_tree(ct, max_radius, hill_mode);
            (hill_mode ? stats.sweeps_b : stats.sweeps_a)++;
            merged = false;
            std::vector<std::pair<uint32_t, uint32_t>> pairs;  // (predator key, prey key)
            std::vector<uint32_t> near;
            for (auto it1 = clumps.begin(); it1 != clumps.end(); ++it1) {
                Clump &c1 = it1->second;
                double r1 = hill_mode ? c1.Hill_radius * Hill_fraction_for_merge : c1.one10th_radius;
                if (!c1.mask) continue;
                if (ct.pts.empty()) continue;
                ct.ball(c1.center_of_mass, r1 + max_radius, near);
                for (uint32_t idx : near) {
                    uint32_t id2 = (uint32_t)ct.pts[idx].ath_density;
                    if (id2 == it1->first) continue;
                    auto it2 = clumps.find(id2);
                    if (it2 == clumps.end()) {
                        std::fprintf(stderr, "Error: Cannot find a clump with peak_id=%u. This should not happen. Please report a bug. Proceed for now.\n", id2);
                        continue;
                    }
                    Clump &c2 = it2->second;
                    if (!c2.mask) continue;
                    double r2 = hill_mode ? c2.Hill_radius * Hill_fraction_for_merge : c2.one10th_radius;
                    double dist = norm(sub(c1.center_of_mass, c2.center_of_mass));
                    bool eat = false;
                    if (dist < std::max(r1, r2)) eat = true;
                    else if (dist < (r1 + r2) && bound(c1, c2) && !saddle_deep(c1, c2, hill_mode)) eat = true;
                    if (eat) {
                        c2.mask = false;
                        pairs.emplace_back(it1->first, id2);
                        to_delete[delete_count++] = id2;
                    }
                }
            }
            if (!pairs.empty()) merged = true;
            if (std::getenv("PLAN_DEBUG_MERGES"))
                for (auto &pr : pairs) std::fprintf(stderr, "merge kind %d pred %u prey %u\n", sweep_kind, pr.first, pr.second);
            // predators in key order, each eating its preys in ball-search order
            for (size_t k = 0; k < pairs.size(); ++k) {
                Clump &pred = clumps[pairs[k].first];
                merge(pred, clumps[pairs[k].second]);
                if (hill_mode) hill(pred);
            }
            for (auto &it : clumps) {
                if (it.second.mask && dispersion_too_large(it.second)) {
                    it.second.mask = false;
                    to_delete[delete_count++] = it.first;
                }
            }
            num_planetesimals = (uint32_t)clumps.size() - delete_count;
        }
        for (auto k : to_delete) {
            if (k == 0 && clumps.count(0) && std::count(to_delete.begin(), to_delete.begin() + delete_count, 0u) == 0) stats.zero_key_quirk++;
            clumps.erase(k);
        }
        (hill_mode ? stats.after_merge_b : stats.after_merge_a) = (uint32_t)clumps.size();
    }
    // re-key to the densest sub-peak, src/tree.hpp:4156-4182
    std::vector<uint32_t> old_keys, new_keys;
    if (std::getenv("PLAN_DEBUG_MERGES"))
        for (auto &it : clumps) {
            std::fprintf(stderr, "clump %u peak %u subs", it.first, it.second.peak_index);
            for (uint32_t o : it.second.potential_subpeak_indices) std::fprintf(stderr, " %u", o);
            std::fprintf(stderr, "\n");
        }
    for (auto &it : clumps) {
        uint32_t k = it.first;
        for (uint32_t o : it.second.potential_subpeak_indices)
            if (tree.pts[k].new_density < tree.pts[o].new_density) k = o;
        if (k != it.first) { old_keys.push_back(it.first); new_keys.push_back(k); }
    }
    for (size_t i = 0; i < old_keys.size(); ++i) {
        auto ins = clumps.emplace(new_keys[i], Clump());
        if (ins.second) {
            auto orig = clumps.find(old_keys[i]);
            std::swap(orig->second, ins.first->second);
            ins.first->second.potential_subpeak_indices.push_back(orig->first);
            clumps.erase(orig);
        } else {
            std::fprintf(stderr, "Real peak index replacing failed. \n");
        }
    }
    phase_mark("merges+rekey");
    // 5. unbind and rebind, src/tree.hpp:4189-4208
    for (auto &it : clumps) {
        remove_unbound(it.second);
        hill(it.second);
    }
    for (auto &it : clumps) for (uint32_t i : it.second.indices) tree.pts[i].in_clump_flag = true;
    for (auto &it : clumps) {
        size_t before;
        do {
            before = it.second.indices.size();
            search_bound_in_hill(it.second);
            hill(it.second);
        } while (it.second.indices.size() > before);
    }
    phase_mark("unbind+rebind");
    // 6. prune, src/tree.hpp:4213-4224
    remove_small_and_low();
    for (auto &it : clumps)
        if (it.second.mask && dispersion_too_large(it.second, std::min(clump_diffuse_threshold + 0.1, 0.475))) del.push_back(it.first);
    for (auto k : del) clumps.erase(k);
    del.clear();
    // 7. rip the envelope, src/tree.hpp:4229-4248
    for (auto &it : clumps) {
        Clump &c = it.second;
        while (c.Hill_radius < c.particles.back().second) {
            auto low = std::lower_bound(c.particles.begin(), c.particles.end(), std::pair<uint32_t, double>(0, c.Hill_radius),
                                        [](const std::pair<uint32_t, double> &a, const std::pair<uint32_t, double> &b) { return a.second < b.second; });
            c.particles.resize(low - c.particles.begin());
            c.indices.resize(c.particles.size());
            if (c.indices.empty()) { del.push_back(it.first); break; }
            kinematics(c);
            remove_unbound(c);
            hill(c);
        }
    }
    for (auto k : del) clumps.erase(k);
    del.clear();
    // 8-9. prune again; drop ghost clumps, src/tree.hpp:4253-4266
    remove_small_and_low();
    for (auto &it : clumps) {
        const V3 &c = it.second.center_of_mass;
        bool in = true;
        for (int d = 0; d < 3; ++d) in = in && (c[d] >= p.box_min[d] && c[d] <= p.box_max[d]);
        if (!in) del.push_back(it.first);
    }
    for (auto k : del) clumps.erase(k);
    del.clear();
    num_planetesimals = (uint32_t)clumps.size();
    std::ostringstream out;
    // the reference formats this line on a stream it shares with WriteBasicResults, which
    // leaves it in scientific notation after the first snapshot (src/tree.hpp:4322, 4943)
    if (stream_scientific) out << std::scientific;
    out << "Finish clump finding for t = " << time << ", ";
    phase_mark("prune+rip+ghost");
    // 10. angular momentum and ranking, src/tree.hpp:4273-4326
    for (auto &it : clumps) angular_momentum(it.second);
    if (num_planetesimals > 0) {
        for (auto &it : clumps) peaks_and_masses.emplace_back(it.first, it.second.total_mass);
        std::sort(peaks_and_masses.begin(), peaks_and_masses.end(), [](const std::pair<uint32_t, double> &a, const std::pair<uint32_t, double> &b) {
            if (a.second == b.second) return a.first < b.first;
            return a.second < b.second;
        });
        if (p.num_peaks > 0 && num_planetesimals > p.num_peaks) {
            size_t drop = num_planetesimals - p.num_peaks;
            for (size_t k = 0; k < drop; ++k) clumps.erase(peaks_and_masses[k].first);
            peaks_and_masses.erase(peaks_and_masses.begin(), peaks_and_masses.begin() + drop);
            num_planetesimals = (uint32_t)clumps.size();
        }
        double tot = 0.;
        for (auto &pm : peaks_and_masses) tot = tot + pm.second;
        out << "found " << num_planetesimals << " clumps; " << " Mp_max = " << peaks_and_masses.back().second << ", Mp_tot = " << tot << "("
            << std::fixed << tot / p.mass_total_code_units * 100 << "%) in code units.";
    } else {
        out << "found zero clumps";
    }
    stats.final_clumps = num_planetesimals;
    return out.str();
}

// ================================================================ outputs
std::string peaks_file_name(const std::string &out_path, double time) {  // src/tree.hpp:4961-4968
    std::ostringstream ts;
    ts << std::setprecision(3) << std::fixed << std::setw(7) << std::setfill('0') << time;
    size_t slash = out_path.find_last_of('/');
    if (slash != std::string::npos) return out_path.substr(0, slash) + "/peaks_at_" + ts.str() + ".txt";
    return "peaks_at_" + ts.str() + ".txt";
}

void write_peaks_file(const std::string &path, const Finder &f) {  // src/tree.hpp:5004-5149
    std::ofstream o(path);
    if (!o.is_open()) std::fprintf(stderr, "Error: Failed to open file %s due to %s\n", path.c_str(), std::strerror(errno));
    o << std::setw(12) << "#peak_id" << std::setw(12) << "Npar" << std::setw(24) << "total_mass" << std::setw(24) << "Hill_radius"
      << std::setw(24) << "center_of_mass[x]" << std::setw(24) << "center_of_mass[y]" << std::setw(24) << "center_of_mass[z]"
      << std::setw(24) << "vel_COM[x]" << std::setw(24) << "vel_COM[y]" << std::setw(24) << "vel_COM[z]"
      << std::setw(24) << "J[x]" << std::setw(24) << "J[y]" << std::setw(24) << "J[z]/(M R_H^2 Omega)"
      << std::setw(24) << "geo_mean_offset[x]" << std::setw(24) << "geo_mean_offset[y]" << std::setw(24) << "geo_mean_offset[z]"
      << std::setw(24) << "median_offset[x]" << std::setw(24) << "median_offset[y]" << std::setw(24) << "median_offset[z]" << std::endl;
    for (auto &pm : f.peaks_and_masses) {
        const Clump &c = f.clumps.at(pm.first);
        size_t npar = c.indices.size();
        for (uint32_t i : c.indices) {
            auto s = f.tree.sinks.find(i);
            if (s != f.tree.sinks.end()) npar += s->second.size() - 1;
        }
        std::vector<std::vector<double>> off(3, std::vector<double>(npar));
        size_t k = 0;
        for (uint32_t i : c.indices) {
            auto s = f.tree.sinks.find(i);
            if (s != f.tree.sinks.end()) {
                for (auto &m : s->second) { for (int d = 0; d < 3; ++d) off[d][k] = m.pos[d] - c.center_of_mass[d]; ++k; }
            } else {
                for (int d = 0; d < 3; ++d) off[d][k] = f.tree.pts[i].pos[d] - c.center_of_mass[d];
                ++k;
            }
        }
        V3 J = c.J;
        double theta = std::acos(c.J[2] / norm(J));
        double phi = std::atan2(c.J[1], c.J[0]);
        double rz[3][3] = {{std::cos(phi), -std::sin(phi), 0}, {std::sin(phi), std::cos(phi), 0}, {0, 0, 1}};
        double ry[3][3] = {{std::cos(theta), 0, std::sin(theta)}, {0, 1, 0}, {-std::sin(theta), 0, std::cos(theta)}};
        double rot[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                rot[a][b] = 0;
                for (int d = 0; d < 3; ++d) rot[a][b] += rz[a][d] * ry[d][b];
            }
        for (size_t q = 0; q < npar; ++q) {
            double t[3] = {off[0][q], off[1][q], off[2][q]};
            for (int d = 0; d < 3; ++d) {
                off[d][q] = 0;
                for (int a = 0; a < 3; ++a) off[d][q] += t[a] * rot[a][d];
            }
        }
        V3 geo, med;
        size_t half = npar / 2;
        bool even = !(npar & 1);
        for (int d = 0; d < 3; ++d) {
            for (auto &v : off[d]) v = std::abs(v);
            double acc = 0.;
            for (double v : off[d]) acc = (v < 1e-32) ? acc - 32 : acc + std::log10(v);
            geo[d] = std::pow(10.0, acc / npar);
            std::nth_element(off[d].begin(), off[d].begin() + half, off[d].end());
            med[d] = off[d][half];
            if (even) med[d] = (med[d] + *std::max_element(off[d].begin(), off[d].begin() + half)) / 2.0;
        }
        o << std::setw(12) << pm.first << std::setw(12) << npar << std::setprecision(16) << std::setw(24) << c.total_mass
          << std::setw(24) << c.Hill_radius << std::setw(24) << c.center_of_mass[0] << std::setw(24) << c.center_of_mass[1]
          << std::setw(24) << c.center_of_mass[2] << std::setw(24) << c.vel_com[0] << std::setw(24) << c.vel_com[1]
          << std::setw(24) << c.vel_com[2] << std::setw(24) << c.J[0] << std::setw(24) << c.J[1] << std::setw(24) << c.J[2]
          << std::setw(24) << geo[0] << std::setw(24) << geo[1] << std::setw(24) << geo[2] << std::setw(24) << med[0]
          << std::setw(24) << med[1] << std::setw(24) << med[2] << std::endl;
    }
}

std::string basic_results_header() {  // src/tree.hpp:4936-4940
    std::ostringstream o;
    const int w = 15;
    o << std::setw(w) << std::setfill(' ') << "#time" << std::setw(w) << "N_peak" << std::setw(w) << "M_p,max,code" << std::setw(w)
      << "M_p,tot,code" << std::setw(w) << "M_p,max,frac" << std::setw(w) << "M_p,tot,frac" << std::setw(w) << "M_p,max,Ceres"
      << std::setw(w) << "M_p,tot,Ceres" << std::endl;
    return o.str();
}

std::string basic_results_line(const Finder &f, const Params &p, double time) {  // src/tree.hpp:4942-4951
    std::ostringstream o;
    const int w = 15;
    double mx = 0, tot = 0;
    for (auto &it : f.clumps) {
        mx = std::max(mx, it.second.total_mass);
        tot += it.second.total_mass;
    }
    o << std::setw(w) << std::setfill(' ') << std::scientific << time;
    o << std::setw(w) << f.num_planetesimals;
    o << std::setw(w) << mx << std::setw(w) << tot;
    o << std::setw(w) << mx / p.mass_total_code_units << std::setw(w) << tot / p.mass_total_code_units;
    o << std::setw(w) << mx * p.mass_physical / p.mass_ceres << std::setw(w) << tot * p.mass_physical / p.mass_ceres;
    o << std::endl;
    return o.str();
}

void write_parlists(const std::string &dir, const Finder &f, uint32_t sampling) {  // src/tree.hpp:5191-5222
    mkdir(dir.c_str(), 0755);
    for (auto &pm : f.peaks_and_masses) {
        const Clump &c = f.clumps.at(pm.first);
        std::ofstream o(dir + "/" + std::to_string(pm.first) + ".txt");
        uint32_t skip = 0;
        for (auto &q : c.particles) {
            if (skip > 0) { skip--; continue; }
            skip = sampling - 1;
            const TreePoint &t = f.tree.pts[q.first];
            o.unsetf(std::ios_base::floatfield);
            o << std::setw(16) << t.original_id;
            o << std::scientific;
            for (int i = 0; i < 3; ++i) o << std::setprecision(16) << std::setw(24) << t.pos[i];
            for (int i = 0; i < 3; ++i) o << std::setprecision(16) << std::setw(24) << t.vel[i];
            o << std::setprecision(16) << std::setw(24) << t.mass << std::endl;
        }
    }
}

}  // namespace orc

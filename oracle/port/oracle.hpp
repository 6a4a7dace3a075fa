// CPU restatement of PLAN's clump-finding path (test infrastructure, not the product).
//
// This is the project's own re-statement of the reference algorithm, written to reproduce the
// reference's results bit for bit on the same input: every floating-point expression keeps the
// reference's operation order, the same libstdc++ algorithms decide ties (std::sort,
// std::push_heap/pop_heap/sort_heap, std::map order), and it must be compiled with
// -ffp-contract=off. Only tests/, bench.py's CPU-baseline leg and __graft_entry__.smoke()
// may use it; the GPU product never links it.
//
// Parity is pinned against the unmodified reference compiled here (oracle/ref) on generated
// snapshots; see tests/golden/make_golden.py. Reference citations are path:line within the
// reference project.
#pragma once

#include <array>
#include <cstdint>
#include <map>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

namespace orc {

// ---------------------------------------------------------------- vectors
struct V3 {
    double x[3] = {0, 0, 0};
    V3() = default;
    V3(double a, double b, double c) { x[0] = a; x[1] = b; x[2] = c; }
    double &operator[](int i) { return x[i]; }
    double operator[](int i) const { return x[i]; }
};
// Elementwise helpers with the evaluation order of SmallVec (src/global.hpp:418-424, 487-640).
inline V3 sub(const V3 &a, const V3 &b) { return V3(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
inline V3 add(const V3 &a, const V3 &b) { return V3(a[0] + b[0], a[1] + b[1], a[2] + b[2]); }
inline V3 mul(const V3 &a, double s) { return V3(a[0] * s, a[1] * s, a[2] * s); }
inline V3 mul(double s, const V3 &a) { return V3(s * a[0], s * a[1], s * a[2]); }
inline V3 div(const V3 &a, double s) { return V3(a[0] / s, a[1] / s, a[2] / s); }
inline double norm2(const V3 &a) {
    double s = 0;
    s += a[0] * a[0];
    s += a[1] * a[1];
    s += a[2] * a[2];
    return s;
}
double norm(const V3 &a);

// ---------------------------------------------------------------- parameters
// NumericalParameters (src/global.hpp:676-874) and its derivation (src/global.cpp:28-47).
struct Params {
    V3 box_center{0, 0, 0}, box_length{0.2, 0.2, 0.2}, box_min{-0.1, -0.1, -0.1}, box_max{0.1, 0.1, 0.1};
    V3 box_half_width{0.1, 0.1, 0.1};
    double max_half_width = 0.1;
    unsigned box_resolution[3] = {128, 128, 128};
    V3 cell_length{0.0015625, 0.0015625, 0.0015625};
    double cell_volume = 0.0015625 * 0.0015625 * 0.0015625;
    V3 ghost_zone_width{0.025, 0.025, 0.025};
    double max_ghost_zone_width = 0.025;
    double q = 1.5, Omega = 1.0;
    V3 shear_vector{0.0, 1.5, 0.0};
    double rho_g0 = 1.0, solid_to_gas_ratio = 0.02;
    std::vector<double> mass_fraction_per_species{1.0};
    std::vector<double> mass_per_particle;
    double mass_total_code_units = 0.0020053;
    double PI = 3.14159265358979323846;
    double four_PI = 4. * 3.14159265358979323846;
    double four_PI_over_three = 3.14159265358979323846 * 4. / 3.;
    double four_PI_G = 0.05;
    double G_tilde = 0.05;
    double mass_ceres = 9.4e20;
    double mass_physical = (0.05 / 0.1) * 1.3e24;
    double grav_constant = 0.05 / (4. * 3.14159265358979323846);
    double shear_speed = 1.5 * 1.0 * 0.2;
    unsigned knn = 64, hop = 32;
    bool fixed_hop = false;
    unsigned num_threads = 0;
    unsigned num_peaks = 0;
    double clump_diffuse_threshold = -1.0, Hill_fraction_for_merge = -1.0;
    double min_trusted_mass = 2.87621e-6;
    // -x/-y/-z user box (progIO->user_box_min/max and flags.user_defined_box_flag,
    // src/global.cpp:398-440)
    bool user_box = false;
    V3 user_box_min{0, 0, 0}, user_box_max{0, 0, 0};

    void derive();  // CalculateNewParameters, src/global.cpp:28-47
};

// Parameter file reader (src/global.cpp:51-225). Returns 0, 3 (cannot open) or 4 (bad value).
int read_param_file(const std::string &path, Params &p);

// ---------------------------------------------------------------- particles
struct Particle {  // src/tree.hpp:1155-1198
    V3 pos, vel;
    double density = 0;
    uint32_t id_in_run = 0, id = 0;
    int property_index = 0;
    uint16_t cpu_id = 0;
};

struct Snapshot {
    double coor_lim[12] = {0};
    std::vector<double> type_info;
    double time = 0, dt = 0;
    uint32_t num_particles = 0;
    std::vector<Particle> parts;
};

// ReadSingleLisFile / ReadMultipleLisFile (src/tree.hpp:1303-1535). Returns 0 or 3.
int read_lis_files(const std::vector<std::string> &files, Snapshot &s);
// Sort by (cpu_id, id_in_run), number, and on the first file set the box and masses
// (src/tree.hpp:1540-1583).
void finish_read(Snapshot &s, Params &p, bool first_file);
// MakeGhostParticles (src/tree.hpp:1626-1754).
void make_ghosts(Snapshot &s, const Params &p);

// ---------------------------------------------------------------- tree
struct TreePoint {  // BHtree::InternalParticle, src/tree.hpp:2367-2410
    V3 pos, vel;
    double mass = 0, ath_density = 0, new_density = 0;
    uint32_t original_id = 0;
    bool sink_flag = false, in_clump_flag = false;
};

struct Node {  // BHtree::TreeNode, src/tree.hpp:2419-2455
    V3 center;
    double half_width = 0;
    uint32_t begin = 0, end = 0, parent = 0, first_daughter = 0;
    uint16_t orthant = 0;
    uint8_t num_daughters = 0, level = 0;
};

using Key = unsigned __int128;
using Heap = std::vector<std::pair<int, double>>;

struct Tree {
    std::vector<TreePoint> pts;
    std::vector<Node> nodes;
    std::unordered_map<uint32_t, std::vector<TreePoint>> sinks;
    V3 root_center;
    double half_width = 0;
    double epsilon = 1. / 4294967296.;
    V3 boxmin, scale;
    V3 cell_length, half_cell_length, cell_length_squared, three_half_cell_length;
    uint64_t check_outside = 0;  // points found outside their node by the tree check
    uint32_t max_leaf_size = 8;  // BHtree::max_leaf_size (64 under --Density_Vs_Scale)

    // BuildTree (src/tree.hpp:2759-2908). `parts` is consumed.
    void build(Params &p, std::vector<Particle> &parts, bool check_pos);
    Key morton(const V3 &pos, uint32_t index) const;
    uint32_t size() const { return (uint32_t)pts.size(); }
    bool within(const V3 &pos, const V3 &c, double hw) const;
    uint32_t pos2node(const V3 &pos) const;
    bool sphere_contains(const V3 &c, double r, uint32_t node) const;
    bool sphere_intersects(const V3 &c, double r, uint32_t node) const;
    // KNN_Search_OpenMP (src/tree.hpp:3198-3251): heap sorted ascending on return.
    // false when the position has no leaf in the tree (the reference then reports "Key2Leaf:
    // leaf cell doesn't exist in tree" and continues with an invalid node, src/tree.hpp:2983-2987)
    bool knn(const V3 &pos, unsigned k, Heap &heap, double estimated_distance = 0) const;
    // BallSearch / RecursiveBallSearchCount (src/tree.hpp:3255-3304).
    void ball(const V3 &c, double r, std::vector<uint32_t> &out) const;
    uint32_t ball_count(const V3 &c, double r) const;
    double quadratic_spline(V3 d) const;
    // RecursiveBallSearchCountWithShear (src/tree.hpp:3306-3402): points within r of c, the
    // nodes compared through their shearing-periodic image where far away
    uint32_t ball_count_sheared(const V3 &c, double r, const V3 &max_distance, double shear_distance, const Params &p) const;
};

// BasicAnalysesWithTree for --Density_Vs_Scale (src/analyses.hpp:196-333): the largest
// count of points within each search radius over the cell centres (and sub-centres for the
// three smallest radii), as a density. `header` is the first snapshot's header line.
struct DensityVsScale {
    std::vector<double> radii, max_rhop;
    std::string header, line;
};
DensityVsScale density_vs_scale(const Tree &t, const Params &p, double time);

// ---------------------------------------------------------------- clumps
struct Clump {  // Planetesimal, src/tree.hpp:4351-4809
    uint32_t peak_index = 0;
    std::vector<uint32_t> potential_subpeak_indices;
    std::vector<uint32_t> indices;
    bool mask = true;
    double total_mass = 0;
    V3 center_of_mass, vel_com;
    std::vector<std::pair<uint32_t, double>> particles;
    double outer_one10th_radius = 0, inner_one10th_radius = 0, one10th_radius = 0;
    double two_sigma_mass_radius = 0, Hill_radius = 0;
    V3 J;
};

// Which x^1.5 and x^(1/3.) to use: the host libm (as the reference) or the project's
// correctly rounded double-double versions (as the GPU path).
enum PowMode { POW_LIBM = 0, POW_CORRECT = 1 };

struct Stats {
    uint32_t naive_peaks = 0, after_merge_a = 0, after_merge_b = 0, final_clumps = 0;
    uint32_t sweeps_a = 0, sweeps_b = 0;
    uint64_t zero_key_quirk = 0;
};

// Acceptance-step statistics of the Hill rebinding (a study mode, PLAN_ORACLE_WINDOW_STATS=1):
// each call's candidate sequence replayed with the reference's test and update under several
// ways a device can step through it (kWindowSchemes; see Finder::count_windows).
constexpr int kWindowSchemes = 5;
struct WindowStats {
    uint64_t calls = 0, candidates = 0, accepted = 0;
    uint64_t steps[kWindowSchemes] = {0};          // over every call
    uint64_t longest_call[kWindowSchemes] = {0};   // the most steps one call takes
    uint64_t mismatch_windows = 0, disagreements = 0;  // windows cut short; calls whose result differed (must be 0)
    uint64_t accepted_per_window[33] = {0};
    struct PerClump {
        uint64_t accepted = 0, steps[kWindowSchemes] = {0};
        uint64_t busy_windows = 0;  // speculative windows (scheme 3) that accept at least one candidate
        uint64_t calls = 0, grown_members = 0;  // calls; members summed over the calls that grew (re-sorted after each)
        // per call: accepted, steps of schemes 0 and 3, busy windows (for the round model)
        std::vector<std::array<uint64_t, 4>> call;
    };
    std::map<uint32_t, PerClump> per_clump;  // by peak, over all the clump's calls
};

struct Finder {
    Params *par = nullptr;
    Tree tree;
    std::map<uint32_t, Clump> clumps;
    std::vector<std::pair<uint32_t, double>> peaks_and_masses;
    double density_threshold = 0, clump_mass_threshold = 0, peak_density_threshold = 0;
    double clump_diffuse_threshold = 0.55, Hill_fraction_for_merge = 0.25;
    uint32_t num_planetesimals = 0;
    int enough_particle_resolution = 0;
    bool median_kernel = true;
    PowMode pow_mode = POW_LIBM;
    int threads = 1;
    // Stage dumps (filled while running).
    std::vector<uint32_t> densest;   // densest-neighbour pointer per tree point
    std::vector<uint32_t> peak_of;   // HOP root per tree point (size() = ignored)
    Stats stats;
    // per snapshot
    uint32_t num_input_particles = 0;
    double time = 0;

    // FindPlanetesimals (src/tree.hpp:3576-4339). Returns the summary line.
    std::string find(uint32_t num_particles_in);
    bool stream_scientific = false;  // the summary stream's state after an earlier snapshot
    double density_kernel(const Heap &heap, uint32_t self, unsigned k) const;
    double pow15(double x) const;
    double hill_pow(double x) const;

    // clump helpers (src/tree.hpp:4431-4747, 4867-4909, 5251-5284)
    void kinematics(Clump &c) const;
    void sort_particles(Clump &c) const;
    void one10th(Clump &c) const;
    bool dispersion_too_large(const Clump &c, double tol = 0.55) const;
    void merge(Clump &pred, Clump &prey) const;
    void remove_unbound(Clump &c) const;
    void search_bound_in_hill(Clump &c);
    void search_bound_in_hill_loop(Clump &c, const std::vector<uint32_t> &near);
    bool window_stats_on = false;
    WindowStats window_stats;
    void count_windows(const Clump &c, const std::vector<uint32_t> &near);
    void hill(Clump &c) const;
    void angular_momentum(Clump &c) const;
    bool bound(const Clump &a, const Clump &b) const;
    bool saddle_deep(const Clump &a, const Clump &b, bool hill_mode) const;
    void remove_small_and_low();
    void build_clump_tree(Tree &ct, double &max_radius, bool hill_mode);
};

// ---------------------------------------------------------------- outputs
// OutputPlanetesimalsInfo (src/tree.hpp:4958-5150) and WriteBasicResults (4935-4953).
std::string peaks_file_name(const std::string &out_path, double time);
void write_peaks_file(const std::string &path, const Finder &f);
std::string basic_results_header();
std::string basic_results_line(const Finder &f, const Params &p, double time);
void write_parlists(const std::string &dir, const Finder &f, uint32_t sampling);

// Correctly rounded x^1.5 and x^(1/3.) (double-double evaluation), shared with the GPU
// path's host-side tests.
double cr_pow15(double x);
double cr_pow_third(double x);

}  // namespace orc

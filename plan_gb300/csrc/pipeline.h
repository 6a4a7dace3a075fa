// Internal device layout and stage entry points of the clump finder.
//
// HBM layout of one snapshot (T = tree points incl. ghosts, Tu = after sink folding):
//   input order  in_pos/in_vel double4_32a[T] (x,y,z,mass | vx,vy,vz,ath_density), in_type
//   keys         kw0..kw2 + kidx u32[T]  (sorted in place)
//   tree points  pos double4_32a[Tu] (x,y,z,mass), vel double4_32a[Tu] (vx,vy,vz,ath_density),
//                dens f64[Tu], orig u32[Tu], tk0..tk2 u32[Tu], sink_n u32[Tu],
//                sink_first u32[Tu] (first sorted slot of the folded run), leaf_of u32[Tu]
//   nodes        ncf double4_32a[nodes] (center, half_width), nbeg/nend/npar/nfd u32,
//                nnd/north/nlev u8
// Everything lives in one arena per context, bump-allocated per snapshot.
#pragma once

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "common.cuh"
#include "plan_gpu.h"
#include "spline.cuh"

namespace plan {

struct Arena {
    char *base = nullptr;
    size_t cap = 0, used = 0, peak = 0;
    bool failed = false;
    void *take(size_t bytes) {
        size_t off = (used + 255) & ~size_t(255);
        if (off + bytes > cap) { failed = true; return nullptr; }
        used = off + bytes;
        if (used > peak) peak = used;
        return base + off;
    }
    template <class T> T *get(size_t n) { return static_cast<T *>(take(n * sizeof(T))); }
};

struct TreeBox {
    double root_center[3];
    double half_width;
    double epsilon;
    double boxmin[3];
    double scale[3];
};

struct DevTree {
    uint32_t T = 0, Tu = 0, nodes = 0, nsinks = 0;
    uint32_t leaf_size = 8;  // max_leaf_size it was built with (64 for --Density_Vs_Scale)
    TreeBox box;
    double4_32a *pos = nullptr, *vel = nullptr;
    double *dens = nullptr;
    uint32_t *orig = nullptr, *tk0 = nullptr, *tk1 = nullptr, *tk2 = nullptr;
    uint32_t *sink_n = nullptr, *sink_first = nullptr, *leaf_of = nullptr;
    uint32_t *sorted_src = nullptr;  // kidx after the Morton sort: input index per sorted slot
    double4_32a *in_pos = nullptr, *in_vel = nullptr;  // input order (for sink members)
    double4_32a *ncf = nullptr;
    uint32_t *nbeg = nullptr, *nend = nullptr, *npar = nullptr, *nfd = nullptr;
    uint8_t *nnd = nullptr, *north = nullptr, *nlev = nullptr;
    float4 *phi = nullptr, *plo = nullptr, *nhi = nullptr, *nlo = nullptr;  // FP32 hi/lo copies
};

// Host-visible scalars of a finder run.
struct FindScalars {
    double density_threshold, peak_density_threshold, clump_mass_threshold;
    double clump_diffuse_threshold, Hill_fraction_for_merge;
    uint32_t knn, hop;
    int median_kernel;    // 0: the spline kernel (fewer than 4 particles per horizontal cell)
    SplineCells spline;   // its cell constants
};

struct Context {
    int device = 0;
    cudaStream_t stream = nullptr;
    Arena arena;           // per-snapshot buffers
    Arena scratch;         // temporary buffers (sorts, scans) reused within a stage
    DevTree tree;
    unsigned *d_err = nullptr;      // device error flags
    uint64_t launches = 0;
    double stage_ms[32] = {0};
    uint64_t counters[32] = {0};
    std::string last_error;
    // host copies kept for the catalogue
    uint32_t n_input = 0;
    double time = 0;
    FindScalars fs{};
    uint32_t *densest = nullptr, *peak = nullptr;  // stage arrays of the last finder run
    cudaEvent_t kev[2] = {nullptr, nullptr};        // brackets one kernel for its timing
    void *noalloc_scratch = nullptr;                // this device's fixed array (plan_morton_order_noalloc)
    int status_from(int rc, const char *what);
    // grow an arena (contents are discarded) to at least `bytes`
    int ensure(Arena &a, size_t bytes);
};

extern thread_local Context *g_ctx;  // for set_cuda_error messages

// Stage 1: upload + unpack + (cpu_id, id_in_run) order + ghosts + keys + sort + sinks + tree.
int build_tree(Context &c, const plan_lis_view &v, plan_params &p, int first_file, cudaStream_t s);
// Keys, sort, sinks and octree for points in input order (pos.w = mass unless a mass
// table is given); used for the particle tree and the clump trees.
int build_octree(Context &c, double4_32a *in_pos, double4_32a *in_vel, const uint32_t *in_type, uint32_t T, const TreeBox &box,
                 const double *mass_table, uint32_t ntypes, DevTree &tr, cudaStream_t s, cudaEvent_t after_sort, uint32_t leaf = 8);
TreeBox make_box(const double center[3], double half_width);
// Stage 2: densities, densest neighbours, HOP groups, clump stage -> host catalogue.
int find_planetesimals(Context &c, plan_params &p, cudaStream_t s, plan_catalogue **out);
// --Density_Vs_Scale on the current tree (dvs.cu): the search radii and the densest sphere
// of each, as BasicAnalysesWithTree reports them.
int density_vs_scale(Context &c, const plan_params &p, double time, std::vector<double> &radii, std::vector<double> &rho, cudaStream_t s);
// Kinetic and pairwise potential energy of particle groups (energy.cu).
int group_energies(Context &c, const float *pos3, const float *vel3, const float *mass, const uint64_t *offsets, uint32_t ngroups, double G,
                   double shear_y, double *e_kin, double *e_pot, uint64_t *zero_pairs, cudaStream_t s);
// --Save_Clumps member lists of a catalogue, formatted on the device (parlist.cu).
int write_parlists_device(Context &c, const plan_catalogue &cat, int file_number, uint32_t sampling, cudaStream_t s);
// KNN queries at arbitrary positions on the current tree (inspection / tests).
int knn_positions(Context &c, const double *pos3, uint32_t nq, uint32_t k, double est, uint32_t *idx, double *dr2);

// Kernel launch helpers shared across translation units
int launch_density(Context &c, const plan_params &p, uint32_t k, cudaStream_t s);
int launch_densest(Context &c, const plan_params &p, uint32_t k, double threshold, uint32_t *densest, cudaStream_t s);

// Device bytes kept per tree point over a snapshot (tree, nodes, HOP and clump buffers),
// and the scratch bytes per input particle; used for sizing and for admission.
constexpr uint64_t kArenaBytesPerTreePoint = 512;
constexpr uint64_t kScratchBytesPerParticle = 160;
// Room for the clump stage's member pool beyond that: a larger pool means fewer compactions
// (and fewer relaunches) while the rebinding loop writes fresh segments. Capped so that the
// largest snapshots still fit the device.
constexpr uint64_t kPoolBytesPerTreePoint = 800;
constexpr uint64_t kPoolBytesMax = 24ull << 30;

// The snapshot arena for T tree points.
inline uint64_t arena_bytes_for(uint64_t T) {
    const uint64_t pool = T * kPoolBytesPerTreePoint < kPoolBytesMax ? T * kPoolBytesPerTreePoint : kPoolBytesMax;
    return T * kArenaBytesPerTreePoint + pool + (64ull << 20);
}

inline unsigned grid_for(size_t n, int threads) {
    size_t b = (n + threads - 1) / threads;
    return (unsigned)(b ? b : 1);
}

}  // namespace plan

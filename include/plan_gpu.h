/* plan_gpu — GB300 (sm_103a) clump finder with PLAN's find-clumps interface.
 *
 * C ABI only: plain pointers, sizes and status codes; no C++ or framework types cross it.
 * The reference program has no plugin or FFI surface: its boundary is the process
 * (command line, parameter file, .lis input, text catalogues) and, inside, the two calls
 * main() makes per snapshot. Each entry point below names the reference interface it
 * replaces (path:line in the reference project).
 *
 * Conventions
 *   - Every call returns an int status: 0 ok, 2 argument, 3 I/O, 4 parameter, 5 CUDA,
 *     6 out of device memory / admission refused, 7 unsupported input, 8 device loop
 *     limit, 9 pending (plan_poll: the request is queued or running). The command-line
 *     front end maps 2/3/4 to the reference's exit codes.
 *   - Host buffers passed in are caller-owned and only read during the call. Device
 *     buffers are owned by the context and released by plan_ctx_destroy.
 *   - A context is bound to one device and is not thread-safe; use one per host thread.
 *   - There is no CPU fallback: without a usable CUDA device plan_ctx_create fails.
 */
#ifndef PLAN_GPU_H
#define PLAN_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PLAN_ABI_VERSION 1

#define PLAN_PENDING 9

typedef struct plan_ctx plan_ctx;
typedef struct plan_lis plan_lis;
typedef struct plan_server plan_server;
typedef struct plan_catalogue plan_catalogue;

/* NumericalParameters (src/global.hpp:676-874): the file-settable values, the reference's
 * fixed constants, and the box-derived values set from the first snapshot of a run
 * (src/tree.hpp:1564-1583, src/global.cpp:28-47). */
typedef struct plan_params {
    /* read from the parameter file */
    double solid_to_gas_ratio;      /* Z */
    uint32_t box_resolution[3];     /* Nx1..Nx3 */
    double four_pi_G;               /* four_pi_G_par */
    uint32_t num_threads;           /* num_threads / omp_threads (host side only) */
    uint32_t num_peaks;             /* num_peaks / num_peak: output cap, 0 = none */
    uint32_t knn;                   /* num_neighbors_in_knn_search / num_knn / knn */
    uint32_t hop;                   /* num_neighbors_to_hop / num_hop / hop */
    int32_t fixed_hop;              /* hop given in the file */
    double clump_diffuse_threshold; /* < 0: choose from resolution */
    double Hill_fraction_for_merge; /* < 0: choose from resolution */
    /* constants of the reference */
    double q, Omega, rho_g0;
    double ghost_zone_width[3];
    /* derived (plan_params_derive / first snapshot) */
    double box_min[3], box_max[3], box_center[3], box_length[3], box_half_width[3];
    double max_half_width, max_ghost_zone_width;
    double cell_length[3], cell_volume;
    double mass_total_code_units, G_tilde, mass_physical, grav_constant, shear_speed;
    double min_trusted_mass;
    uint32_t ntypes;
    double mass_per_particle[16];
    double mass_fraction_per_species[16];
    int32_t box_set;                /* box and masses taken from a first snapshot */
    /* command-line flags */
    int32_t no_ghost;               /* --No_Ghost */
    int32_t user_box;               /* -x/-y/-z given (src/global.cpp:398-440) */
    double user_box_min[3], user_box_max[3]; /* their limits, lo <= hi; 0,0 on an axis = the box's extent */
    int32_t density_vs_scale;       /* --Density_Vs_Scale: the tree is built as that analysis
                                       wants it (64-point leaves, no ghosts, ghost zone = box) */
} plan_params;

/* Defaults of NumericalParameters (src/global.hpp:686-862). */
void plan_params_init(plan_params *p);
/* NumericalParameters::ReadNumericalParameters (src/global.cpp:51-225). Returns 0, 3 or 4. */
int plan_params_read(const char *path, plan_params *p);
/* NumericalParameters::CalculateNewParameters (src/global.cpp:28-47). */
void plan_params_derive(plan_params *p);

/* ---------------------------------------------------------------- snapshot input */
/* ParticleSet::ReadSingleLisFile / ReadMultipleLisFile (src/tree.hpp:1303-1535): read one
 * combined file (nfiles = 1) or the per-processor files of one snapshot into page-locked
 * host memory. Truncated files are an I/O error (3), never read past their end. */
int plan_lis_read(const char *const *paths, int nfiles, plan_lis **out);
void plan_lis_free(plan_lis *lis);
uint64_t plan_lis_count(const plan_lis *lis);
double plan_lis_time(const plan_lis *lis);

/* A snapshot already in host memory: the parsed header and blocks of 44-byte records
 * (3 x f32 pos, 3 x f32 vel, f32 density, i32 type, i64 id_in_run, i32 cpu_id). */
typedef struct plan_lis_view {
    double coor_lim[12];
    uint32_t ntypes;
    double type_info[16];
    double time, dt;
    uint32_t nblocks;
    const void *const *records;
    const uint64_t *counts;
} plan_lis_view;
int plan_lis_get_view(const plan_lis *lis, plan_lis_view *view);

/* ---------------------------------------------------------------- device context */
int plan_ctx_create(int device, plan_ctx **out);
void plan_ctx_destroy(plan_ctx *ctx);
const char *plan_last_error(const plan_ctx *ctx);
/* Free the context's snapshot buffers (they grow back on the next snapshot); the stage
 * arrays of the last snapshot are gone afterwards. New, for the serving loop's admission. */
int plan_ctx_release(plan_ctx *ctx);
/* Device bytes a snapshot of n particles needs (the serving admission estimate). */
uint64_t plan_footprint_bytes(uint64_t n_particles, const plan_params *p);

/* ParticleSet::ReadLisFile tail + MakeGhostParticles + BHtree::BuildTree
 * (src/tree.hpp:1540-1754, 2759-2908; called at src/main.cpp:72-73): copy the records to
 * the device, sort them by (cpu_id, id_in_run), make shearing-periodic ghosts, build
 * Morton keys, sort, fold equal keys into sink particles and build the octree.
 * `first_file` != 0 sets the box and particle masses in *p as the reference does for the
 * first snapshot of a run. `stream` is a cudaStream_t (NULL = the context's stream). */
int plan_build_tree(plan_ctx *ctx, const plan_lis_view *snap, plan_params *p, int first_file, void *stream);

/* BHtree::FindPlanetesimals (src/tree.hpp:3576-4339; called at src/main.cpp:79): KNN
 * densities, densest neighbours, HOP groups, the two merge sweeps, unbinding, Hill
 * rebinding, pruning and angular momenta, all on the device. The result is a host-side
 * catalogue owned by the caller (plan_catalogue_free). */
int plan_find_planetesimals(plan_ctx *ctx, plan_params *p, void *stream, plan_catalogue **out);

/* Both of the above in one call. */
int plan_find_clumps(plan_ctx *ctx, const plan_lis_view *snap, plan_params *p, int first_file, void *stream, plan_catalogue **out);

/* ---------------------------------------------------------------- catalogue */
typedef struct plan_clump_info {
    uint32_t peak_id;          /* tree index of the peak particle (catalogue key) */
    uint32_t npar;             /* members, counting every particle of a sink */
    double total_mass, hill_radius;
    double com[3], vel_com[3], J[3];
} plan_clump_info;

void plan_catalogue_free(plan_catalogue *cat);
/* Clumps in output order (ascending mass, ties by peak id; src/tree.hpp:4293-4301). */
uint32_t plan_catalogue_count(const plan_catalogue *cat);
int plan_catalogue_get(const plan_catalogue *cat, uint32_t i, plan_clump_info *info);
/* The stdout summary line of FindPlanetesimals (src/tree.hpp:4269, 4320-4325). */
const char *plan_catalogue_summary(const plan_catalogue *cat);
/* PlanetesimalList::OutputPlanetesimalsInfo (src/tree.hpp:4958-5150): peaks_at_<time>.txt
 * next to out_path; with save_clumps also ParList.<NNNN>/<peak_id>.txt
 * (src/tree.hpp:5191-5222), NNNN = file_number, every `sampling`-th member. */
int plan_catalogue_write_peaks(const plan_catalogue *cat, const char *out_path, int save_clumps, int file_number, uint32_t sampling);
/* OutputSinglePlanetesimal (src/tree.hpp:5191-5222) for every clump of a catalogue, with
 * the lines formatted on the context's device: ParList.<NNNN>/<peak_id>.txt in the working
 * directory, byte-identical to the member lists plan_catalogue_write_peaks writes with
 * save_clumps (which formats them on the host). NNNN = file_number, every `sampling`-th member. */
int plan_catalogue_write_parlists(plan_ctx *ctx, const plan_catalogue *cat, int file_number, uint32_t sampling);
/* PlanetesimalList::WriteBasicResults (src/tree.hpp:4935-4953): the line for this snapshot
 * (with the header first when with_header != 0) into buf; returns the length or -1. */
int plan_catalogue_basic_results(const plan_catalogue *cat, const plan_params *p, int with_header, char *buf, size_t cap);

/* BasicAnalysesWithTree for --Density_Vs_Scale (src/analyses.hpp:196-333) on the tree of the
 * last plan_build_tree, which must have had p->density_vs_scale set (64-point leaves, no
 * ghosts): the search radii (half a cell times 1, 2, 4, ...) and, for each, the largest
 * count of points within that radius of a cell centre or sub-centre as a density
 * (count m / (4 pi / 3 r^3)). time = the snapshot's time (shear of the periodic images).
 * Writes up to cap values to radii and rho; *nlev = the number of radii. */
int plan_density_vs_scale(plan_ctx *ctx, const plan_params *p, double time, double *radii, double *rho, int cap, int *nlev);

/* Batched boundness (new, no counterpart in the reference): for each group g of particles
 * [offsets[g], offsets[g+1]) (float32 positions, velocities, masses),
 *   e_kin[g] = 1/2 sum m |v_c - s (x_c - x) - v|^2 with s = (0, q Omega, 0), the shear
 *              correction of the reference's boundness test (src/tree.hpp:4657-4659), and
 *   e_pot[g] = -G sum_{i<j} m_i m_j / r_ij (no softening; coincident pairs are left out and
 *              counted in *zero_pairs).
 * A group is bound when e_kin + e_pot < 0. All groups go through one persistent pass over
 * 128 x 128 pair tiles; row sums of m_j / r_ij are FP32 with compensation, the mass of the
 * row, the tile and group sums FP64.
 * G, q and Omega come from p. */
int plan_group_energies(plan_ctx *ctx, const float *pos3, const float *vel3, const float *mass, const uint64_t *offsets, uint32_t ngroups,
                        const plan_params *p, double *e_kin, double *e_pot, uint64_t *zero_pairs);

/* ---------------------------------------------------------------- serving
 * New, no counterpart in the reference (which processes its snapshot list one by one):
 * snapshots submitted from any thread run concurrently on one device, each on one of
 * `workers` contexts with its own stream and buffers. A request is admitted in arrival order
 * when a worker is free and the device footprints (plan_footprint_bytes) of the running
 * requests plus its own fit in `hbm_budget` bytes (0 = 90% of the device's free memory at
 * creation); when the oldest waiting request does not fit, later ones that fit may start
 * first, at most 2 x workers times before it. Workers keep their buffers between requests
 * and give them back (plan_ctx_release) when a waiting request needs the room. Each request
 * is computed exactly as plan_find_clumps computes it alone. */
int plan_server_create(int device, int workers, uint64_t hbm_budget, plan_server **out);
/* Waits for the running requests; queued ones are dropped. */
void plan_server_destroy(plan_server *srv);
/* Queue one snapshot (first_file as in plan_find_clumps; p is copied). The view's host
 * records must stay valid until plan_poll has returned the request. Status 6 when the
 * snapshot alone does not fit the budget. */
int plan_submit(plan_server *srv, const plan_lis_view *snap, const plan_params *p, int first_file, uint64_t *request);
/* The request's catalogue (caller frees) and its latency from submission to completion, in
 * milliseconds: 0 when done, PLAN_PENDING while queued or running (wait = 0; wait != 0
 * blocks until done), or the request's error status with its message in
 * plan_server_error. A request is returned once. */
int plan_poll(plan_server *srv, uint64_t request, int wait, plan_catalogue **out, double *latency_ms);
/* Message of the last failed request returned by plan_poll on this server (or of a refused
 * plan_submit), copied for the calling thread: valid until that thread calls this again. */
const char *plan_server_error(const plan_server *srv);
/* Largest sum of worker holds seen against the budget, and how many holds were given back. */
int plan_server_stats(const plan_server *srv, uint64_t *peak_held_bytes, uint64_t *releases);
/* Over the requests run so far, each from its start on a worker to its end: the time at least
 * one ran (busy_ms) and the time two or more ran at once on their workers' streams
 * (overlap_ms). No reference counterpart: it shows the workers' work overlapping. */
int plan_server_overlap(const plan_server *srv, double *busy_ms, double *overlap_ms);

/* ---------------------------------------------------------------- inspection
 * Stage arrays of the last snapshot, for parity tests and profiling. */
enum plan_stage_array {
    PLAN_ARR_TREE_POS = 1,      /* double[Tu][4]: x, y, z, mass of sorted tree points */
    PLAN_ARR_TREE_VEL = 2,      /* double[Tu][4]: vx, vy, vz, ath_density */
    PLAN_ARR_DENSITY = 3,       /* double[Tu]: new_density */
    PLAN_ARR_ORIG_ID = 4,       /* uint32[Tu]: original id (input order incl. ghosts) */
    PLAN_ARR_KEYS = 5,          /* uint32[Tu][3]: Morton keys, low word first */
    PLAN_ARR_NODE_F = 6,        /* double[nodes][4]: center xyz, half_width */
    PLAN_ARR_NODE_U = 7,        /* uint32[nodes][7]: begin, end, parent, first_daughter,
                                   orthant, num_daughters, level */
    PLAN_ARR_DENSEST = 8,       /* uint32[Tu]: densest-neighbour pointer */
    PLAN_ARR_PEAK = 9,          /* uint32[Tu]: HOP root (Tu for points below threshold) */
    PLAN_ARR_SINK_COUNT = 10,   /* uint32[Tu]: particles folded into each tree point */
};
/* Number of elements of a stage array (0 if not available). */
uint64_t plan_stage_count(const plan_ctx *ctx, int which);
/* Copy a stage array to host memory; bytes must be at least count * element size. */
int plan_stage_copy(plan_ctx *ctx, int which, void *host_dst, size_t bytes);
/* KNN_Search_OpenMP (src/tree.hpp:3198-3251) for arbitrary positions on the last tree:
 * k neighbours of each of nq positions (est = 0: the reference's own first radius), sorted
 * ascending as the reference returns them. */
int plan_knn(plan_ctx *ctx, const double *pos3, uint32_t nq, uint32_t k, double est, uint32_t *idx, double *dr2);
/* std::sort with AscendingMorton (src/tree.hpp:2269-2273, 2831) of n 96-bit keys given in
 * input order (3 x u32 each, low word first): order[i] receives the input index of the i-th
 * sorted key, with equal keys in the order the library's introsort leaves them. */
int plan_morton_order(plan_ctx *ctx, const uint32_t *keys3, uint32_t n, uint32_t *order);
/* plan_morton_order without any device allocation (no counterpart in the reference). The
 * keys and all sort scratch live in a fixed device array inside the library, sized for at
 * most PLAN_NOALLOC_SORT_MAX keys; larger n returns status 6 with a message. Nothing in the
 * array has to start at zero. Calls on the same device share the array, so they must not
 * overlap (one call at a time per device, across all contexts and threads). The first call
 * on a device looks the array up with cudaGetSymbolAddress: make it before any stream
 * capture on that device. */
#define PLAN_NOALLOC_SORT_MAX 65536u
int plan_morton_order_noalloc(plan_ctx *ctx, const uint32_t *keys3, uint32_t n, uint32_t *order);
/* Wall time per stage of the last snapshot in milliseconds (CUDA events):
 * [0] upload+unpack, [1] ghosts, [2] keys+sort, [3] tree, [4] density KNN, [5] HOP KNN,
 * [6] grouping, [7] clump stage, [8] catalogue download. */
int plan_stage_times(const plan_ctx *ctx, double *ms, int n);
/* Launch count of this library's kernels since the context was created. */
uint64_t plan_kernel_launches(const plan_ctx *ctx);
/* Counters of the last snapshot: [0] input N, [1] tree points T (with ghosts), [2] unique
 * tree points, [3] nodes, [4] sinks, [5] density-threshold points, [6] naive groups,
 * [7] final clumps, [8] KNN boundary ties, [9] device error flags. */
int plan_counters(const plan_ctx *ctx, uint64_t *out, int n);

#ifdef __cplusplus
}
#endif
#endif

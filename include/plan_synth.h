/* Synthetic Athena particle snapshots (.lis) for tests and benchmarks.
 *
 * The reference ships no data, so every workload is generated. The generator is
 * deterministic across hosts: it draws from a counter-based splitmix64 stream and uses only
 * IEEE +,-,*,/ and sqrt (its exp/log are series evaluations of its own), so the same spec
 * gives byte-identical files on x86-64 and aarch64.
 *
 * File layout written (read by the reference at src/tree.hpp:1434-1535):
 *   12 x f32 grid+domain limits, i32 ntypes, ntypes x f32 type_info, f32 time, f32 dt,
 *   i64 N, then N records of 44 B: 3 x f32 pos, 3 x f32 vel, f32 density, i32 type,
 *   i64 id_in_run, i32 cpu_id.
 * The per-particle density is the nearest-grid-point deposit count*m/V_cell on the
 * nx^3 grid, because the reference prunes clumps on it (src/tree.hpp:3533-3540).
 */
#ifndef PLAN_SYNTH_H
#define PLAN_SYNTH_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct plan_synth_spec {
    uint64_t n;              /* total particles */
    uint64_t seed;
    double frac_uniform;     /* fraction uniform in the box */
    double frac_sheets;      /* fraction in Gaussian sheets thin in y (x-z planes) */
    int32_t n_sheets;
    double sheet_sigma;      /* sheet thickness (standard deviation in y) */
    int32_t n_clumps;        /* Plummer spheres; they take the remaining particles */
    int32_t mass_function;   /* 0: equal split; 1: dN/dM ~ M^slope on [m_lo,m_hi] x total */
    double mf_slope, mf_lo, mf_hi;
    double a_lo, a_hi;       /* equal split: scale radius log-uniform in [a_lo,a_hi];
                                mass function: a = a_lo * (G M / 3)^(1/3), i.e. a fixed
                                fraction of the Hill radius, proportional to M^(1/3)   */
    double unbound_frac;     /* fraction of clumps whose velocities are scaled */
    double unbound_vscale;
    double G;                /* gravitational constant used for virial velocities */
    double half_box;         /* box is [-half_box, half_box)^3 */
    int32_t nx;              /* grid cells per side for the density field */
    double Z;                /* solid-to-gas ratio: total mass Z*Lx*Ly*sqrt(2 pi) */
    float time;              /* snapshot time written to the header */
} plan_synth_spec;

typedef struct plan_synth_info {
    uint64_t n_uniform, n_sheets, n_clumps;
    double particle_mass;
    double mean_density;     /* total mass / box volume */
    double clump_mass_min, clump_mass_max;  /* realised, in units of the total mass */
} plan_synth_info;

/* Fill a spec with the defaults for one of the named workloads:
 *   1: 262,144 particles, 80% uniform + 16 equal Plummer spheres (a in [1e-3,3e-3])
 *   2: 16,777,216 particles, 60% uniform, 25% in 4 sheets, 15% in 200 mass-function clumps
 *   5: 134,217,728 particles, 70% uniform, 20% in 16 sheets, 10% in 2,000 clumps
 * n overrides the particle count when non-zero (clump counts scale as in the workloads). */
int plan_synth_default_spec(int workload, uint64_t n, uint64_t seed, plan_synth_spec *spec);

/* Generate into a caller-owned record buffer of n*44 bytes (header written separately). */
int plan_synth_records(const plan_synth_spec *spec, void *records44, plan_synth_info *info);

/* Generate and write one combined .lis file. Returns 0 on success. */
int plan_synth_write_lis(const char *path, const plan_synth_spec *spec, plan_synth_info *info);

/* The four_pi_G_par that puts the density threshold of the reference
 * (2 Omega^2/(pi G), x9/8 for coarse sampling, src/tree.hpp:3633-3637) at the mean density. */
double plan_synth_four_pi_G_for_mean(const plan_synth_spec *spec, int32_t nx1, int32_t nx2);

#ifdef __cplusplus
}
#endif
#endif

// Deterministic synthetic .lis snapshots (see include/plan_synth.h).
//
// Reproducibility across hosts is the design constraint: no libm transcendental is called
// (glibc's exp/log/pow may differ in the last bit between x86-64 and aarch64, and GCC
// contracts to FMA on aarch64 unless told otherwise), so this file is compiled with
// -ffp-contract=off and evaluates exp/log from series with IEEE basic operations only.
#include "plan_synth.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

constexpr double kLn2Hi = 6.93147180369123816490e-01;
constexpr double kLn2Lo = 1.90821492927058770002e-10;
constexpr double kPi = 3.14159265358979323846;

inline uint64_t mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// Counter-based stream: value(stream, i) depends only on (seed, stream, i).
struct Rng {
    uint64_t seed, stream, ctr;
    Rng(uint64_t s, uint64_t st, uint64_t c0 = 0) : seed(s), stream(st), ctr(c0) {}
    uint64_t next() { return mix64(mix64(seed ^ (stream * 0xd1b54a32d192ed03ULL)) + ctr++); }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
    double uniform_open() {  // (0,1)
        double u;
        do { u = uniform(); } while (u == 0.0);
        return u;
    }
    // Irwin-Hall(12) - 6: a bounded, libm-free stand-in for a unit normal.
    double normalish() {
        double s = 0.0;
        for (int k = 0; k < 12; ++k) s += uniform();
        return s - 6.0;
    }
};

inline double pow2i(int k) {
    uint64_t bits = (uint64_t)(k + 1023) << 52;
    double d;
    std::memcpy(&d, &bits, 8);
    return d;
}

// exp(x) for |x| < 700: x = k ln2 + r, |r| <= ln2/2, Taylor series to degree 24.
double det_exp(double x) {
    double kd = x / (kLn2Hi + kLn2Lo);
    int k = (int)(kd >= 0 ? kd + 0.5 : kd - 0.5);
    double r = (x - k * kLn2Hi) - k * kLn2Lo;
    double term = 1.0, sum = 1.0;
    for (int n = 1; n <= 24; ++n) {
        term = term * r / n;
        sum = sum + term;
    }
    return sum * pow2i(k);
}

// log(x) for x > 0 normal: x = m 2^e with m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s).
double det_log(double x) {
    uint64_t bits;
    std::memcpy(&bits, &x, 8);
    int e = (int)((bits >> 52) & 0x7ff) - 1023;
    uint64_t mb = (bits & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL;
    double m;
    std::memcpy(&m, &mb, 8);
    if (m > 1.4142135623730951) { m = m * 0.5; e += 1; }
    double s = (m - 1.0) / (m + 1.0), s2 = s * s, term = s, sum = 0.0;
    for (int n = 1; n <= 61; n += 2) {
        sum = sum + term / n;
        term = term * s2;
    }
    return 2.0 * sum + (e * kLn2Lo + e * kLn2Hi);
}

inline double det_pow(double x, double y) { return det_exp(y * det_log(x)); }

// Uniform direction by rejection from the cube (exactly isotropic, only basic ops).
void unit_vector(Rng &g, double v[3]) {
    for (;;) {
        double x = 2.0 * g.uniform() - 1.0, y = 2.0 * g.uniform() - 1.0, z = 2.0 * g.uniform() - 1.0;
        double r2 = x * x + y * y + z * z;
        if (r2 > 1e-6 && r2 <= 1.0) {
            double r = std::sqrt(r2);
            v[0] = x / r; v[1] = y / r; v[2] = z / r;
            return;
        }
    }
}

inline double wrap(double x, double lo, double L) {
    while (x < lo) x += L;
    while (x >= lo + L) x -= L;
    return x;
}

// Float32 position strictly inside [lo, lo+L) after rounding.
inline float to_box_float(double x, float flo, float fhi) {
    float f = (float)x;
    if (f < flo) f = flo;
    if (f >= fhi) f = std::nextafter(fhi, flo);
    return f;
}

struct Rec {
    float pos[3], vel[3], dens;
    int32_t type;
    int64_t id;
    int32_t cpu;
};
static_assert(sizeof(float) * 7 + 4 + 8 + 4 == 44, "record size");

void put_rec(unsigned char *dst, const Rec &r) {
    std::memcpy(dst, r.pos, 12);
    std::memcpy(dst + 12, r.vel, 12);
    std::memcpy(dst + 24, &r.dens, 4);
    std::memcpy(dst + 28, &r.type, 4);
    std::memcpy(dst + 32, &r.id, 8);
    std::memcpy(dst + 40, &r.cpu, 4);
}

}  // namespace

extern "C" int plan_synth_default_spec(int workload, uint64_t n, uint64_t seed, plan_synth_spec *s) {
    if (!s) return 1;
    std::memset(s, 0, sizeof(*s));
    s->seed = seed;
    s->G = 0;  // filled from the density threshold below
    s->half_box = 0.1;
    s->nx = 128;
    s->Z = 0.02;
    s->time = 0.0f;
    s->sheet_sigma = 2e-3;
    s->unbound_vscale = 2.0;
    s->mf_slope = -1.6;
    s->mf_lo = 1e-5;
    s->mf_hi = 1e-2;
    switch (workload) {
    case 1:
        s->n = n ? n : 262144ULL;
        s->frac_uniform = 0.8;
        s->n_clumps = 16;
        s->mass_function = 0;
        s->a_lo = 1e-3; s->a_hi = 3e-3;
        break;
    case 2:
        s->n = n ? n : 16777216ULL;
        s->frac_uniform = 0.6;
        s->frac_sheets = 0.25;
        s->n_sheets = 4;
        s->n_clumps = n ? (int32_t)std::max<uint64_t>(1, (uint64_t)(200.0 * (double)n / 16777216.0 + 0.5)) : 200;
        s->mass_function = 1;
        s->a_lo = 0.05; s->a_hi = 0;
        s->unbound_frac = 0.1;
        break;
    case 5:
        s->n = n ? n : 134217728ULL;
        s->frac_uniform = 0.7;
        s->frac_sheets = 0.2;
        s->n_sheets = 16;
        s->n_clumps = n ? (int32_t)std::max<uint64_t>(1, (uint64_t)(2000.0 * (double)n / 134217728.0 + 0.5)) : 2000;
        s->mass_function = 1;
        s->a_lo = 0.05; s->a_hi = 0;
        s->unbound_frac = 0.1;
        break;
    default:
        return 2;
    }
    // G from four_pi_G_par: the density threshold equals the mean particle density.
    double fourpiG = plan_synth_four_pi_G_for_mean(s, s->nx, s->nx);
    s->G = fourpiG / (4.0 * kPi);
    return 0;
}

extern "C" double plan_synth_four_pi_G_for_mean(const plan_synth_spec *s, int32_t nx1, int32_t nx2) {
    // rho_thr = 2 Omega^2 / (pi G) with Omega = 1, times 9/8 when M/N/V_cell > rho_thr/4.
    // With G = four_pi_G/(4 pi): rho_thr = 8/four_pi_G. Choosing four_pi_G = 8/rho_mean
    // (or 9/rho_mean when the 9/8 branch fires) puts rho_thr at rho_mean.
    double L = 2.0 * s->half_box;
    double mtot = s->Z * L * L * std::sqrt(2.0 * kPi);
    double rho_mean = mtot / (L * L * L);
    double cell = L / (double)s->nx;
    double mpp_over_vcell = mtot / (double)s->n / (cell * cell * cell);
    (void)nx1; (void)nx2;
    // The 9/8 branch compares against rho_thr/4 = rho_mean/4 under either choice.
    return (mpp_over_vcell > rho_mean / 4.0) ? 9.0 / rho_mean : 8.0 / rho_mean;
}

extern "C" int plan_synth_records(const plan_synth_spec *s, void *out, plan_synth_info *info) {
    if (!s || !out || s->n == 0) return 1;
    const uint64_t N = s->n;
    const double L = 2.0 * s->half_box, lo = -s->half_box;
    const float flo = (float)lo, fhi = (float)(lo + L);
    const double mtot = s->Z * L * L * std::sqrt(2.0 * kPi);
    const double m = mtot / (double)N;
    uint64_t nu = (uint64_t)((double)N * s->frac_uniform);
    uint64_t ns = (s->n_sheets > 0) ? (uint64_t)((double)N * s->frac_sheets) : 0;
    if (nu + ns > N) ns = N - nu;
    uint64_t nc = N - nu - ns;
    if (s->n_clumps <= 0) { nu += nc; nc = 0; }

    std::vector<Rec> recs(N);
    // 1) uniform background
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)nu; ++i) {
        Rng g(s->seed, 1, (uint64_t)i * 8);
        Rec &r = recs[i];
        for (int d = 0; d < 3; ++d) r.pos[d] = to_box_float(lo + L * g.uniform(), flo, fhi);
        for (int d = 0; d < 3; ++d) r.vel[d] = 0.0f;
    }
    // 2) Gaussian sheets: x, z uniform; y around a per-sheet centre
    std::vector<double> sheet_y(s->n_sheets > 0 ? s->n_sheets : 1);
    {
        Rng g(s->seed, 2);
        for (int k = 0; k < s->n_sheets; ++k) sheet_y[k] = lo + L * g.uniform();
    }
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < (int64_t)ns; ++j) {
        Rng g(s->seed, 3, (uint64_t)j * 24);
        Rec &r = recs[nu + j];
        int k = (int)(j % s->n_sheets);
        r.pos[0] = to_box_float(lo + L * g.uniform(), flo, fhi);
        r.pos[2] = to_box_float(lo + L * g.uniform(), flo, fhi);
        r.pos[1] = to_box_float(wrap(sheet_y[k] + s->sheet_sigma * g.normalish(), lo, L), flo, fhi);
        for (int d = 0; d < 3; ++d) r.vel[d] = 0.0f;
    }
    // 3) Plummer clumps
    int nk = nc ? s->n_clumps : 0;
    std::vector<double> cm(nk), ca(nk), cen(3 * (size_t)nk), vs(nk);
    std::vector<uint64_t> cnt(nk), off(nk + 1, 0);
    double mmin = 1e300, mmax = 0;
    if (nk) {
        Rng g(s->seed, 4);
        std::vector<double> w(nk);
        double wsum = 0;
        for (int k = 0; k < nk; ++k) {
            if (s->mass_function == 1) {
                // inverse CDF of dN/dM ~ M^slope on [lo, hi]
                double e = s->mf_slope + 1.0;
                double alo = det_pow(s->mf_lo, e), ahi = det_pow(s->mf_hi, e);
                double u = g.uniform();
                w[k] = det_pow(alo + u * (ahi - alo), 1.0 / e);
            } else {
                w[k] = 1.0;
            }
            wsum += w[k];
        }
        // particle counts proportional to the drawn masses, summing to nc
        uint64_t acc = 0;
        for (int k = 0; k < nk; ++k) {
            cnt[k] = (uint64_t)((double)nc * w[k] / wsum);
            if (cnt[k] < 2) cnt[k] = 2;
            acc += cnt[k];
        }
        // fix rounding: give the remainder to (or take the excess from) the largest clumps
        while (acc < nc) {
            int big = 0;
            for (int k = 1; k < nk; ++k) if (cnt[k] > cnt[big]) big = k;
            cnt[big] += nc - acc;
            acc = nc;
        }
        while (acc > nc) {
            int big = 0;
            for (int k = 1; k < nk; ++k) if (cnt[k] > cnt[big]) big = k;
            if (cnt[big] <= 2) break;
            uint64_t take = std::min<uint64_t>(acc - nc, cnt[big] - 2);
            cnt[big] -= take;
            acc -= take;
        }
        acc = 0;
        for (int k = 0; k < nk; ++k) { off[k] = acc; acc += cnt[k]; }
        off[nk] = acc;
        if (acc != nc) return 4;  // too few clump particles for the requested clump count
        for (int k = 0; k < nk; ++k) {
            cm[k] = (double)cnt[k] * m;
            double frac = cm[k] / mtot;
            if (frac < mmin) mmin = frac;
            if (frac > mmax) mmax = frac;
            if (s->mass_function == 1) {
                // a = a_lo x Hill radius (G M / 3 Omega^2)^(1/3): proportional to M^(1/3)
                ca[k] = s->a_lo * det_pow(s->G * cm[k] / 3.0, 1.0 / 3.0);
            } else {
                double u = g.uniform();
                ca[k] = det_exp(det_log(s->a_lo) + u * (det_log(s->a_hi) - det_log(s->a_lo)));
            }
            for (int d = 0; d < 3; ++d) cen[3 * k + d] = lo + L * g.uniform();
            vs[k] = (g.uniform() < s->unbound_frac) ? s->unbound_vscale : 1.0;
        }
    }
    // clump particles are written after uniform and sheet particles
    const uint64_t cbase = N - nc;
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k < nk; ++k) {
        Rng g(s->seed, 100 + (uint64_t)k);
        double a = ca[k], M = cm[k];
        for (uint64_t j = 0; j < cnt[k]; ++j) {
            Rec &r = recs[cbase + off[k] + j];
            double rad;
            for (;;) {  // Plummer cumulative mass M(<r) = M r^3/(r^2+a^2)^{3/2}, truncated at 10a
                double X = g.uniform_open();
                double t = det_pow(X, -2.0 / 3.0) - 1.0;
                if (t <= 0) continue;
                rad = a / std::sqrt(t);
                if (rad <= 10.0 * a) break;
            }
            double dir[3];
            unit_vector(g, dir);
            // speed from the Plummer distribution function (Aarseth, Henon & Wielen 1974):
            // q = v/v_esc with density g(q) = q^2 (1-q^2)^{7/2}, by rejection.
            double q;
            for (;;) {
                double x1 = g.uniform(), x2 = g.uniform();
                double om = 1.0 - x1 * x1;
                double gq = x1 * x1 * om * om * om * std::sqrt(om);
                if (0.1 * x2 < gq) { q = x1; break; }
            }
            double vesc = std::sqrt(2.0 * s->G * M / std::sqrt(rad * rad + a * a));
            double vdir[3];
            unit_vector(g, vdir);
            double v = q * vesc * vs[k];
            for (int d = 0; d < 3; ++d) {
                r.pos[d] = to_box_float(wrap(cen[3 * k + d] + rad * dir[d], lo, L), flo, fhi);
                r.vel[d] = (float)(v * vdir[d]);
            }
        }
    }
    // density field: nearest-grid-point deposit on nx^3 cells
    const int nx = s->nx;
    const double cell = L / nx, vcell = cell * cell * cell;
    std::vector<uint32_t> counts((size_t)nx * nx * nx, 0);
    std::vector<uint32_t> cid(N);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)N; ++i) {
        int c[3];
        for (int d = 0; d < 3; ++d) {
            int v = (int)(((double)recs[i].pos[d] - lo) / cell);
            c[d] = v < 0 ? 0 : (v >= nx ? nx - 1 : v);
        }
        cid[i] = (uint32_t)(((size_t)c[2] * nx + c[1]) * nx + c[0]);
    }
    for (uint64_t i = 0; i < N; ++i) counts[cid[i]]++;
    unsigned char *dst = static_cast<unsigned char *>(out);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)N; ++i) {
        Rec &r = recs[i];
        r.dens = (float)((double)counts[cid[i]] * m / vcell);
        r.type = 0;
        r.id = i;
        r.cpu = 0;
        put_rec(dst + 44 * (size_t)i, r);
    }
    if (info) {
        info->n_uniform = nu;
        info->n_sheets = ns;
        info->n_clumps = N - nu - ns;
        info->particle_mass = m;
        info->mean_density = mtot / (L * L * L);
        info->clump_mass_min = nk ? mmin : 0;
        info->clump_mass_max = nk ? mmax : 0;
    }
    return 0;
}

extern "C" int plan_synth_write_lis(const char *path, const plan_synth_spec *s, plan_synth_info *info) {
    if (!path || !s) return 1;
    std::vector<unsigned char> body((size_t)s->n * 44);
    int rc = plan_synth_records(s, body.data(), info);
    if (rc) return rc;
    FILE *f = std::fopen(path, "wb");
    if (!f) return 3;
    float lim[12];
    float flo = (float)(-s->half_box), fhi = (float)s->half_box;
    for (int i = 0; i < 12; i += 2) { lim[i] = flo; lim[i + 1] = fhi; }
    int32_t ntypes = 1;
    float tinfo = 1.0f, t = s->time, dt = 0.0f;
    int64_t n = (int64_t)s->n;
    bool ok = std::fwrite(lim, 4, 12, f) == 12 && std::fwrite(&ntypes, 4, 1, f) == 1 &&
              std::fwrite(&tinfo, 4, 1, f) == 1 && std::fwrite(&t, 4, 1, f) == 1 &&
              std::fwrite(&dt, 4, 1, f) == 1 && std::fwrite(&n, 8, 1, f) == 1 &&
              std::fwrite(body.data(), 1, body.size(), f) == body.size();
    std::fclose(f);
    return ok ? 0 : 3;
}

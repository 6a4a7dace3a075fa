// Catalogue assembly and writers (src/tree.hpp:4291-4326, 4935-5222).
//
// The device delivers each final clump with its mass, centre of mass, velocity, the raw
// angular-momentum sum and its members. What the reference computes with libm for output
// only - the printed Hill radius pow(M G/3/Omega^2, 1/3.), the J normalisation, the
// geometric-mean and median offsets after the rotation by J (acos/atan2/cos/sin/log10/pow)
// - is computed here with the host libm, so printed numbers carry the reference's bits.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iomanip>
#include <numeric>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <thread>
#include <vector>

#include "../catalogue.h"

namespace plan {

static void offsets(plan_catalogue::Clump &k) {
    const size_t n = k.opos.size() / 3;
    k.geo[0] = k.geo[1] = k.geo[2] = 0;
    k.med[0] = k.med[1] = k.med[2] = 0;
    if (n == 0) return;
    double s = 0;  // SmallVec::Norm sums from 0 in order
    s += k.J[0] * k.J[0];
    s += k.J[1] * k.J[1];
    s += k.J[2] * k.J[2];
    double jn = std::sqrt(s);
    double theta = std::acos(k.J[2] / jn);
    double phi = std::atan2(k.J[1], k.J[0]);
    double rz[3][3] = {{std::cos(phi), -std::sin(phi), 0}, {std::sin(phi), std::cos(phi), 0}, {0, 0, 1}};
    double ry[3][3] = {{std::cos(theta), 0, std::sin(theta)}, {0, 1, 0}, {-std::sin(theta), 0, std::cos(theta)}};
    double rot[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            rot[a][b] = 0;
            for (int d = 0; d < 3; ++d) rot[a][b] += rz[a][d] * ry[d][b];
        }
    std::vector<double> off[3];
    for (int d = 0; d < 3; ++d) off[d].resize(n);
    for (size_t q = 0; q < n; ++q) {
        double t[3];
        for (int d = 0; d < 3; ++d) t[d] = k.opos[3 * q + d] - k.com[d];
        for (int d = 0; d < 3; ++d) {
            double v = 0;
            for (int a = 0; a < 3; ++a) v += t[a] * rot[a][d];
            off[d][q] = v;
        }
    }
    const size_t half = n / 2;
    const bool even = !(n & 1);
    for (int d = 0; d < 3; ++d) {
        for (auto &v : off[d]) v = std::abs(v);
        double acc = 0.;
        for (double v : off[d]) acc = (v < 1e-32) ? acc - 32 : acc + std::log10(v);
        k.geo[d] = std::pow(10.0, acc / n);
        std::nth_element(off[d].begin(), off[d].begin() + half, off[d].end());
        k.med[d] = off[d][half];
        if (even) k.med[d] = (k.med[d] + *std::max_element(off[d].begin(), off[d].begin() + half)) / 2.0;
    }
}

void finish_catalogue(plan_catalogue &cat, uint32_t num_peaks) {
    auto &cl = cat.clumps;  // key order on entry
    for (auto &k : cl) {
        k.hill = pow(k.M * cat.grav_constant / 3. / cat.Omega / cat.Omega, 1. / 3.);
        double units = k.M * k.hill * k.hill * cat.Omega;
        for (int d = 0; d < 3; ++d) k.J[d] = k.Jsum[d] / units;
    }
    // ranking (src/tree.hpp:4293-4301) and the num_peaks cap (4303-4318)
    std::vector<size_t> order(cl.size());
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        if (cl[a].M == cl[b].M) return cl[a].key < cl[b].key;
        return cl[a].M < cl[b].M;
    });
    std::vector<char> keep(cl.size(), 1);
    if (num_peaks > 0 && cl.size() > num_peaks) {
        size_t drop = cl.size() - num_peaks;
        for (size_t i = 0; i < drop; ++i) keep[order[i]] = 0;
        order.erase(order.begin(), order.begin() + drop);
    }
    // WriteBasicResults sums over the map in key order
    cat.basic_max = 0;
    cat.basic_tot = 0;
    for (size_t i = 0; i < cl.size(); ++i) {
        if (!keep[i]) continue;
        cat.basic_max = std::max(cat.basic_max, cl[i].M);
        cat.basic_tot += cl[i].M;
    }
    std::vector<plan_catalogue::Clump> ranked;
    ranked.reserve(order.size());
    for (size_t i : order) ranked.push_back(std::move(cl[i]));
    cl.swap(ranked);
    cat.num = (uint32_t)cl.size();
    cat.mp_tot_sorted = 0.;
    for (auto &k : cl) cat.mp_tot_sorted = cat.mp_tot_sorted + k.M;
    cat.mp_max = cl.empty() ? 0 : cl.back().M;
    // offsets: one thread per block of clumps (each clump's sums stay sequential)
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned w = 0; w < nt; ++w)
        th.emplace_back([&, w]() {
            for (size_t i = w; i < cl.size(); i += nt) offsets(cl[i]);
        });
    for (auto &t : th) t.join();
}

}  // namespace plan

using plan::finish_catalogue;

extern "C" {

void plan_catalogue_free(plan_catalogue *cat) { delete cat; }

uint32_t plan_catalogue_count(const plan_catalogue *cat) { return cat ? (uint32_t)cat->clumps.size() : 0; }

int plan_catalogue_get(const plan_catalogue *cat, uint32_t i, plan_clump_info *info) {
    if (!cat || !info || i >= cat->clumps.size()) return 2;
    const auto &k = cat->clumps[i];
    info->peak_id = k.key;
    info->npar = k.npar;
    info->total_mass = k.M;
    info->hill_radius = k.hill;
    for (int d = 0; d < 3; ++d) {
        info->com[d] = k.com[d];
        info->vel_com[d] = k.vcom[d];
        info->J[d] = k.J[d];
    }
    return 0;
}

const char *plan_catalogue_summary(const plan_catalogue *cat) {
    if (!cat) return "";
    // FindPlanetesimals' stdout line for the first snapshot of a run (default stream state)
    std::ostringstream o;
    o << "Finish clump finding for t = " << cat->time << ", ";
    if (cat->num > 0) {
        o << "found " << cat->num << " clumps; " << " Mp_max = " << cat->mp_max << ", Mp_tot = " << cat->mp_tot_sorted << "(" << std::fixed
          << cat->mp_tot_sorted / cat->mass_total_code_units * 100 << "%) in code units.";
    } else {
        o << "found zero clumps";
    }
    const_cast<plan_catalogue *>(cat)->summary = o.str();
    return cat->summary.c_str();
}

int plan_catalogue_write_peaks(const plan_catalogue *cat, const char *out_path, int save_clumps, int file_number, uint32_t sampling) {
    if (!cat || !out_path) return 2;
    std::ostringstream ts;
    ts << std::setprecision(3) << std::fixed << std::setw(7) << std::setfill('0') << cat->time;
    std::string op(out_path), name;
    size_t slash = op.find_last_of('/');
    if (slash != std::string::npos) name = op.substr(0, slash) + "/peaks_at_" + ts.str() + ".txt";
    else name = "peaks_at_" + ts.str() + ".txt";
    FILE *f = std::fopen(name.c_str(), "w");
    if (!f) {
        std::fprintf(stderr, "Error: Failed to open file %s due to %s\n", name.c_str(), std::strerror(errno));
        return 3;
    }
    std::ostringstream o;
    o << std::setw(12) << "#peak_id" << std::setw(12) << "Npar" << std::setw(24) << "total_mass" << std::setw(24) << "Hill_radius"
      << std::setw(24) << "center_of_mass[x]" << std::setw(24) << "center_of_mass[y]" << std::setw(24) << "center_of_mass[z]"
      << std::setw(24) << "vel_COM[x]" << std::setw(24) << "vel_COM[y]" << std::setw(24) << "vel_COM[z]" << std::setw(24) << "J[x]"
      << std::setw(24) << "J[y]" << std::setw(24) << "J[z]/(M R_H^2 Omega)" << std::setw(24) << "geo_mean_offset[x]" << std::setw(24)
      << "geo_mean_offset[y]" << std::setw(24) << "geo_mean_offset[z]" << std::setw(24) << "median_offset[x]" << std::setw(24)
      << "median_offset[y]" << std::setw(24) << "median_offset[z]" << std::endl;
    std::string dir;
    if (save_clumps) {
        std::ostringstream sid;
        sid << std::setw(4) << std::setfill('0') << file_number;
        dir = "ParList." + sid.str();
        mkdir(dir.c_str(), 0755);
    }
    if (sampling == 0) sampling = 1;
    for (const auto &k : cat->clumps) {
        if (save_clumps) {  // OutputSinglePlanetesimal (src/tree.hpp:5191-5222)
            FILE *pf = std::fopen((dir + "/" + std::to_string(k.key) + ".txt").c_str(), "w");
            if (pf) {
                std::ostringstream po;
                uint32_t skip = 0;
                for (size_t q = 0; q < k.orig.size(); ++q) {
                    if (skip > 0) { --skip; continue; }
                    skip = sampling - 1;
                    po.unsetf(std::ios_base::floatfield);
                    po << std::setw(16) << k.orig[q];
                    po << std::scientific;
                    for (int d = 0; d < 3; ++d) po << std::setprecision(16) << std::setw(24) << k.pos[3 * q + d];
                    for (int d = 0; d < 3; ++d) po << std::setprecision(16) << std::setw(24) << k.vel[3 * q + d];
                    po << std::setprecision(16) << std::setw(24) << k.mass[q] << std::endl;
                }
                std::string str = po.str();
                std::fwrite(str.data(), 1, str.size(), pf);
                std::fclose(pf);
            } else {
                std::fprintf(stderr, "Error: Failed to open file: %s/%u.txt. But we proceed.\n", dir.c_str(), k.key);
            }
        }
        o << std::setw(12) << k.key << std::setw(12) << k.npar << std::setprecision(16) << std::setw(24) << k.M << std::setw(24) << k.hill
          << std::setw(24) << k.com[0] << std::setw(24) << k.com[1] << std::setw(24) << k.com[2] << std::setw(24) << k.vcom[0]
          << std::setw(24) << k.vcom[1] << std::setw(24) << k.vcom[2] << std::setw(24) << k.J[0] << std::setw(24) << k.J[1]
          << std::setw(24) << k.J[2] << std::setw(24) << k.geo[0] << std::setw(24) << k.geo[1] << std::setw(24) << k.geo[2]
          << std::setw(24) << k.med[0] << std::setw(24) << k.med[1] << std::setw(24) << k.med[2] << std::endl;
    }
    std::string str = o.str();
    bool ok = std::fwrite(str.data(), 1, str.size(), f) == str.size();
    std::fclose(f);
    return ok ? 0 : 3;
}

int plan_catalogue_basic_results(const plan_catalogue *cat, const plan_params *p, int with_header, char *buf, size_t cap) {
    if (!cat || !p || !buf) return -1;
    std::ostringstream o;
    const int w = 15;
    if (with_header)
        o << std::setw(w) << std::setfill(' ') << "#time" << std::setw(w) << "N_peak" << std::setw(w) << std::setfill(' ') << "M_p,max,code"
          << std::setw(w) << std::setfill(' ') << "M_p,tot,code" << std::setw(w) << std::setfill(' ') << "M_p,max,frac" << std::setw(w)
          << std::setfill(' ') << "M_p,tot,frac" << std::setw(w) << std::setfill(' ') << "M_p,max,Ceres" << std::setw(w) << std::setfill(' ')
          << "M_p,tot,Ceres" << std::endl;
    o << std::setw(w) << std::setfill(' ') << std::scientific << cat->time;
    o << std::setw(w) << std::setfill(' ') << cat->num;
    o << std::setw(w) << std::setfill(' ') << cat->basic_max << std::setw(w) << std::setfill(' ') << cat->basic_tot;
    o << std::setw(w) << std::setfill(' ') << cat->basic_max / p->mass_total_code_units << std::setw(w) << std::setfill(' ')
      << cat->basic_tot / p->mass_total_code_units;
    o << std::setw(w) << std::setfill(' ') << cat->basic_max * p->mass_physical / 9.4e20 << std::setw(w) << std::setfill(' ')
      << cat->basic_tot * p->mass_physical / 9.4e20;
    o << std::endl;
    std::string s = o.str();
    if (s.size() + 1 > cap) return -1;
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return (int)s.size();
}

}  // extern "C"

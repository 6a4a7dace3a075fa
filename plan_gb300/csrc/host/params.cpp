// Parameter handling of the reference (src/global.hpp:676-874, src/global.cpp:28-225),
// host side: these are scalars computed once per run with the host's libm, exactly as
// the reference computes them.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <unordered_map>

#include "plan_gpu.h"

namespace {
constexpr double kPi = 3.14159265358979323846;

void trim(std::string &s) {
    size_t b = 0, e = s.size();
    while (b < e && std::isspace(static_cast<unsigned char>(s[b]))) ++b;
    while (e > b && std::isspace(static_cast<unsigned char>(s[e - 1]))) --e;
    s = s.substr(b, e - b);
}
}  // namespace

extern "C" void plan_params_init(plan_params *p) {
    std::memset(p, 0, sizeof(*p));
    p->solid_to_gas_ratio = 0.02;
    for (int d = 0; d < 3; ++d) {
        p->box_resolution[d] = 128;
        p->box_center[d] = 0.0;
        p->box_length[d] = 0.2;
        p->box_min[d] = -0.1;
        p->box_max[d] = 0.1;
        p->box_half_width[d] = 0.1;
        p->cell_length[d] = 0.0015625;
        p->ghost_zone_width[d] = 0.025;
    }
    p->max_half_width = 0.1;
    p->max_ghost_zone_width = 0.025;
    p->cell_volume = 0.0015625 * 0.0015625 * 0.0015625;
    p->four_pi_G = 0.05;
    p->num_threads = 0;
    p->num_peaks = 0;
    p->knn = 64;
    p->hop = 32;
    p->fixed_hop = 0;
    p->clump_diffuse_threshold = -1.0;
    p->Hill_fraction_for_merge = -1.0;
    p->q = 1.5;
    p->Omega = 1.0;
    p->rho_g0 = 1.0;
    p->mass_total_code_units = 0.0020053;
    p->G_tilde = p->four_pi_G * p->rho_g0 / p->Omega / p->Omega;
    p->mass_physical = (p->G_tilde / 0.1) * 1.3e24;
    p->grav_constant = p->four_pi_G / (4. * kPi);
    p->shear_speed = p->q * p->Omega * p->box_length[0];
    p->min_trusted_mass = 2.87621e-6;
    p->ntypes = 1;
    p->mass_fraction_per_species[0] = 1;
}

extern "C" void plan_params_derive(plan_params *p) {  // CalculateNewParameters, src/global.cpp:28-47
    for (int d = 0; d < 3; ++d) p->box_half_width[d] = p->box_length[d] / 2.0;
    p->max_half_width = 0.0;
    for (int d = 0; d < 3; ++d) {
        p->max_half_width = std::max(p->max_half_width, p->box_half_width[d]);
        p->max_ghost_zone_width = std::max(p->max_ghost_zone_width, p->ghost_zone_width[d]);
    }
    for (int d = 0; d < 3; ++d) p->cell_length[d] = p->box_length[d] / p->box_resolution[d];
    p->cell_volume = 1.0;
    for (int d = 0; d < 3; ++d) p->cell_volume = p->cell_volume * p->cell_length[d];
    p->mass_total_code_units = std::sqrt(2 * kPi) * p->box_length[0] * p->box_length[1] * p->solid_to_gas_ratio;
    p->G_tilde = p->four_pi_G / p->Omega / p->Omega;
    p->mass_physical = (p->G_tilde / 0.1) * 1.3e24;
    p->grav_constant = p->four_pi_G / (4. * kPi);
    p->shear_speed = p->q * p->Omega * p->box_length[0];
    p->min_trusted_mass = 3 * std::pow(p->cell_length[0], 3) * p->Omega * p->Omega / p->rho_g0 / p->grav_constant;
}

extern "C" int plan_params_read(const char *path, plan_params *p) {  // src/global.cpp:51-225
    if (!path || !p) return 2;
    std::ifstream in(path);
    if (!in.is_open()) {
        std::fprintf(stderr, "Error: Failed to open file %s\n", path);
        return 3;
    }
    std::unordered_map<std::string, double> kv;  // first occurrence of a name wins (emplace)
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
            double v1 = 0, v2 = 0;
            char c;
            iss >> v1 >> c >> v2;
            kv.emplace(name, v1 / v2);
        } else {
            try {
                kv.emplace(name, std::stod(value));
            } catch (...) {
                std::fprintf(stderr, "Error: cannot read a number for %s in %s\n", name.c_str(), path);
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
    if (get("Z", v)) p->solid_to_gas_ratio = v;
    if (get("Nx1", v)) p->box_resolution[0] = (uint32_t)v;
    if (get("Nx2", v)) p->box_resolution[1] = (uint32_t)v;
    if (get("Nx3", v)) p->box_resolution[2] = (uint32_t)v;
    if (get("four_pi_G_par", v)) p->four_pi_G = v;
    if (get("omp_threads", v)) p->num_threads = (uint32_t)v;
    if (get("num_threads", v)) p->num_threads = (uint32_t)v;
    if (get("num_peaks", v)) p->num_peaks = (uint32_t)v;
    if (get("num_peak", v)) p->num_peaks = (uint32_t)v;
    if (get("num_neighbors_in_knn_search", v)) p->knn = (uint32_t)v;
    if (get("num_knn", v)) p->knn = (uint32_t)v;
    if (get("knn", v)) p->knn = (uint32_t)v;
    if (get("num_neighbors_to_hop", v)) { p->hop = (uint32_t)v; p->fixed_hop = 1; }
    if (get("num_hop", v)) { p->hop = (uint32_t)v; p->fixed_hop = 1; }
    if (get("hop", v)) { p->hop = (uint32_t)v; p->fixed_hop = 1; }
    if (get("clump_diffuse_threshold", v)) {
        p->clump_diffuse_threshold = v;
        if (v < 0) return 4;
    }
    if (get("Hill_fraction_for_merge", v)) {
        p->Hill_fraction_for_merge = v;
        if (v < 0) return 4;
    }
    plan_params_derive(p);
    return 0;
}

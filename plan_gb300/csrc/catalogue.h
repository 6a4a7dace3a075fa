// Host-side catalogue produced by plan_find_planetesimals.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "plan_gpu.h"

struct plan_catalogue {
    struct Clump {
        uint32_t key = 0, npar = 0;
        double M = 0, hill = 0, com[3] = {0, 0, 0}, vcom[3] = {0, 0, 0}, Jsum[3] = {0, 0, 0}, J[3] = {0, 0, 0};
        double geo[3] = {0, 0, 0}, med[3] = {0, 0, 0};
        // members in the clump's `particles` order (tree points)
        std::vector<uint32_t> orig;
        std::vector<double> pos, vel, mass;
        // offset sources in `indices` order with sink particles expanded
        std::vector<double> opos;
    };
    std::vector<Clump> clumps;  // output order: ascending mass, ties by peak id
    double time = 0;
    uint32_t num = 0;
    double mp_max = 0, mp_tot_sorted = 0;       // summary line (mass order)
    double basic_max = 0, basic_tot = 0;        // WriteBasicResults (key order)
    double mass_total_code_units = 0, mass_physical = 0;
    double grav_constant = 0, Omega = 1;
    std::string summary;
    bool have_members = false;
};

namespace plan {
// Finish a catalogue on the host (clumps arrive in key order): ranking by mass, the
// num_peaks cap, Hill radii and J normalisation with the host libm (the printed values are
// those of the reference's own libm calls), offsets and the summary text.
void finish_catalogue(plan_catalogue &cat, uint32_t num_peaks);
}  // namespace plan

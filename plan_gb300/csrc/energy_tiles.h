// Tile widths of the batched boundness pass, one per group-size class: a group of n particles
// is in class k when n < kEnergyClassBound[k] (the last class has no bound). The widths are
// measured choices: plan_gb300/tune_energy.py times every width for every class on the GPU,
// prints the timings it chose from and writes this file.
// PLAN_ENERGY_TILES="w0,w1,w2,w3" overrides them for one run (the tuner's switch).
#pragma once

#include <cstdint>

namespace plan {

constexpr int kEnergyClasses = 4;
constexpr uint64_t kEnergyClassBound[kEnergyClasses - 1] = {64, 512, 8192};
constexpr int kEnergyTile[kEnergyClasses] = {32, 128, 256, 256};

}  // namespace plan

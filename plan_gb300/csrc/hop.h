// HOP grouping interface.
#pragma once

#include "pipeline.h"

namespace plan {

struct HopGroups {
    uint32_t n_members = 0, n_groups = 0;
    uint32_t *members = nullptr;  // tree indices, grouped by peak, in the reference's insertion order
    uint32_t *key = nullptr;      // peak (root) index per group, ascending
    uint32_t *off = nullptr;      // group g = members[off[g], off[g+1])
    uint32_t *peak = nullptr;     // root per tree point (above-threshold points)
    uint32_t *above = nullptr;    // 1 where density >= threshold
};

int hop_groups(Context &c, const uint32_t *densest, double thr, HopGroups &out, cudaStream_t s);

}  // namespace plan

// Front of the pipeline: device ingest of .lis records, (cpu_id, id_in_run) order,
// shearing-periodic ghosts, Morton keys, radix sort, sink folding and the octree.
//
// Reference: ParticleSet::ReadLisFile/MakeGhostParticles (src/tree.hpp:1540-1754) and
// BHtree::BuildTree (src/tree.hpp:2759-2908). The octree is built bottom-up in parallel
// from the sorted keys but reproduces the reference's node numbering exactly: a node at
// tree level L+1 gets index level_offset[L] + (rank of its key prefix among level-(L+1)
// nodes), which is the depth-first creation order of FillTree within a level.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "octree_rules.cuh"
#include "pipeline.h"
#include "sort.h"

namespace plan {

namespace {

struct MassTable {
    double m[16];
    uint32_t ntypes;
};

// ---------------------------------------------------------------- ingest
__global__ void k_unpack(const unsigned char *rec, size_t n, double4_32a *pos, double4_32a *vel, uint32_t *type, uint32_t *kw0,
                         uint32_t *kw1, uint32_t *kw2, uint32_t *kidx) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned char *r = rec + 44 * i;
    float f[7];
    for (int k = 0; k < 7; ++k) {
        uint32_t u = (uint32_t)r[4 * k] | ((uint32_t)r[4 * k + 1] << 8) | ((uint32_t)r[4 * k + 2] << 16) | ((uint32_t)r[4 * k + 3] << 24);
        f[k] = __uint_as_float(u);
    }
    auto u32at = [&](int off) {
        return (uint32_t)r[off] | ((uint32_t)r[off + 1] << 8) | ((uint32_t)r[off + 2] << 16) | ((uint32_t)r[off + 3] << 24);
    };
    pos[i] = make_double4_32a((double)f[0], (double)f[1], (double)f[2], 0.0);
    vel[i] = make_double4_32a((double)f[3], (double)f[4], (double)f[5], (double)f[6]);
    type[i] = u32at(28);
    kw0[i] = u32at(32);               // id_in_run: low 32 bits of the i64 (src/tree.hpp:1507)
    kw1[i] = u32at(40) & 0xffffu;     // cpu_id as uint16 (src/tree.hpp:1510)
    kw2[i] = 0;
    kidx[i] = (uint32_t)i;
}

__global__ void k_count_descents(const uint32_t *kw0, const uint32_t *kw1, size_t n, unsigned long long *out) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x + 1;
    if (i >= n) return;
    uint64_t a = ((uint64_t)kw1[i - 1] << 32) | kw0[i - 1], b = ((uint64_t)kw1[i] << 32) | kw0[i];
    if (b < a) atomicAdd(&out[0], 1ull);
    if (b == a) atomicAdd(&out[1], 1ull);
}

__global__ void k_gather_in(const uint32_t *perm, size_t n, const double4_32a *pos, const double4_32a *vel, const uint32_t *type, double4_32a *pos2,
                            double4_32a *vel2, uint32_t *type2) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t s = perm[i];
    pos2[i] = pos[s];
    vel2[i] = vel[s];
    type2[i] = type[s];
}

// ---------------------------------------------------------------- user box (src/tree.hpp:1585-1620)
struct UserBox {
    double lo[3], hi[3];
};

// 1 for particles (in (cpu_id, id_in_run) order) inside the closed user box (SmallVec::InRange,
// src/global.hpp:543-549)
__global__ void k_box_flags(const uint32_t *order, uint32_t n, const double4_32a *pos, UserBox b, uint32_t *flag) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double4_32a p = pos[order[i]];
    const bool in = p.x >= b.lo[0] && p.x <= b.hi[0] && p.y >= b.lo[1] && p.y <= b.hi[1] && p.z >= b.lo[2] && p.z <= b.hi[2];
    flag[i] = in ? 1u : 0u;
}

// stable compaction of the kept particles: their file-order index and their rank before the
// selection (the particle id, assigned before the box is applied)
__global__ void k_box_compact(const uint32_t *order, uint32_t n, const uint32_t *flag, const uint32_t *off, uint32_t *src, uint32_t *rank) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !flag[i]) return;
    src[off[i]] = order[i];
    rank[off[i]] = i;
}

// particle ids of the tree points: kept originals take their rank before the selection, ghosts
// keep theirs (numbered from the kept count, src/tree.hpp:1633)
__global__ void k_box_ids(uint32_t *orig, uint32_t n, uint32_t nkept, const uint32_t *rank) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const uint32_t o = orig[t];
    if (o < nkept) orig[t] = rank[o];
}

// ---------------------------------------------------------------- ghosts
struct GhostGeom {
    double lo[3], hi[3];      // non-ghost region
    double box_min1, box_max1, len0, len1, shear_dt;  // shear_dt = shear_speed * time
};

__global__ void k_ghost_count_x(const double4_32a *pos, uint32_t n, GhostGeom g, uint32_t *cnt) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x = pos[i].x;
    cnt[i] = (x > g.hi[0] ? 1u : 0u) + (x < g.lo[0] ? 1u : 0u);
}

// x ghosts, written at n + off[i] (src/tree.hpp:1657-1676)
__global__ void k_ghost_write_x(double4_32a *pos, double4_32a *vel, uint32_t *type, uint32_t n, GhostGeom g, const uint32_t *off) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double4_32a p = pos[i];
    uint32_t o = n + off[i];
    if (p.x > g.hi[0]) {
        double4_32a q = p;
        q.x = q.x - g.len0;
        double ny = q.y + g.shear_dt;
        q.y = ny - (double)(int)((ny - g.box_min1) / g.len1) * g.len1;
        pos[o] = q; vel[o] = vel[i]; type[o] = type[i];
        ++o;
    }
    if (p.x < g.lo[0]) {
        double4_32a q = p;
        q.x = q.x + g.len0;
        double ny = q.y - g.shear_dt;
        q.y = ny + (double)(int)((g.box_max1 - ny) / g.len1) * g.len1;
        pos[o] = q; vel[o] = vel[i]; type[o] = type[i];
    }
}

// y ghosts of the range [from, from+m): (y < lo) first, then (y > hi) (src/tree.hpp:1694-1721)
__global__ void k_ghost_count_y(const double4_32a *pos, uint32_t from, uint32_t m, GhostGeom g, uint32_t *cnt) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    double y = pos[from + k].y;
    cnt[k] = (y < g.lo[1] ? 1u : 0u) + (y > g.hi[1] ? 1u : 0u);
}

__global__ void k_ghost_write_y(double4_32a *pos, double4_32a *vel, uint32_t *type, uint32_t from, uint32_t m, GhostGeom g, const uint32_t *off,
                                uint32_t dst0) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    uint32_t i = from + k;
    double4_32a p = pos[i];
    uint32_t o = dst0 + off[k];
    if (p.y < g.lo[1]) {
        double4_32a q = p;
        q.y = q.y + g.len1;
        pos[o] = q; vel[o] = vel[i]; type[o] = type[i];
        ++o;
    }
    if (p.y > g.hi[1]) {
        double4_32a q = p;
        q.y = q.y - g.len1;
        pos[o] = q; vel[o] = vel[i]; type[o] = type[i];
    }
}

// exact number of ghosts of all kinds (order independent), to size buffers before writing
__global__ void k_ghost_total(const double4_32a *pos, uint32_t n, GhostGeom g, unsigned long long *tot) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned c = 0;
    if (i < n) {
        double4_32a p = pos[i];
        if (p.x > g.hi[0]) {
            double ny = p.y + g.shear_dt;
            double y = ny - (double)(int)((ny - g.box_min1) / g.len1) * g.len1;
            c += 1 + (y < g.lo[1] ? 1 : 0) + (y > g.hi[1] ? 1 : 0);
        }
        if (p.x < g.lo[0]) {
            double ny = p.y - g.shear_dt;
            double y = ny + (double)(int)((g.box_max1 - ny) / g.len1) * g.len1;
            c += 1 + (y < g.lo[1] ? 1 : 0) + (y > g.hi[1] ? 1 : 0);
        }
        c += (p.y < g.lo[1] ? 1 : 0) + (p.y > g.hi[1] ? 1 : 0);
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(tot, (unsigned long long)c);
}

// ---------------------------------------------------------------- box and keys
__global__ void k_minmax(const double4_32a *pos, uint32_t n, double *out /* per block: 6 */) {
    __shared__ double s[6][256];
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double4_32a p = pos[i];
        mn[0] = fmin(mn[0], p.x); mn[1] = fmin(mn[1], p.y); mn[2] = fmin(mn[2], p.z);
        mx[0] = fmax(mx[0], p.x); mx[1] = fmax(mx[1], p.y); mx[2] = fmax(mx[2], p.z);
    }
    for (int d = 0; d < 3; ++d) { s[d][threadIdx.x] = mn[d]; s[3 + d][threadIdx.x] = mx[d]; }
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st)
            for (int d = 0; d < 3; ++d) {
                s[d][threadIdx.x] = fmin(s[d][threadIdx.x], s[d][threadIdx.x + st]);
                s[3 + d][threadIdx.x] = fmax(s[3 + d][threadIdx.x], s[3 + d][threadIdx.x + st]);
            }
        __syncthreads();
    }
    if (threadIdx.x < 6) out[blockIdx.x * 6 + threadIdx.x] = s[threadIdx.x][0];
}

__device__ inline void morton_of(const TreeBox &b, double x, double y, double z, uint32_t &w0, uint32_t &w1, uint32_t &w2) {
    double s[3] = {x - b.boxmin[0], y - b.boxmin[1], z - b.boxmin[2]};
    w0 = w1 = w2 = 0;
    for (int d = 0; d < 3; ++d) {
        double sd = s[d] * b.scale[d];
        uint32_t u = double_to_cell(sd);
        uint32_t a0, a1, a2;
        dilate3(u, a0, a1, a2);
        // shift the 96-bit dilated value left by d
        uint32_t c0 = a0 << d, c1 = (a1 << d) | (d ? a0 >> (32 - d) : 0u), c2 = (a2 << d) | (d ? a1 >> (32 - d) : 0u);
        w0 |= c0; w1 |= c1; w2 |= c2;
    }
}

__global__ void k_keys(double4_32a *pos, const uint32_t *type, uint32_t n, TreeBox b, MassTable mt, uint32_t *kw0, uint32_t *kw1,
                       uint32_t *kw2, uint32_t *kidx, unsigned *err) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double4_32a p = pos[i];
    uint32_t t = type ? type[i] : 0u;
    if (t >= mt.ntypes) { atomicOr(err, (unsigned)kDevErrCapacity); t = 0; }
    p.w = mt.m[t];
    pos[i] = p;
    uint32_t a, bb, c;
    morton_of(b, p.x, p.y, p.z, a, bb, c);
    kw0[i] = a; kw1[i] = bb; kw2[i] = c & 0xffffffffu;
    kidx[i] = i;
}

__global__ void k_keys_keep_mass(const double4_32a *pos, uint32_t n, TreeBox b, uint32_t *kw0, uint32_t *kw1, uint32_t *kw2, uint32_t *kidx) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double4_32a p = pos[i];
    uint32_t a, bb, c;
    morton_of(b, p.x, p.y, p.z, a, bb, c);
    kw0[i] = a; kw1[i] = bb; kw2[i] = c;
    kidx[i] = i;
}

// run starts among sorted keys (96-bit equality)
__global__ void k_run_flags(const uint32_t *kw0, const uint32_t *kw1, const uint32_t *kw2, uint32_t n, uint32_t *flag) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    flag[i] = (i == 0 || kw0[i] != kw0[i - 1] || kw1[i] != kw1[i - 1] || kw2[i] != kw2[i - 1]) ? 1u : 0u;
}

__global__ void k_run_starts(const uint32_t *flag, const uint32_t *rank, uint32_t n, uint32_t *starts) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (flag[i]) starts[rank[i]] = i;
}

// SortPoints + MakeSinkParticle (src/tree.hpp:2591-2651): one thread per tree point.
__global__ void k_sortpoints(const uint32_t *starts, uint32_t Tu, uint32_t T, const uint32_t *kidx, const uint32_t *kw0,
                             const uint32_t *kw1, const uint32_t *kw2, const double4_32a *in_pos, const double4_32a *in_vel, double4_32a *pos,
                             double4_32a *vel, uint32_t *orig, uint32_t *tk0, uint32_t *tk1, uint32_t *tk2, uint32_t *sink_n,
                             uint32_t *sink_first) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= Tu) return;
    uint32_t j = starts[t], e = (t + 1 < Tu) ? starts[t + 1] : T;
    uint32_t src = kidx[j];
    double4_32a p = in_pos[src], v = in_vel[src];
    if (e - j > 1) {
        double mass = 0.0, vx = 0.0, vy = 0.0, vz = 0.0;
        for (uint32_t k = j; k < e; ++k) {
            double4_32a q = in_pos[kidx[k]], w = in_vel[kidx[k]];
            vx = vx + q.w * w.x;
            vy = vy + q.w * w.y;
            vz = vz + q.w * w.z;
            mass = mass + q.w;
        }
        p.w = mass;
        v.x = vx / mass; v.y = vy / mass; v.z = vz / mass;
    }
    pos[t] = p;
    vel[t] = v;
    orig[t] = src;  // particle ids equal the input-order index (src/tree.hpp:1558-1560, 1660)
    tk0[t] = kw0[j]; tk1[t] = kw1[j]; tk2[t] = kw2[j];
    sink_n[t] = e - j;
    sink_first[t] = j;
}

// ---------------------------------------------------------------- octree
// LEAF = max_leaf_size: 8 by default, 64 for the particle tree of --Density_Vs_Scale runs
template <uint32_t LEAF>
__global__ void k_lcp(const uint32_t *k0, const uint32_t *k1, const uint32_t *k2, uint32_t n, uint8_t *lcp_prev, uint8_t *win) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    lcp_prev[i] = octree_prev_lcp(k0, k1, k2, i);
    win[i] = octree_window_lcp<LEAF>(k0, k1, k2, n, i);  // the (LEAF + 1)-key window starting at i
}

// leaf digit level (CountNodesLeaves' count > max_leaf_size rule, src/tree.hpp:2674)
template <uint32_t LEAF>
__global__ void k_leaf_level(const uint8_t *win, uint32_t n, uint8_t *leaf_lvl) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    leaf_lvl[i] = octree_leaf_level<LEAF>(win, i);
}

__global__ void k_level_block_counts(const uint8_t *lcp_prev, const uint8_t *leaf_lvl, uint32_t n, uint32_t *bc /* [nb][32] */) {
    __shared__ uint32_t s[32];
    if (threadIdx.x < 32) s[threadIdx.x] = 0;
    __syncthreads();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    int a = 32, l = 0;
    if (i < n) { a = lcp_prev[i]; l = leaf_lvl[i]; }
    for (int L = 1; L < 32; ++L) {
        unsigned b = __ballot_sync(0xffffffffu, starts_level(L, a, l));
        if ((threadIdx.x & 31) == 0 && b) atomicAdd(&s[L], (uint32_t)__popc(b));
    }
    __syncthreads();
    if (threadIdx.x < 32) bc[(size_t)blockIdx.x * 32 + threadIdx.x] = s[threadIdx.x];
}

// per level: exclusive scan over blocks; totals to level_count[L]
__global__ void k_level_scan(uint32_t *bc, uint32_t nb, uint32_t *level_count) {
    int L = blockIdx.x;
    __shared__ uint32_t carry;
    __shared__ uint32_t warp_sums[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t start = 0; start < nb; start += blockDim.x) {
        uint32_t b = start + threadIdx.x;
        uint32_t v = b < nb ? bc[(size_t)b * 32 + L] : 0;
        int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        uint32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[w] = x;
        __syncthreads();
        if (w == 0) {
            uint32_t q = lane < (int)(blockDim.x / 32) ? warp_sums[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, q, o);
                if (lane >= o) q += y;
            }
            warp_sums[lane] = q;
        }
        __syncthreads();
        uint32_t excl = x - v + (w ? warp_sums[w - 1] : 0) + carry;
        if (b < nb) bc[(size_t)b * 32 + L] = excl;
        uint32_t tot = warp_sums[blockDim.x / 32 - 1];
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) level_count[L] = carry;
}

struct LevelBase {
    uint32_t base[33];
};

__global__ void k_nodes(const uint8_t *lcp_prev, const uint8_t *leaf_lvl, const uint32_t *k0, const uint32_t *k1, const uint32_t *k2,
                        uint32_t n, const uint32_t *bc, LevelBase lb, TreeBox box, double4_32a *ncf, uint32_t *nbeg, uint32_t *npar,
                        uint32_t *nfd, uint32_t *nnd, uint8_t *north, uint8_t *nlev, uint32_t *leaf_of, uint32_t nn, unsigned *err) {
    __shared__ uint32_t s_cnt[32][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    int a = 32, l = 0;
    if (i < n) { a = lcp_prev[i]; l = leaf_lvl[i]; }
    for (int L = 1; L < 32; ++L) {
        unsigned b = __ballot_sync(0xffffffffu, starts_level(L, a, l));
        if (lane == 0) s_cnt[L][warp] = __popc(b);
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t run = 0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) {
            uint32_t c = s_cnt[threadIdx.x][w];
            s_cnt[threadIdx.x][w] = run;
            run += c;
        }
    }
    __syncthreads();
    if (i == 0) {  // root (src/tree.hpp:2872-2881)
        ncf[0] = make_double4_32a(box.root_center[0], box.root_center[1], box.root_center[2], box.half_width);
        nbeg[0] = 0;
        npar[0] = 0xffffffffu;
        nfd[0] = lb.base[1];
        north[0] = 0;
        nlev[0] = 1;
    }
    double c[3] = {box.root_center[0], box.root_center[1], box.root_center[2]};
    double hw = box.half_width;
    uint32_t prev_idx = 0;
    const unsigned lt = (1u << lane) - 1u;
    for (int L = 1; L < 32; ++L) {
        bool st = starts_level(L, a, l);
        unsigned b = __ballot_sync(0xffffffffu, st);
        if (i >= n) continue;
        uint32_t excl = bc[(size_t)blockIdx.x * 32 + L] + s_cnt[L][warp] + __popc(b & lt);
        if (L > l) continue;
        int dg = key_digit(k0[i], k1[i], k2[i], L);
        hw = 0.5 * hw;
        for (int d = 0; d < 3; ++d) c[d] = c[d] + hw * (double)(((dg >> d) & 1) ? 1 : -1);
        if (L == l) {
            uint32_t lf = lb.base[L] + excl - (st ? 0u : 1u);
            if (lf < nn) leaf_of[i] = lf;
            else atomicOr(err, (unsigned)kDevErrBadNode);
        }
        if (L == a && a > 0) prev_idx = lb.base[a] + excl - 1;  // parent of this point's first node
        if (!st) continue;
        uint32_t idx = lb.base[L] + excl;
        uint32_t parent = (L == a + 1) ? (a == 0 ? 0u : prev_idx) : prev_idx;
        if (idx >= nn || parent >= nn) {  // inconsistent counts: record, never write out of range
            atomicOr(err, (unsigned)kDevErrBadNode);
            continue;
        }
        ncf[idx] = make_double4_32a(c[0], c[1], c[2], hw);
        nbeg[idx] = i;
        npar[idx] = parent;
        north[idx] = (uint8_t)dg;
        nlev[idx] = (uint8_t)(L + 1);
        nfd[idx] = 0;
        if (L > a + 1) nfd[prev_idx] = idx;  // this node is the first daughter of its parent
        atomicAdd(&nnd[parent], 1u);
        prev_idx = idx;
    }
}

// node ends, one tree level at a time from the top: the next sibling's begin, or the
// parent's end for the last daughter
__global__ void k_node_end_level(uint32_t first, uint32_t count, const uint32_t *nbeg, const uint32_t *npar, const uint32_t *nfd,
                                 const uint32_t *nnd, uint32_t *nend, uint32_t nn, unsigned *err) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    uint32_t idx = first + k;
    uint32_t p = npar[idx];
    if (p >= nn || idx + 1 > nn) {
        atomicOr(err, (unsigned)kDevErrBadNode);
        return;
    }
    nend[idx] = (idx + 1 < nfd[p] + nnd[p] && idx + 1 < nn) ? nbeg[idx + 1] : nend[p];
}

}  // namespace

// Keys, radix sort, sink folding and the octree for T points given in input order with
// their masses in pos.w (or from the type table). Used for the particle tree and for the
// clump trees of the merge sweeps (src/tree.hpp:2759-2908, 5251-5284). Buffers kept by
// the tree come from the snapshot arena; temporaries from the scratch arena, released on
// return.
int build_octree(Context &c, double4_32a *in_pos, double4_32a *in_vel, const uint32_t *in_type, uint32_t T, const TreeBox &box,
                 const double *mass_table, uint32_t ntypes, DevTree &tr, cudaStream_t s, cudaEvent_t after_sort, uint32_t leaf) {
    if (leaf != 8 && leaf != 64) return kErrArgument;
    Arena &A = c.arena;
    Arena &S = c.scratch;
    const size_t mark = S.used;
    struct Restore { Arena &a; size_t m; ~Restore() { a.used = m; } } restore{S, mark};
    uint32_t *kw0 = A.get<uint32_t>(T + 1), *kw1 = A.get<uint32_t>(T + 1), *kw2 = A.get<uint32_t>(T + 1), *kidx = A.get<uint32_t>(T + 1);
    uint32_t *d_tot = A.get<uint32_t>(4);
    if (A.failed) return kErrOutOfMemory;
    size_t sort_bytes = std::max(radix_sort96_scratch_bytes(T), scan_u32_scratch_bytes(T));
    void *scr = S.take(sort_bytes);
    uint32_t *flag = S.get<uint32_t>(T + 1);
    if (!scr || !flag) return kErrOutOfMemory;
    MassTable mt;
    mt.ntypes = ntypes ? ntypes : 1;
    for (int t = 0; t < 16; ++t) mt.m[t] = mass_table ? mass_table[t] : 0.0;
    if (mass_table) {
        k_keys<<<grid_for(T, 256), 256, 0, s>>>(in_pos, in_type, T, box, mt, kw0, kw1, kw2, kidx, c.d_err);
    } else {
        k_keys_keep_mass<<<grid_for(T, 256), 256, 0, s>>>(in_pos, T, box, kw0, kw1, kw2, kidx);
    }
    c.launches++;
    int rc = radix_sort96(kw0, kw1, kw2, kidx, T, scr, sort_bytes, s);
    if (rc) return rc;
    c.launches += 36;
    if (after_sort) cudaEventRecord(after_sort, s);

    // sink folding (src/tree.hpp:2608-2651)
    k_run_flags<<<grid_for(T, 256), 256, 0, s>>>(kw0, kw1, kw2, T, flag);
    uint32_t *rank = S.get<uint32_t>(T + 1);
    uint32_t *starts = S.get<uint32_t>(T + 1);
    if (!rank || !starts) return kErrOutOfMemory;
    rc = scan_u32(flag, rank, T, d_tot, scr, sort_bytes, s);
    if (rc) return rc;
    k_run_starts<<<grid_for(T, 256), 256, 0, s>>>(flag, rank, T, starts);
    uint32_t Tu = 0;
    PLAN_CUDA(cudaMemcpyAsync(&Tu, d_tot, 4, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaStreamSynchronize(s));
    c.launches += 5;
    if (Tu < T) {
        // Repeated keys: which particle represents a sink, and the order its velocities are
        // summed in, follow the library sort's order of equal keys. Redo the sort from the
        // input order with the introsort of the library; the runs (and Tu) are unchanged.
        if (mass_table) {
            k_keys<<<grid_for(T, 256), 256, 0, s>>>(in_pos, in_type, T, box, mt, kw0, kw1, kw2, kidx, c.d_err);
        } else {
            k_keys_keep_mass<<<grid_for(T, 256), 256, 0, s>>>(in_pos, T, box, kw0, kw1, kw2, kidx);
        }
        c.launches++;
        const size_t mb = morton_sort_scratch_bytes(T);
        void *ms = nullptr;
        PLAN_CUDA(cudaMallocAsync(&ms, mb, s));
        rc = morton_sort_std(c, kw0, kw1, kw2, kidx, T, ms, mb, s);
        cudaFreeAsync(ms, s);
        if (rc) return rc;
        c.counters[19] += 1;  // sorts that took the library order of equal keys
    }
    tr = DevTree();
    tr.T = T;
    tr.Tu = Tu;
    tr.box = box;
    tr.in_pos = in_pos;
    tr.in_vel = in_vel;
    tr.sorted_src = kidx;
    tr.pos = A.get<double4_32a>(Tu);
    tr.vel = A.get<double4_32a>(Tu);
    tr.dens = A.get<double>(Tu);
    tr.orig = A.get<uint32_t>(Tu);
    tr.tk0 = A.get<uint32_t>(Tu);
    tr.tk1 = A.get<uint32_t>(Tu);
    tr.tk2 = A.get<uint32_t>(Tu);
    tr.sink_n = A.get<uint32_t>(Tu);
    tr.sink_first = A.get<uint32_t>(Tu);
    tr.leaf_of = A.get<uint32_t>(Tu);
    if (A.failed) return kErrOutOfMemory;
    k_sortpoints<<<grid_for(Tu, 256), 256, 0, s>>>(starts, Tu, T, kidx, kw0, kw1, kw2, in_pos, in_vel, tr.pos, tr.vel, tr.orig, tr.tk0,
                                                   tr.tk1, tr.tk2, tr.sink_n, tr.sink_first);
    c.launches++;
    tr.nsinks = T - Tu;
    tr.leaf_size = leaf;

    // octree (src/tree.hpp:2848-2886)
    uint8_t *lcp_prev = S.get<uint8_t>(Tu), *win = S.get<uint8_t>(Tu), *leaf_lvl = S.get<uint8_t>(Tu);
    const uint32_t nb = grid_for(Tu, 256);
    uint32_t *bc = S.get<uint32_t>((size_t)nb * 32);
    uint32_t *d_lc = S.get<uint32_t>(32);
    if (!lcp_prev || !win || !leaf_lvl || !bc || !d_lc) return kErrOutOfMemory;
    if (leaf == 64) {
        k_lcp<64><<<nb, 256, 0, s>>>(tr.tk0, tr.tk1, tr.tk2, Tu, lcp_prev, win);
        k_leaf_level<64><<<nb, 256, 0, s>>>(win, Tu, leaf_lvl);
    } else {
        k_lcp<8><<<nb, 256, 0, s>>>(tr.tk0, tr.tk1, tr.tk2, Tu, lcp_prev, win);
        k_leaf_level<8><<<nb, 256, 0, s>>>(win, Tu, leaf_lvl);
    }
    k_level_block_counts<<<nb, 256, 0, s>>>(lcp_prev, leaf_lvl, Tu, bc);
    PLAN_CUDA(cudaMemsetAsync(d_lc, 0, 32 * 4, s));
    k_level_scan<<<32, 1024, 0, s>>>(bc, nb, d_lc);
    uint32_t lc[32];
    PLAN_CUDA(cudaMemcpyAsync(lc, d_lc, sizeof(lc), cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaStreamSynchronize(s));
    c.launches += 4;
    LevelBase lb;
    lb.base[0] = 0;
    uint32_t run = 1;  // the root
    for (int L = 1; L < 32; ++L) { lb.base[L] = run; run += lc[L]; }
    lb.base[32] = run;
    const uint32_t nn = run;
    tr.nodes = nn;
    tr.ncf = A.get<double4_32a>(nn);
    tr.nbeg = A.get<uint32_t>(nn);
    tr.nend = A.get<uint32_t>(nn);
    tr.npar = A.get<uint32_t>(nn);
    tr.nfd = A.get<uint32_t>(nn);
    uint32_t *nnd32 = A.get<uint32_t>(nn);
    tr.north = A.get<uint8_t>(nn);
    tr.nlev = A.get<uint8_t>(nn);
    if (A.failed) return kErrOutOfMemory;
    PLAN_CUDA(cudaMemsetAsync(nnd32, 0, (size_t)nn * 4, s));
    PLAN_CUDA(cudaMemsetAsync(tr.nfd, 0, (size_t)nn * 4, s));
    PLAN_CUDA(cudaMemsetAsync(tr.npar, 0, (size_t)nn * 4, s));
    PLAN_CUDA(cudaMemsetAsync(tr.nbeg, 0, (size_t)nn * 4, s));
    PLAN_CUDA(cudaMemsetAsync(tr.nend, 0, (size_t)nn * 4, s));
    PLAN_CUDA(cudaMemsetAsync(tr.leaf_of, 0, (size_t)Tu * 4, s));
    k_nodes<<<nb, 256, 0, s>>>(lcp_prev, leaf_lvl, tr.tk0, tr.tk1, tr.tk2, Tu, bc, lb, box, tr.ncf, tr.nbeg, tr.npar, tr.nfd, nnd32,
                               tr.north, tr.nlev, tr.leaf_of, nn, c.d_err);
    PLAN_CUDA(cudaMemcpyAsync(tr.nend, &Tu, 4, cudaMemcpyHostToDevice, s));
    c.launches++;
    for (int L = 1; L < 32; ++L) {
        if (!lc[L]) continue;
        k_node_end_level<<<grid_for(lc[L], 256), 256, 0, s>>>(lb.base[L], lc[L], tr.nbeg, tr.npar, tr.nfd, nnd32, tr.nend, nn, c.d_err);
        c.launches++;
    }
    PLAN_CUDA(cudaGetLastError());
    tr.nnd = reinterpret_cast<uint8_t *>(nnd32);  // num_daughters kept as u32
    unsigned h_err = 0;
    PLAN_CUDA(cudaMemcpyAsync(&h_err, c.d_err, 4, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaStreamSynchronize(s));
    if (h_err & kDevErrBadNode) {
        c.last_error = "octree construction produced inconsistent node indices";
        return kErrDeviceLimit;
    }
    return kOk;
}

// Box of a tree whose root is given (BuildTree with check_pos = false, src/tree.hpp:2798-2804,
// 2824-2825).
TreeBox make_box(const double center[3], double half_width) {
    TreeBox box;
    box.half_width = half_width;
    for (int d = 0; d < 3; ++d) {
        box.root_center[d] = center[d];
        box.boxmin[d] = center[d] - half_width;
        double bmax = center[d] + half_width;
        box.scale[d] = 1.0 / (bmax - box.boxmin[d]);
    }
    box.epsilon = 2 * half_width / std::pow(2, 31);
    return box;
}

// ------------------------------------------------------------------ host side of stage 1
int build_tree(Context &c, const plan_lis_view &v, plan_params &p, int first_file, cudaStream_t s) {
    cudaEvent_t ev[6];
    for (auto &e : ev) cudaEventCreate(&e);
    cudaEventRecord(ev[0], s);
    uint64_t N64 = 0;
    for (uint32_t b = 0; b < v.nblocks; ++b) N64 += v.counts[b];
    if (N64 == 0) {
        c.last_error = "the snapshot holds no particles";
        return kErrUnsupported;
    }
    if (N64 >= 0xfffffff0ull) return kErrUnsupported;
    uint32_t N = (uint32_t)N64;  // the particles that take part (after the user box)
    c.n_input = N;
    c.time = v.time;
    // phase A (scratch arena): raw records and the unpacked particles in file order
    c.scratch.used = 0;
    c.scratch.failed = false;
    Arena &S = c.scratch;
    unsigned char *d_rec = S.get<unsigned char>((size_t)N * 44);
    double4_32a *tmp_pos = S.get<double4_32a>(N), *tmp_vel = S.get<double4_32a>(N);
    uint32_t *tmp_type = S.get<uint32_t>(N);
    uint32_t *aw0 = S.get<uint32_t>(N), *aw1 = S.get<uint32_t>(N), *aw2 = S.get<uint32_t>(N), *aidx = S.get<uint32_t>(N);
    unsigned long long *d_desc = S.get<unsigned long long>(4);
    size_t sortA = radix_sort96_scratch_bytes(N);
    void *scrA = S.take(sortA);
    uint32_t *sel_src = nullptr, *sel_rank = nullptr, *sel_tot = nullptr;
    if (p.user_box) {
        sel_src = S.get<uint32_t>(N);
        sel_rank = S.get<uint32_t>(N);
        sel_tot = S.get<uint32_t>(4);
    }
    if (S.failed) return kErrOutOfMemory;

    // 1. upload and unpack; a single block already in device memory is read in place
    const unsigned char *src = d_rec;
    cudaPointerAttributes pa{};
    if (v.nblocks == 1 && cudaPointerGetAttributes(&pa, v.records[0]) == cudaSuccess && pa.type == cudaMemoryTypeDevice &&
        pa.device == c.device) {
        src = static_cast<const unsigned char *>(v.records[0]);
        c.counters[20] = 0;
    } else {
        cudaGetLastError();
        size_t at = 0;
        for (uint32_t b = 0; b < v.nblocks; ++b) {
            PLAN_CUDA(cudaMemcpyAsync(d_rec + at * 44, v.records[b], v.counts[b] * 44, cudaMemcpyDefault, s));
            at += v.counts[b];
        }
        c.counters[20] = (uint64_t)N * 44;  // bytes uploaded
    }
    k_unpack<<<grid_for(N, 256), 256, 0, s>>>(src, N, tmp_pos, tmp_vel, tmp_type, aw0, aw1, aw2, aidx);
    PLAN_CUDA(cudaMemsetAsync(d_desc, 0, 32, s));
    k_count_descents<<<grid_for(N, 256), 256, 0, s>>>(aw0, aw1, N, d_desc);
    c.launches += 2;
    unsigned long long h_desc[2];
    PLAN_CUDA(cudaMemcpyAsync(h_desc, d_desc, 16, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaStreamSynchronize(s));
    if (h_desc[0]) {  // not yet in (cpu_id, id_in_run) order (src/tree.hpp:1552-1557)
        int rc = radix_sort96(aw0, aw1, aw2, aidx, N, scrA, sortA, s, 0x0ffu);
        if (rc) return rc;
        c.launches += 24;
    }
    c.counters[10] = h_desc[1];  // duplicate (cpu_id, id_in_run) pairs: order left stable

    // box and masses from the first snapshot (src/tree.hpp:1564-1583), on the host
    if (first_file || !p.box_set) {
        for (int d = 0; d < 3; ++d) {
            p.box_min[d] = v.coor_lim[6 + 2 * d];
            p.box_max[d] = v.coor_lim[7 + 2 * d];
            p.box_center[d] = (p.box_min[d] + p.box_max[d]) / 2.0;
            p.box_length[d] = p.box_max[d] - p.box_min[d];
        }
        plan_params_derive(&p);
        p.ntypes = v.ntypes;
        double sum = 0;
        for (uint32_t t = 0; t < v.ntypes && t < 16; ++t) { p.mass_fraction_per_species[t] = v.type_info[t]; sum += v.type_info[t]; }
        for (uint32_t t = 0; t < v.ntypes && t < 16; ++t) {
            p.mass_fraction_per_species[t] /= sum;
            p.mass_total_code_units = p.solid_to_gas_ratio * p.box_length[0] * p.box_length[1] * std::sqrt(2. * 3.14159265358979323846);
            p.mass_per_particle[t] = p.mass_fraction_per_species[t] * p.mass_total_code_units / N;
        }
        p.box_set = 1;
    }
    // --Density_Vs_Scale runs build this tree with 64-point leaves, no ghosts and the ghost
    // zone as wide as the box (BasicAnalyses, src/analyses.hpp:29-33, run after the read)
    if (p.density_vs_scale) {
        p.max_ghost_zone_width = p.max_half_width;
        p.no_ghost = 1;
    }
    // user box (src/tree.hpp:1585-1620): an axis given as 0,0 takes the box's extent; a box
    // that holds the whole domain changes nothing; otherwise only the particles inside it
    // take part, keeping their ids and order
    const uint32_t *gather_from = aidx;
    bool selected = false;
    if (p.user_box) {
        UserBox ub;
        bool covers = true;
        for (int d = 0; d < 3; ++d) {
            if (p.user_box_min[d] == 0 && p.user_box_max[d] == 0) {
                p.user_box_min[d] = p.box_min[d];
                p.user_box_max[d] = p.box_max[d];
            }
            ub.lo[d] = p.user_box_min[d];
            ub.hi[d] = p.user_box_max[d];
        }
        for (int d = 0; d < 3; ++d)
            covers = covers && p.box_min[d] >= ub.lo[d] && p.box_min[d] <= ub.hi[d] && p.box_max[d] >= ub.lo[d] && p.box_max[d] <= ub.hi[d];
        if (!covers) {
            // aw0/aw1 (the sort keys) are free after the sort; the sort scratch serves the scan
            k_box_flags<<<grid_for(N, 256), 256, 0, s>>>(aidx, N, tmp_pos, ub, aw0);
            int rc = scan_u32(aw0, aw1, N, sel_tot, scrA, sortA, s);
            if (rc) return rc;
            k_box_compact<<<grid_for(N, 256), 256, 0, s>>>(aidx, N, aw0, aw1, sel_src, sel_rank);
            c.launches += 2;
            uint32_t kept = 0;
            PLAN_CUDA(cudaMemcpyAsync(&kept, sel_tot, 4, cudaMemcpyDeviceToHost, s));
            PLAN_CUDA(cudaStreamSynchronize(s));
            if (kept == 0) {
                c.last_error = "no particle lies inside the user box (-x/-y/-z)";
                return kErrUnsupported;
            }
            N = kept;
            c.n_input = N;
            gather_from = sel_src;
            selected = true;
        }
    }
    GhostGeom g;
    for (int d = 0; d < 3; ++d) {
        double w = p.box_half_width[d] - p.ghost_zone_width[d];
        if (w < 0) w = 0;
        g.lo[d] = p.box_center[d] - w;
        g.hi[d] = p.box_center[d] + w;
    }
    g.box_min1 = p.box_min[1];
    g.box_max1 = p.box_max[1];
    g.len0 = p.box_length[0];
    g.len1 = p.box_length[1];
    g.shear_dt = p.shear_speed * v.time;
    uint64_t G = 0;
    if (!p.no_ghost) {
        // over every particle of the file: an upper bound when a user box keeps fewer
        k_ghost_total<<<grid_for((uint32_t)N64, 256), 256, 0, s>>>(tmp_pos, (uint32_t)N64, g, d_desc + 2);
        PLAN_CUDA(cudaMemcpyAsync(&G, d_desc + 2, 8, cudaMemcpyDeviceToHost, s));
        PLAN_CUDA(cudaStreamSynchronize(s));
        c.launches++;
    }
    const uint64_t Tmax = N64 + G;
    if (Tmax >= 0xfffffff0ull) return kErrUnsupported;
    // phase B (snapshot arena): everything the later stages keep, sized by the exact count
    {
        int erc = c.ensure(c.arena, (size_t)arena_bytes_for(Tmax) + (selected ? (size_t)N * 4 : 0));
        if (erc) return erc;
    }
    c.arena.used = 0;
    c.arena.failed = false;
    Arena &A = c.arena;
    double4_32a *in_pos = A.get<double4_32a>(Tmax), *in_vel = A.get<double4_32a>(Tmax);
    uint32_t *in_type = A.get<uint32_t>(Tmax);
    uint32_t *kw0 = A.get<uint32_t>(Tmax), *kw1 = A.get<uint32_t>(Tmax), *kw2 = A.get<uint32_t>(Tmax), *kidx = A.get<uint32_t>(Tmax);
    uint32_t *d_u32 = A.get<uint32_t>(Tmax + 1);   // counts / offsets
    uint32_t *d_tot = A.get<uint32_t>(4);
    uint32_t *keep_rank = selected ? A.get<uint32_t>(N) : nullptr;  // ids of the kept particles
    if (A.failed) return kErrOutOfMemory;
    k_gather_in<<<grid_for(N, 256), 256, 0, s>>>(gather_from, N, tmp_pos, tmp_vel, tmp_type, in_pos, in_vel, in_type);
    c.launches++;
    if (selected) PLAN_CUDA(cudaMemcpyAsync(keep_rank, sel_rank, (size_t)N * 4, cudaMemcpyDeviceToDevice, s));
    cudaEventRecord(ev[1], s);
    // phase A buffers are dead from here on: the scratch arena is reused
    PLAN_CUDA(cudaStreamSynchronize(s));
    c.scratch.used = 0;
    size_t sort_bytes = std::max(radix_sort96_scratch_bytes(Tmax), scan_u32_scratch_bytes(Tmax));
    void *scr = c.scratch.take(sort_bytes);
    if (!scr) return kErrOutOfMemory;

    // 2. ghosts (src/tree.hpp:1626-1754)
    uint32_t T = N, Gx = 0, Gy = 0;
    if (!p.no_ghost) {
        k_ghost_count_x<<<grid_for(N, 256), 256, 0, s>>>(in_pos, N, g, d_u32);
        int rc = scan_u32(d_u32, d_u32, N, d_tot, scr, sort_bytes, s);
        if (rc) return rc;
        k_ghost_write_x<<<grid_for(N, 256), 256, 0, s>>>(in_pos, in_vel, in_type, N, g, d_u32);
        PLAN_CUDA(cudaMemcpyAsync(&Gx, d_tot, 4, cudaMemcpyDeviceToHost, s));
        PLAN_CUDA(cudaStreamSynchronize(s));
        // y ghosts of the x ghosts, then of the originals
        uint32_t Gy1 = 0, Gy2 = 0;
        if (Gx) {
            k_ghost_count_y<<<grid_for(Gx, 256), 256, 0, s>>>(in_pos, N, Gx, g, d_u32);
            rc = scan_u32(d_u32, d_u32, Gx, d_tot, scr, sort_bytes, s);
            if (rc) return rc;
            k_ghost_write_y<<<grid_for(Gx, 256), 256, 0, s>>>(in_pos, in_vel, in_type, N, Gx, g, d_u32, N + Gx);
            PLAN_CUDA(cudaMemcpyAsync(&Gy1, d_tot, 4, cudaMemcpyDeviceToHost, s));
            PLAN_CUDA(cudaStreamSynchronize(s));
        }
        k_ghost_count_y<<<grid_for(N, 256), 256, 0, s>>>(in_pos, 0, N, g, d_u32);
        rc = scan_u32(d_u32, d_u32, N, d_tot, scr, sort_bytes, s);
        if (rc) return rc;
        k_ghost_write_y<<<grid_for(N, 256), 256, 0, s>>>(in_pos, in_vel, in_type, 0, N, g, d_u32, N + Gx + Gy1);
        PLAN_CUDA(cudaMemcpyAsync(&Gy2, d_tot, 4, cudaMemcpyDeviceToHost, s));
        PLAN_CUDA(cudaStreamSynchronize(s));
        c.launches += 12;
        Gy = Gy1 + Gy2;
        T = N + Gx + Gy;
        if (T > Tmax) return kErrUnsupported;
    }
    cudaEventRecord(ev[2], s);

    // 3. root box (src/tree.hpp:2763-2804) from the particle extent, on the host
    const int mmb = 152 * 4;
    double *d_mm = c.scratch.get<double>(6 * mmb);
    if (!d_mm) return kErrOutOfMemory;
    k_minmax<<<mmb, 256, 0, s>>>(in_pos, T, d_mm);
    std::vector<double> h_mm(6 * mmb);
    PLAN_CUDA(cudaMemcpyAsync(h_mm.data(), d_mm, 6 * mmb * sizeof(double), cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaStreamSynchronize(s));
    c.launches++;
    double mn[3], mx[3];
    for (int d = 0; d < 3; ++d) { mn[d] = h_mm[d]; mx[d] = h_mm[3 + d]; }
    for (int b = 1; b < mmb; ++b)
        for (int d = 0; d < 3; ++d) { mn[d] = std::min(h_mm[6 * b + d], mn[d]); mx[d] = std::max(h_mm[6 * b + 3 + d], mx[d]); }
    double ext = 0.0;
    for (int d = 0; d < 3; ++d) ext = std::max(ext, mx[d] - mn[d]);
    TreeBox box;
    box.half_width = p.max_half_width + p.max_ghost_zone_width;
    for (int d = 0; d < 3; ++d) box.root_center[d] = p.box_center[d];
    if (ext < box.half_width) {
        box.half_width = (std::ceil(ext * 100.) + 1) / 100.;
        for (int d = 0; d < 3; ++d) {
            if (mx[d] - mn[d] < 0.5 * p.box_length[d]) {
                box.root_center[d] = (mx[d] + mn[d]) / 2.0;
                box.root_center[d] = std::round(box.root_center[d] * 1000.) / 1000.;
            } else {
                box.root_center[d] = p.box_center[d];
            }
        }
    }
    for (int d = 0; d < 3; ++d) {
        box.boxmin[d] = box.root_center[d] - box.half_width;
        double bmax = box.root_center[d] + box.half_width;
        box.scale[d] = 1.0 / (bmax - box.boxmin[d]);
    }
    box.epsilon = 2 * box.half_width / std::pow(2, 31);

    // 4-6. keys, sort, sinks, octree
    {
        MassTable mt;
        mt.ntypes = std::max<uint32_t>(1, std::min<uint32_t>(p.ntypes, 16));
        for (int t = 0; t < 16; ++t) mt.m[t] = p.mass_per_particle[t];
        int rc = build_octree(c, in_pos, in_vel, in_type, T, box, mt.m, mt.ntypes, c.tree, s, ev[3], p.density_vs_scale ? 64u : 8u);
        if (rc) return rc;
    }
    if (selected) {
        k_box_ids<<<grid_for(c.tree.Tu, 256), 256, 0, s>>>(c.tree.orig, c.tree.Tu, N, keep_rank);
        c.launches++;
    }
    cudaEventRecord(ev[4], s);
    PLAN_CUDA(cudaStreamSynchronize(s));
    float ms;
    cudaEventElapsedTime(&ms, ev[0], ev[1]); c.stage_ms[0] = ms;
    cudaEventElapsedTime(&ms, ev[1], ev[2]); c.stage_ms[1] = ms;
    cudaEventElapsedTime(&ms, ev[2], ev[3]); c.stage_ms[2] = ms;
    cudaEventElapsedTime(&ms, ev[3], ev[4]); c.stage_ms[3] = ms;
    for (auto &e : ev) cudaEventDestroy(e);
    c.counters[0] = N;
    c.counters[1] = T;
    c.counters[2] = c.tree.Tu;
    c.counters[3] = c.tree.nodes;
    c.counters[4] = T - c.tree.Tu;
    return kOk;
}

}  // namespace plan

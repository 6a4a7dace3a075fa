// HOP groups from densest-neighbour pointers (src/tree.hpp:3766-3809).
//
// Pointers only climb in (density, -index), so they form a forest whose roots are the peaks.
// The reference walks chains serially in index order and appends each newly met chain
// segment to its peak's member list; that order feeds later floating-point sums, so it is
// reproduced exactly: a member j is appended during the walk that starts at
//   s(j) = the smallest index in j's subtree (the first walk that passes through j),
// and within one walk in chain order, i.e. by decreasing depth. Members are therefore
// sorted by (root, s, -depth). Roots and depths come from synchronous pointer jumping,
// s from concurrent atomicMin walks that stop once a smaller index already passed.
#include "pipeline.h"
#include "sort.h"
#include "hop.h"

namespace plan {

namespace {

__global__ void k_hop_init(const uint32_t *densest, const double *dens, double thr, uint32_t n, uint32_t *nxt, uint32_t *dep,
                           uint32_t *smin, uint32_t *above) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    bool a = dens[i] >= thr;
    above[i] = a ? 1u : 0u;
    nxt[i] = densest[i];
    dep[i] = (densest[i] == i || !a) ? 0u : 1u;
    smin[i] = 0xffffffffu;
}

// one synchronous pointer-jumping round (Wyllie): reads old arrays, writes new ones
__global__ void k_hop_jump(const uint32_t *nxt, const uint32_t *dep, uint32_t *nxt2, uint32_t *dep2, uint32_t n, unsigned *changed) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t j = nxt[i];
    uint32_t jj = nxt[j];
    nxt2[i] = jj;
    dep2[i] = dep[i] + (j != i ? dep[j] : 0u);
    if (jj != j) *changed = 1u;
}

__global__ void k_hop_smin(const uint32_t *densest, const uint32_t *above, uint32_t n, uint32_t *smin, unsigned *err) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !above[i]) return;
    uint32_t j = i;
    for (uint32_t guard = 0; guard <= n; ++guard) {
        uint32_t old = atomicMin(&smin[j], i);
        if (old <= i) return;        // a smaller start passed here and continues upward
        uint32_t p = densest[j];
        if (p == j) return;          // reached the peak
        j = p;
    }
    atomicOr(err, (unsigned)kDevErrLoopLimit);
}

__global__ void k_hop_keys(const uint32_t *above, const uint32_t *pos_of, const uint32_t *root, const uint32_t *smin, const uint32_t *dep,
                           uint32_t n, uint32_t *w0, uint32_t *w1, uint32_t *w2, uint32_t *payload) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !above[i]) return;
    uint32_t o = pos_of[i];
    w2[o] = root[i];
    w1[o] = smin[i];
    w0[o] = 0xffffffffu - dep[i];
    payload[o] = i;
}

__global__ void k_group_flags(const uint32_t *w2, uint32_t m, uint32_t *flag) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    flag[k] = (k == 0 || w2[k] != w2[k - 1]) ? 1u : 0u;
}

__global__ void k_group_table(const uint32_t *flag, const uint32_t *rank, const uint32_t *w2, uint32_t m, uint32_t *g_key, uint32_t *g_off) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m || !flag[k]) return;
    uint32_t g = rank[k];
    g_key[g] = w2[k];
    g_off[g] = k;
}

}  // namespace

int hop_groups(Context &c, const uint32_t *densest, double thr, HopGroups &out, cudaStream_t s) {
    const uint32_t n = c.tree.Tu;
    Arena &A = c.arena;
    uint32_t *nxt = A.get<uint32_t>(n), *dep = A.get<uint32_t>(n), *nxt2 = A.get<uint32_t>(n), *dep2 = A.get<uint32_t>(n);
    uint32_t *smin = A.get<uint32_t>(n), *above = A.get<uint32_t>(n), *pos_of = A.get<uint32_t>(n);
    unsigned *d_changed = A.get<unsigned>(4);
    uint32_t *d_tot = A.get<uint32_t>(4);
    if (A.failed) return kErrOutOfMemory;
    const unsigned g = grid_for(n, 256);
    k_hop_init<<<g, 256, 0, s>>>(densest, c.tree.dens, thr, n, nxt, dep, smin, above);
    c.launches++;
    for (int round = 0; round < 40; ++round) {
        PLAN_CUDA(cudaMemsetAsync(d_changed, 0, 4, s));
        k_hop_jump<<<g, 256, 0, s>>>(nxt, dep, nxt2, dep2, n, d_changed);
        c.launches++;
        std::swap(nxt, nxt2);
        std::swap(dep, dep2);
        unsigned h = 0;
        PLAN_CUDA(cudaMemcpyAsync(&h, d_changed, 4, cudaMemcpyDeviceToHost, s));
        PLAN_CUDA(cudaStreamSynchronize(s));
        if (!h) break;
        if (round == 39) return kErrDeviceLimit;
    }
    k_hop_smin<<<g, 256, 0, s>>>(densest, above, n, smin, c.d_err);
    c.launches++;
    // compact the above-threshold points and sort them by (root, s, -depth)
    c.scratch.used = 0;
    c.scratch.failed = false;
    size_t scan_b = scan_u32_scratch_bytes(n);
    void *scr = c.scratch.take(scan_b);
    if (!scr) return kErrOutOfMemory;
    int rc = scan_u32(above, pos_of, n, d_tot, scr, scan_b, s);
    if (rc) return rc;
    uint32_t m = 0;
    PLAN_CUDA(cudaMemcpyAsync(&m, d_tot, 4, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaStreamSynchronize(s));
    out.n_members = m;
    out.members = A.get<uint32_t>(m ? m : 1);
    uint32_t *w0 = c.scratch.get<uint32_t>(m + 1), *w1 = c.scratch.get<uint32_t>(m + 1), *w2 = c.scratch.get<uint32_t>(m + 1);
    if (A.failed || c.scratch.failed) return kErrOutOfMemory;
    k_hop_keys<<<g, 256, 0, s>>>(above, pos_of, nxt, smin, dep, n, w0, w1, w2, out.members);
    c.launches++;
    size_t sb = radix_sort96_scratch_bytes(m);
    void *scr2 = c.scratch.take(sb);
    if (!scr2) return kErrOutOfMemory;
    rc = radix_sort96(w0, w1, w2, out.members, m, scr2, sb, s);
    if (rc) return rc;
    c.launches += 36;
    // group table: one entry per root, ascending (the std::map order of src/tree.hpp:4855)
    uint32_t *flag = c.scratch.get<uint32_t>(m + 1), *rank = c.scratch.get<uint32_t>(m + 1);
    void *scr3 = c.scratch.take(scan_u32_scratch_bytes(m + 1));
    if (!flag || !rank || !scr3) return kErrOutOfMemory;
    k_group_flags<<<grid_for(m, 256), 256, 0, s>>>(w2, m, flag);
    rc = scan_u32(flag, rank, m, d_tot, scr3, scan_u32_scratch_bytes(m + 1), s);
    if (rc) return rc;
    uint32_t ng = 0;
    PLAN_CUDA(cudaMemcpyAsync(&ng, d_tot, 4, cudaMemcpyDeviceToHost, s));
    PLAN_CUDA(cudaStreamSynchronize(s));
    out.n_groups = ng;
    out.key = A.get<uint32_t>(ng + 1);
    out.off = A.get<uint32_t>(ng + 1);
    if (A.failed) return kErrOutOfMemory;
    k_group_table<<<grid_for(m, 256), 256, 0, s>>>(flag, rank, w2, m, out.key, out.off);
    PLAN_CUDA(cudaMemcpyAsync(out.off + ng, &m, 4, cudaMemcpyHostToDevice, s));
    c.launches += 2;
    out.peak = nxt;  // root per tree point (valid for above-threshold points)
    out.above = above;
    PLAN_CUDA(cudaGetLastError());
    return kOk;
}

}  // namespace plan

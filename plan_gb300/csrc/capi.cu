// C entry points (include/plan_gpu.h): context management, the BuildTree and
// FindPlanetesimals seams, and inspection of stage arrays.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "catalogue.h"
#include "hop.h"
#include "pipeline.h"
#include "sort.h"

namespace plan {

thread_local Context *g_ctx = nullptr;

// The fixed device array of plan_morton_order_noalloc: the keys (4 x u32 per key) and the sort
// scratch of up to PLAN_NOALLOC_SORT_MAX keys. Nothing in it has to start at zero (every call
// writes what it later reads); calls on one device share it and must not overlap.
constexpr size_t kNoAllocBytes = 6u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

int set_cuda_error(cudaError_t e, const char *what, const char *file, int line) {
    if (g_ctx) {
        char buf[512];
        std::snprintf(buf, sizeof(buf), "CUDA error %s (%s) at %s:%d: %s", cudaGetErrorName(e), cudaGetErrorString(e), file, line, what);
        g_ctx->last_error = buf;
    }
    if (e == cudaErrorMemoryAllocation) return kErrOutOfMemory;
    return kErrDevice;
}

int Context::status_from(int rc, const char *what) {
    if (rc != kOk && last_error.empty()) last_error = std::string(what) + ": status " + std::to_string(rc);
    return rc;
}

int Context::ensure(Arena &a, size_t bytes) {
    if (a.cap >= bytes) return kOk;
    if (a.base) cudaFree(a.base);
    a.base = nullptr;
    a.cap = 0;
    a.used = 0;
    size_t want = bytes + bytes / 16 + (64u << 20);
    cudaError_t e = cudaMalloc(&a.base, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        last_error = "device allocation of " + std::to_string(want >> 20) + " MiB failed";
        return kErrOutOfMemory;
    }
    a.cap = want;
    return kOk;
}

// Device bytes for a snapshot of n input particles with the ghost count of a uniform box
// (T = 1.5625 n); the exact count is known, and the arena grown to it, during the build.
static void footprint(uint64_t n, uint64_t &arena, uint64_t &scratch) {
    uint64_t T = n + n * 9 / 16 + 1024;
    arena = arena_bytes_for(T);
    scratch = (4 * n + 1024) * 40 > n * kScratchBytesPerParticle ? (4 * n + 1024) * 40 : n * kScratchBytesPerParticle;
    scratch += 64ull << 20;
}

}  // namespace plan

using namespace plan;

struct plan_ctx {
    Context c;
};

extern "C" {

int plan_ctx_create(int device, plan_ctx **out) {
    if (!out) return kErrArgument;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0 || device < 0 || device >= ndev) {
        cudaGetLastError();
        return kErrDevice;
    }
    plan_ctx *h = new plan_ctx();
    Context &c = h->c;
    g_ctx = &c;
    c.device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&c.d_err, 16) != cudaSuccess || cudaMemset(c.d_err, 0, 16) != cudaSuccess ||
        cudaEventCreate(&c.kev[0]) != cudaSuccess || cudaEventCreate(&c.kev[1]) != cudaSuccess) {
        delete h;
        return kErrDevice;
    }
    *out = h;
    return kOk;
}

void plan_ctx_destroy(plan_ctx *h) {
    if (!h) return;
    Context &c = h->c;
    cudaSetDevice(c.device);
    if (c.stream) cudaStreamSynchronize(c.stream);
    if (c.arena.base) cudaFree(c.arena.base);
    if (c.scratch.base) cudaFree(c.scratch.base);
    if (c.d_err) cudaFree(c.d_err);
    for (auto &e : c.kev)
        if (e) cudaEventDestroy(e);
    if (c.stream) cudaStreamDestroy(c.stream);
    if (g_ctx == &c) g_ctx = nullptr;
    delete h;
}

const char *plan_last_error(const plan_ctx *h) { return h ? h->c.last_error.c_str() : "no context"; }

int plan_ctx_release(plan_ctx *h) {
    if (!h) return kErrArgument;
    Context &c = h->c;
    cudaSetDevice(c.device);
    if (c.stream) cudaStreamSynchronize(c.stream);
    for (Arena *a : {&c.arena, &c.scratch}) {
        if (a->base) cudaFree(a->base);
        a->base = nullptr;
        a->cap = a->used = 0;
        a->failed = false;
    }
    c.tree = DevTree{};
    c.densest = c.peak = nullptr;
    return kOk;
}

uint64_t plan_footprint_bytes(uint64_t n, const plan_params *) {
    uint64_t a, s;
    footprint(n, a, s);
    return a + s;
}

int plan_build_tree(plan_ctx *h, const plan_lis_view *v, plan_params *p, int first_file, void *stream) {
    if (!h || !v || !p) return kErrArgument;
    Context &c = h->c;
    g_ctx = &c;
    c.last_error.clear();
    cudaSetDevice(c.device);
    uint64_t n = 0;
    for (uint32_t b = 0; b < v->nblocks; ++b) n += v->counts[b];
    uint64_t need_a, need_s;
    footprint(n, need_a, need_s);
    if (c.ensure(c.scratch, need_s)) return c.status_from(kErrOutOfMemory, "plan_build_tree");
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c.stream;
    cudaMemsetAsync(c.d_err, 0, 16, s);
    int rc = build_tree(c, *v, *p, first_file, s);
    if (rc == kOk) {
        unsigned err = 0;
        cudaMemcpy(&err, c.d_err, 4, cudaMemcpyDeviceToHost);
        c.counters[9] = err;
        if (err) {
            c.last_error = "device error flags " + std::to_string(err) + " while building the tree";
            rc = kErrDeviceLimit;
        }
    }
    return c.status_from(rc, "plan_build_tree");
}

int plan_find_planetesimals(plan_ctx *h, plan_params *p, void *stream, plan_catalogue **out) {
    if (!h || !p) return kErrArgument;
    Context &c = h->c;
    g_ctx = &c;
    c.last_error.clear();
    cudaSetDevice(c.device);
    if (!c.tree.Tu) return kErrArgument;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c.stream;
    if (out) *out = nullptr;
    cudaMemsetAsync(c.d_err, 0, 16, s);
    int rc = find_planetesimals(c, *p, s, out);
    unsigned err = 0;
    cudaMemcpy(&err, c.d_err, 4, cudaMemcpyDeviceToHost);
    c.counters[9] = err;
    if (rc == kOk && err) {
        c.last_error = "device error flags " + std::to_string(err) + " while finding clumps";
        rc = kErrDeviceLimit;
        if (out && *out) {
            plan_catalogue_free(*out);
            *out = nullptr;
        }
    }
    return c.status_from(rc, "plan_find_planetesimals");
}

int plan_find_clumps(plan_ctx *h, const plan_lis_view *v, plan_params *p, int first_file, void *stream, plan_catalogue **out) {
    int rc = plan_build_tree(h, v, p, first_file, stream);
    if (rc) return rc;
    return plan_find_planetesimals(h, p, stream, out);
}

uint64_t plan_stage_count(const plan_ctx *h, int which) {
    if (!h) return 0;
    const DevTree &t = h->c.tree;
    switch (which) {
    case PLAN_ARR_TREE_POS: case PLAN_ARR_TREE_VEL: case PLAN_ARR_DENSITY: case PLAN_ARR_ORIG_ID: case PLAN_ARR_KEYS:
    case PLAN_ARR_SINK_COUNT:
        return t.Tu;
    case PLAN_ARR_NODE_F: case PLAN_ARR_NODE_U:
        return t.nodes;
    case PLAN_ARR_DENSEST: case PLAN_ARR_PEAK:
        return h->c.densest ? t.Tu : 0;
    default:
        return 0;
    }
}

int plan_stage_copy(plan_ctx *h, int which, void *dst, size_t bytes) {
    if (!h || !dst) return kErrArgument;
    Context &c = h->c;
    g_ctx = &c;
    cudaSetDevice(c.device);
    const DevTree &t = c.tree;
    size_t n = plan_stage_count(h, which);
    if (!n) return kErrArgument;
    auto copy = [&](const void *src, size_t b) -> int {
        if (bytes < b) return kErrArgument;
        PLAN_CUDA(cudaMemcpy(dst, src, b, cudaMemcpyDeviceToHost));
        return kOk;
    };
    switch (which) {
    case PLAN_ARR_TREE_POS: return copy(t.pos, n * 32);
    case PLAN_ARR_TREE_VEL: return copy(t.vel, n * 32);
    case PLAN_ARR_DENSITY: return copy(t.dens, n * 8);
    case PLAN_ARR_ORIG_ID: return copy(t.orig, n * 4);
    case PLAN_ARR_SINK_COUNT: return copy(t.sink_n, n * 4);
    case PLAN_ARR_DENSEST: return copy(c.densest, n * 4);
    case PLAN_ARR_PEAK: {  // points below the density threshold belong to no group (src/tree.hpp:3775-3779)
        if (bytes < n * 4) return kErrArgument;
        std::vector<uint32_t> pk(n);
        std::vector<double> dn(n);
        PLAN_CUDA(cudaMemcpy(pk.data(), c.peak, n * 4, cudaMemcpyDeviceToHost));
        PLAN_CUDA(cudaMemcpy(dn.data(), t.dens, n * 8, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < n; ++i)
            if (dn[i] < c.fs.density_threshold) pk[i] = (uint32_t)n;
        std::memcpy(dst, pk.data(), n * 4);
        return kOk;
    }
    case PLAN_ARR_KEYS: {
        if (bytes < n * 12) return kErrArgument;
        std::vector<uint32_t> a(n), b(n), d(n);
        PLAN_CUDA(cudaMemcpy(a.data(), t.tk0, n * 4, cudaMemcpyDeviceToHost));
        PLAN_CUDA(cudaMemcpy(b.data(), t.tk1, n * 4, cudaMemcpyDeviceToHost));
        PLAN_CUDA(cudaMemcpy(d.data(), t.tk2, n * 4, cudaMemcpyDeviceToHost));
        uint32_t *o = static_cast<uint32_t *>(dst);
        for (size_t i = 0; i < n; ++i) { o[3 * i] = a[i]; o[3 * i + 1] = b[i]; o[3 * i + 2] = d[i]; }
        return kOk;
    }
    case PLAN_ARR_NODE_F: return copy(t.ncf, n * 32);
    case PLAN_ARR_NODE_U: {
        if (bytes < n * 28) return kErrArgument;
        std::vector<uint32_t> b(n), e(n), p(n), fd(n), nd(n);
        std::vector<uint8_t> o(n), l(n);
        PLAN_CUDA(cudaMemcpy(b.data(), t.nbeg, n * 4, cudaMemcpyDeviceToHost));
        PLAN_CUDA(cudaMemcpy(e.data(), t.nend, n * 4, cudaMemcpyDeviceToHost));
        PLAN_CUDA(cudaMemcpy(p.data(), t.npar, n * 4, cudaMemcpyDeviceToHost));
        PLAN_CUDA(cudaMemcpy(fd.data(), t.nfd, n * 4, cudaMemcpyDeviceToHost));
        PLAN_CUDA(cudaMemcpy(nd.data(), t.nnd, n * 4, cudaMemcpyDeviceToHost));
        PLAN_CUDA(cudaMemcpy(o.data(), t.north, n, cudaMemcpyDeviceToHost));
        PLAN_CUDA(cudaMemcpy(l.data(), t.nlev, n, cudaMemcpyDeviceToHost));
        uint32_t *u = static_cast<uint32_t *>(dst);
        for (size_t i = 0; i < n; ++i) {
            u[7 * i] = b[i]; u[7 * i + 1] = e[i]; u[7 * i + 2] = p[i]; u[7 * i + 3] = fd[i];
            u[7 * i + 4] = o[i]; u[7 * i + 5] = nd[i]; u[7 * i + 6] = l[i];
        }
        return kOk;
    }
    default:
        return kErrArgument;
    }
}

int plan_knn(plan_ctx *h, const double *pos3, uint32_t nq, uint32_t k, double est, uint32_t *idx, double *dr2) {
    if (!h || !pos3 || !idx || !dr2) return kErrArgument;
    Context &c = h->c;
    g_ctx = &c;
    cudaSetDevice(c.device);
    c.last_error.clear();
    cudaMemsetAsync(c.d_err, 0, 16, c.stream);
    int rc = knn_positions(c, pos3, nq, k, est, idx, dr2);
    unsigned err = 0;
    cudaMemcpy(&err, c.d_err, 4, cudaMemcpyDeviceToHost);
    if (rc == kOk && (err & kDevErrKey2Leaf)) {
        c.last_error = "a query position has no leaf in the tree (the reference's Key2Leaf failure; its KNN is undefined there)";
        rc = kErrUnsupported;
    } else if (rc == kOk && err) {
        c.last_error = "device error flags " + std::to_string(err) + " in the KNN";
        rc = kErrDeviceLimit;
    }
    return c.status_from(rc, "plan_knn");
}

int plan_morton_order(plan_ctx *h, const uint32_t *keys3, uint32_t n, uint32_t *order) {
    if (!h || (n && (!keys3 || !order))) return kErrArgument;
    Context &c = h->c;
    g_ctx = &c;
    c.last_error.clear();
    cudaSetDevice(c.device);
    if (n == 0) return kOk;
    cudaStream_t s = c.stream;
    std::vector<uint32_t> w(4 * (size_t)n);
    for (uint32_t i = 0; i < n; ++i) {
        w[i] = keys3[3 * (size_t)i];
        w[(size_t)n + i] = keys3[3 * (size_t)i + 1];
        w[2 * (size_t)n + i] = keys3[3 * (size_t)i + 2];
        w[3 * (size_t)n + i] = i;
    }
    uint32_t *d = nullptr;
    void *scr = nullptr;
    const size_t sb = morton_sort_scratch_bytes(n);
    int rc = kOk;
    if (cudaMallocAsync(&d, w.size() * 4, s) != cudaSuccess || cudaMallocAsync(&scr, sb, s) != cudaSuccess) {
        cudaGetLastError();
        rc = kErrOutOfMemory;
    }
    if (!rc && cudaMemcpyAsync(d, w.data(), w.size() * 4, cudaMemcpyHostToDevice, s) != cudaSuccess) rc = kErrDevice;
    if (!rc) rc = morton_sort_std(c, d, d + n, d + 2 * (size_t)n, d + 3 * (size_t)n, n, scr, sb, s);
    if (!rc && cudaMemcpyAsync(order, d + 3 * (size_t)n, (size_t)n * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) rc = kErrDevice;
    if (d) cudaFreeAsync(d, s);
    if (scr) cudaFreeAsync(scr, s);
    if (cudaStreamSynchronize(s) != cudaSuccess && !rc) rc = kErrDevice;
    return c.status_from(rc, "plan_morton_order");
}

int plan_morton_order_noalloc(plan_ctx *h, const uint32_t *keys3, uint32_t n, uint32_t *order) {
    if (!h || (n && (!keys3 || !order))) return kErrArgument;
    Context &c = h->c;
    g_ctx = &c;
    c.last_error.clear();
    cudaSetDevice(c.device);
    if (n == 0) return kOk;
    if (n > PLAN_NOALLOC_SORT_MAX) {
        c.last_error = "plan_morton_order_noalloc: " + std::to_string(n) + " keys exceed the fixed limit of " +
                       std::to_string(PLAN_NOALLOC_SORT_MAX);
        return kErrOutOfMemory;
    }
    const size_t key_bytes = (4 * (size_t)n * 4 + 255) & ~size_t(255), sb = morton_sort_scratch_bytes(n);
    if (key_bytes + sb > kNoAllocBytes) {
        c.last_error = "plan_morton_order_noalloc: the fixed device array is too small for " + std::to_string(n) + " keys";
        return kErrOutOfMemory;
    }
    if (!c.noalloc_scratch) {  // this device's copy of the array, looked up once
        cudaError_t e = cudaGetSymbolAddress(&c.noalloc_scratch, g_noalloc_scratch);
        if (e != cudaSuccess) {
            cudaGetLastError();
            c.noalloc_scratch = nullptr;
            c.last_error = std::string("plan_morton_order_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
            return kErrDevice;
        }
    }
    cudaStream_t s = c.stream;
    std::vector<uint32_t> w(4 * (size_t)n);
    for (uint32_t i = 0; i < n; ++i) {
        w[i] = keys3[3 * (size_t)i];
        w[(size_t)n + i] = keys3[3 * (size_t)i + 1];
        w[2 * (size_t)n + i] = keys3[3 * (size_t)i + 2];
        w[3 * (size_t)n + i] = i;
    }
    uint32_t *d = static_cast<uint32_t *>(c.noalloc_scratch);
    void *scr = static_cast<unsigned char *>(c.noalloc_scratch) + key_bytes;
    int rc = kOk;
    if (cudaMemcpyAsync(d, w.data(), w.size() * 4, cudaMemcpyHostToDevice, s) != cudaSuccess) rc = kErrDevice;
    if (!rc) rc = morton_sort_std(c, d, d + n, d + 2 * (size_t)n, d + 3 * (size_t)n, n, scr, sb, s);
    if (!rc && cudaMemcpyAsync(order, d + 3 * (size_t)n, (size_t)n * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) rc = kErrDevice;
    if (cudaStreamSynchronize(s) != cudaSuccess && !rc) rc = kErrDevice;
    return c.status_from(rc, "plan_morton_order_noalloc");
}

int plan_density_vs_scale(plan_ctx *h, const plan_params *p, double time, double *radii, double *rho, int cap, int *nlev) {
    if (!h || !p || !nlev) return kErrArgument;
    Context &c = h->c;
    g_ctx = &c;
    c.last_error.clear();
    cudaSetDevice(c.device);
    if (!c.tree.Tu || c.tree.leaf_size != 64) {
        c.last_error = "plan_density_vs_scale: no tree built for it (plan_build_tree with density_vs_scale set)";
        return kErrArgument;
    }
    std::vector<double> r, v;
    cudaMemsetAsync(c.d_err, 0, 16, c.stream);
    int rc = density_vs_scale(c, *p, time, r, v, c.stream);
    if (rc == kOk) {
        unsigned err = 0;
        cudaMemcpy(&err, c.d_err, 4, cudaMemcpyDeviceToHost);
        if (err) {
            c.last_error = "device error flags " + std::to_string(err) + " in the ball counts";
            rc = kErrDeviceLimit;
        }
    }
    if (rc == kOk) {
        *nlev = (int)r.size();
        for (int i = 0; i < (int)r.size() && i < cap; ++i) {
            if (radii) radii[i] = r[i];
            if (rho) rho[i] = v[i];
        }
    }
    return c.status_from(rc, "plan_density_vs_scale");
}

int plan_group_energies(plan_ctx *h, const float *pos3, const float *vel3, const float *mass, const uint64_t *offsets, uint32_t ngroups,
                        const plan_params *p, double *e_kin, double *e_pot, uint64_t *zero_pairs) {
    if (!h || !p || !offsets || (ngroups && (!e_kin || !e_pot))) return kErrArgument;
    if (ngroups && offsets[ngroups] && (!pos3 || !vel3 || !mass)) return kErrArgument;
    Context &c = h->c;
    g_ctx = &c;
    c.last_error.clear();
    cudaSetDevice(c.device);
    const int rc = group_energies(c, pos3, vel3, mass, offsets, ngroups, p->grav_constant, p->q * p->Omega, e_kin, e_pot, zero_pairs,
                                  c.stream);
    return c.status_from(rc, "plan_group_energies");
}

int plan_catalogue_write_parlists(plan_ctx *h, const plan_catalogue *cat, int file_number, uint32_t sampling) {
    if (!h || !cat) return kErrArgument;
    Context &c = h->c;
    g_ctx = &c;
    c.last_error.clear();
    cudaSetDevice(c.device);
    int rc = write_parlists_device(c, *cat, file_number, sampling, c.stream);
    return c.status_from(rc, "plan_catalogue_write_parlists");
}

int plan_stage_times(const plan_ctx *h, double *ms, int n) {
    if (!h || !ms) return kErrArgument;
    for (int i = 0; i < n && i < 32; ++i) ms[i] = h->c.stage_ms[i];
    return kOk;
}

uint64_t plan_kernel_launches(const plan_ctx *h) { return h ? h->c.launches : 0; }

int plan_counters(const plan_ctx *h, uint64_t *out, int n) {
    if (!h || !out) return kErrArgument;
    for (int i = 0; i < n && i < 32; ++i) out[i] = h->c.counters[i];
    return kOk;
}

}  // extern "C"

// .lis reader (src/tree.hpp:1303-1535): header parsing on the host, records copied raw
// into page-locked memory so the upload is one DMA per file; unpacking happens on the
// device. Unlike the reference, a file shorter than its declared record count is an I/O
// error instead of a read past the end of the buffer.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "plan_gpu.h"

struct plan_lis {
    plan_lis_view view;
    std::vector<void *> blocks;      // pinned
    std::vector<const void *> ptrs;
    std::vector<uint64_t> counts;
};

namespace {

bool read_header(FILE *f, plan_lis_view &v, int64_t &n) {
    float lim[12], fv;
    if (std::fread(lim, 4, 12, f) != 12) return false;
    for (int i = 0; i < 12; ++i) v.coor_lim[i] = (double)lim[i];
    uint32_t ntypes = 0;
    if (std::fread(&ntypes, 4, 1, f) != 1) return false;
    if (ntypes > 16) return false;
    v.ntypes = ntypes;
    for (uint32_t i = 0; i < ntypes; ++i) {
        if (std::fread(&fv, 4, 1, f) != 1) return false;
        v.type_info[i] = (double)fv;
    }
    if (std::fread(&fv, 4, 1, f) != 1) return false;
    v.time = (double)fv;
    if (std::fread(&fv, 4, 1, f) != 1) return false;
    v.dt = (double)fv;
    if (std::fread(&n, 8, 1, f) != 1) return false;
    return n >= 0;
}

}  // namespace

extern "C" int plan_lis_read(const char *const *paths, int nfiles, plan_lis **out) {
    if (!paths || nfiles <= 0 || !out) return 2;
    *out = nullptr;
    plan_lis *l = new plan_lis();
    std::memset(&l->view, 0, sizeof(l->view));
    for (int k = 0; k < nfiles; ++k) {
        FILE *f = std::fopen(paths[k], "rb");
        if (!f) {
            std::fprintf(stderr, "Error: Failed to open file %s\n", paths[k]);
            plan_lis_free(l);
            return 3;
        }
        int64_t n = 0;
        plan_lis_view hv;
        std::memset(&hv, 0, sizeof(hv));
        bool ok = read_header(f, hv, n);
        if (ok && k == 0) {
            std::memcpy(l->view.coor_lim, hv.coor_lim, sizeof(hv.coor_lim));
            l->view.ntypes = hv.ntypes;
            std::memcpy(l->view.type_info, hv.type_info, sizeof(hv.type_info));
            l->view.time = hv.time;
            l->view.dt = hv.dt;
        }
        void *buf = nullptr;
        if (ok && n > 0) {
            if (cudaMallocHost(&buf, (size_t)n * 44) != cudaSuccess) {
                cudaGetLastError();
                buf = std::malloc((size_t)n * 44);  // unpinned staging still works, slower
                if (!buf) ok = false;
            }
            if (ok && std::fread(buf, 44, (size_t)n, f) != (size_t)n) ok = false;
        }
        std::fclose(f);
        if (!ok) {
            std::fprintf(stderr, "Error: %s is truncated or malformed\n", paths[k]);
            if (buf) {
                if (cudaFreeHost(buf) != cudaSuccess) { cudaGetLastError(); std::free(buf); }
            }
            plan_lis_free(l);
            return 3;
        }
        l->blocks.push_back(buf);
        l->ptrs.push_back(buf);
        l->counts.push_back((uint64_t)n);
    }
    l->view.nblocks = (uint32_t)l->ptrs.size();
    l->view.records = l->ptrs.data();
    l->view.counts = l->counts.data();
    *out = l;
    return 0;
}

extern "C" void plan_lis_free(plan_lis *l) {
    if (!l) return;
    for (void *b : l->blocks) {
        if (b && cudaFreeHost(b) != cudaSuccess) {
            cudaGetLastError();
            std::free(b);
        }
    }
    delete l;
}

extern "C" uint64_t plan_lis_count(const plan_lis *l) {
    uint64_t n = 0;
    if (l) for (uint64_t c : l->counts) n += c;
    return n;
}

extern "C" double plan_lis_time(const plan_lis *l) { return l ? l->view.time : 0.0; }

extern "C" int plan_lis_get_view(const plan_lis *l, plan_lis_view *v) {
    if (!l || !v) return 2;
    *v = l->view;
    return 0;
}

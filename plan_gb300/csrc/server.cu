// The serving loop: plan_submit / plan_poll over a pool of contexts on one device.
//
// Admission and dispatch are ServeQueue's (host/serve_core.hpp). Each worker thread owns one
// context (its own stream and buffers, so requests overlap on the device) and runs a request
// with plan_find_clumps exactly as a caller would alone; the catalogue is handed back by
// plan_poll. The budget counts plan_footprint_bytes per worker hold.
#include <cuda_runtime.h>

#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "host/serve_core.hpp"
#include "pipeline.h"

namespace {

struct Job {
    plan_lis_view view{};
    plan_params params{};
    int first_file = 1;
    plan_catalogue *cat = nullptr;
    std::string error;
};

}  // namespace

struct plan_server {
    int device = 0;
    std::vector<plan_ctx *> ctx;
    std::unique_ptr<plan::ServeQueue> q;
    mutable std::mutex mu;
    std::string error;
};

extern "C" {

int plan_server_create(int device, int workers, uint64_t hbm_budget, plan_server **out) {
    if (!out || workers < 1 || workers > 64) return plan::kErrArgument;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return plan::kErrDevice;
    }
    if (hbm_budget == 0) {
        size_t fr = 0, tot = 0;
        if (cudaSetDevice(device) != cudaSuccess || cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
            cudaGetLastError();
            return plan::kErrDevice;
        }
        hbm_budget = (uint64_t)fr / 10 * 9;
    }
    auto *srv = new plan_server();
    srv->device = device;
    srv->ctx.assign((size_t)workers, nullptr);
    plan_server *S = srv;
    auto init = [S](int w) -> int { return plan_ctx_create(S->device, &S->ctx[(size_t)w]); };
    auto fini = [S](int w) -> int {
        plan_ctx_destroy(S->ctx[(size_t)w]);
        S->ctx[(size_t)w] = nullptr;
        return 0;
    };
    auto release = [S](int w) -> int { return S->ctx[(size_t)w] ? plan_ctx_release(S->ctx[(size_t)w]) : 0; };
    auto run = [S](int w, plan::ServeRequest &r) -> int {
        Job *j = static_cast<Job *>(r.payload);
        plan_ctx *c = S->ctx[(size_t)w];
        if (!c) {
            j->error = "worker context unavailable";
            return plan::kErrDevice;
        }
        const int rc = plan_find_clumps(c, &j->view, &j->params, j->first_file, nullptr, &j->cat);
        if (rc) j->error = plan_last_error(c);
        r.result = j->cat;
        return rc;
    };
    srv->q.reset(new plan::ServeQueue(workers, hbm_budget, 2u * (uint32_t)workers, init, run, release, fini));
    *out = srv;
    return plan::kOk;
}

void plan_server_destroy(plan_server *srv) {
    if (!srv) return;
    srv->q->shutdown();  // the running requests finish; the workers' contexts are destroyed
    srv->q->drain([](plan::ServeRequest &r) {
        Job *j = static_cast<Job *>(r.payload);
        if (j && j->cat) plan_catalogue_free(j->cat);
        delete j;
    });
    srv->q.reset();
    delete srv;
}

int plan_submit(plan_server *srv, const plan_lis_view *snap, const plan_params *p, int first_file, uint64_t *request) {
    if (!srv || !snap || !p || !request) return plan::kErrArgument;
    uint64_t n = 0;
    for (uint32_t b = 0; b < snap->nblocks; ++b) n += snap->counts[b];
    auto *j = new Job();
    j->view = *snap;
    j->params = *p;
    j->first_file = first_file;
    const uint64_t id = srv->q->submit(plan_footprint_bytes(n, p), j);
    if (id == 0) {
        delete j;
        const bool closing = srv->q->stopping();
        std::lock_guard<std::mutex> lk(srv->mu);
        if (closing) {
            srv->error = "the serving loop is shutting down and takes no more requests";
            return plan::kErrArgument;
        }
        srv->error = "the snapshot alone needs more device memory than the serving budget";
        return plan::kErrOutOfMemory;
    }
    *request = id;
    return plan::kOk;
}

int plan_poll(plan_server *srv, uint64_t request, int wait, plan_catalogue **out, double *latency_ms) {
    if (!srv || !out) return plan::kErrArgument;
    *out = nullptr;
    plan::ServeRequest r;
    const int got = srv->q->take(request, wait != 0, r);
    if (got < 0) return plan::kErrArgument;
    if (got == 0) return PLAN_PENDING;
    Job *j = static_cast<Job *>(r.payload);
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count();
    const int rc = r.status;
    if (rc == plan::kOk) {
        *out = j->cat;
    } else {
        if (j->cat) plan_catalogue_free(j->cat);
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->error = j->error.empty() ? "request failed with status " + std::to_string(rc) + " (no worker context)" : j->error;
    }
    delete j;
    return rc;
}

const char *plan_server_error(const plan_server *srv) {
    // a copy per calling thread: another thread may replace the server's message meanwhile
    static thread_local std::string copy;
    if (!srv) return "no server";
    std::lock_guard<std::mutex> lk(srv->mu);
    copy = srv->error;
    return copy.c_str();
}

int plan_server_stats(const plan_server *srv, uint64_t *peak_held_bytes, uint64_t *releases) {
    if (!srv) return plan::kErrArgument;
    if (peak_held_bytes) *peak_held_bytes = srv->q->peak_held_bytes();
    if (releases) *releases = srv->q->releases();
    return plan::kOk;
}

int plan_server_overlap(const plan_server *srv, double *busy_ms, double *overlap_ms) {
    if (!srv) return plan::kErrArgument;
    double b = 0, o = 0;
    srv->q->overlap(b, o);
    if (busy_ms) *busy_ms = b;
    if (overlap_ms) *overlap_ms = o;
    return plan::kOk;
}

}  // extern "C"

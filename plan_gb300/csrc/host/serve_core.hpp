// Admission and dispatch for the serving loop: pure host C++ (threads, no CUDA), so the
// policy is tested on the CPU with a stand-in executor.
//
// Requests arrive from any thread. Each carries its device footprint (bytes its snapshot
// needs). A request starts when a worker is free and the footprints of the running requests
// plus its own fit the budget. Requests start in arrival order; when the oldest waiting one
// does not fit, a later one that fits may go first, but the oldest is passed over at most
// `max_bypass` times, after which nothing starts ahead of it (no starvation). Workers keep
// the buffers of their largest request: a worker's hold counts against the budget until the
// executor releases it, which the scheduler asks of idle workers when a waiting request needs
// the room (the release runs before that request starts, so the budget holds on the device).
#pragma once

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

namespace plan {

struct ServeRequest {
    uint64_t id = 0;
    uint64_t footprint = 0;
    void *payload = nullptr;  // owned by the caller of submit()
    int status = -1;          // -1 queued, -2 running, else the executor's status
    void *result = nullptr;   // executor's output (e.g. a catalogue)
    std::chrono::steady_clock::time_point t_submit, t_start, t_done;
    int worker = -1;
    uint32_t bypassed = 0;    // times a later request started first
    uint64_t start_seq = 0;   // 1, 2, ... in the order requests were started
};

class ServeQueue {
   public:
    // init(worker) runs once on the worker's thread before anything else (status 0 = ok) and
    // fini(worker) last; run(worker, request) does one request there (status 0 = ok).
    // release(worker) frees what an idle worker keeps between requests; the scheduler calls it
    // from whichever thread is scheduling, never while that worker runs a request.
    using RunFn = std::function<int(int, ServeRequest &)>;
    using WorkerFn = std::function<int(int)>;

    ServeQueue(int workers, uint64_t budget, uint32_t max_bypass, WorkerFn init, RunFn run, WorkerFn release, WorkerFn fini)
        : budget_(budget), max_bypass_(max_bypass), run_(std::move(run)), release_(std::move(release)), init_(std::move(init)),
          fini_(std::move(fini)) {
        if (workers < 1) workers = 1;
        held_.assign(workers, 0);
        busy_.assign(workers, 0);
        release_pending_.assign(workers, 0);
        assigned_.assign(workers, nullptr);
        for (int w = 0; w < workers; ++w) threads_.emplace_back([this, w] { worker_loop(w); });
    }

    ~ServeQueue() { shutdown(); }

    // Let the running requests finish, start nothing more and join the workers.
    void shutdown() {
        {
            std::unique_lock<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_work_.notify_all();
        for (auto &t : threads_)
            if (t.joinable()) t.join();
    }

    // After shutdown(): hand every request not yet taken (queued, or done but never taken) to f.
    template <class F>
    void drain(F f) {
        std::unique_lock<std::mutex> lk(mu_);
        for (auto &it : all_) f(*it.second);
        all_.clear();
        queue_.clear();
    }

    // Queue a request; returns its id (1, 2, ...), or 0 if its footprint alone exceeds the budget.
    uint64_t submit(uint64_t footprint, void *payload) {
        std::unique_lock<std::mutex> lk(mu_);
        if (footprint > budget_ || stop_) return 0;
        auto r = std::make_shared<ServeRequest>();
        r->id = ++next_id_;
        r->footprint = footprint;
        r->payload = payload;
        r->t_submit = std::chrono::steady_clock::now();
        all_[r->id] = r;
        queue_.push_back(r);
        schedule_locked();
        return r->id;
    }

    // 1 when done (status and result filled in), 0 when still queued or running, -1 unknown id.
    // wait != 0 blocks until done. A finished request is forgotten once taken.
    int take(uint64_t id, bool wait, ServeRequest &out) {
        std::unique_lock<std::mutex> lk(mu_);
        auto it = all_.find(id);
        if (it == all_.end()) return -1;
        std::shared_ptr<ServeRequest> r = it->second;
        if (wait) cv_done_.wait(lk, [&] { return r->status >= 0 || r->status < -2; });
        if (r->status == -1 || r->status == -2) return 0;
        out = *r;
        all_.erase(it);
        return 1;
    }

    uint64_t in_flight_bytes() const {
        std::unique_lock<std::mutex> lk(mu_);
        uint64_t s = 0;
        for (uint64_t h : held_) s += h;
        return s;
    }
    uint64_t peak_held_bytes() const {
        std::unique_lock<std::mutex> lk(mu_);
        return peak_held_;
    }
    uint64_t releases() const {
        std::unique_lock<std::mutex> lk(mu_);
        return releases_;
    }
    // Over the requests run so far, from each one's start on its worker to its end: the time
    // at least one ran (busy_ms) and the time two or more ran at once (overlap_ms).
    void overlap(double &busy_ms, double &overlap_ms) const {
        std::vector<std::pair<std::chrono::steady_clock::time_point, int>> ev;
        {
            std::unique_lock<std::mutex> lk(mu_);
            for (const auto &sp : spans_) {
                ev.emplace_back(sp.first, +1);
                ev.emplace_back(sp.second, -1);
            }
        }
        std::sort(ev.begin(), ev.end(), [](const auto &a, const auto &b) { return a.first < b.first || (a.first == b.first && a.second < b.second); });
        busy_ms = overlap_ms = 0;
        int running = 0;
        for (size_t k = 0; k + 1 < ev.size(); ++k) {
            running += ev[k].second;
            const double dt = std::chrono::duration<double, std::milli>(ev[k + 1].first - ev[k].first).count();
            if (running >= 1) busy_ms += dt;
            if (running >= 2) overlap_ms += dt;
        }
    }
    int workers() const { return (int)held_.size(); }
    // once true, stays true: submit refuses everything from then on
    bool stopping() const {
        std::unique_lock<std::mutex> lk(mu_);
        return stop_;
    }

   private:
    // Start what can start; called with the lock held. Nothing starts once shutting down (a
    // worker that has left its loop would never run it).
    void schedule_locked() {
        if (stop_) return;
        bool started = true;
        while (started && !queue_.empty()) {
            started = false;
            uint64_t held = 0;
            for (uint64_t h : held_) held += h;
            for (size_t qi = 0; qi < queue_.size(); ++qi) {
                const std::shared_ptr<ServeRequest> r = queue_[qi];
                if (qi > 0 && queue_.front()->bypassed >= max_bypass_) break;  // the oldest waits no longer
                // a free worker: prefer one that already holds enough, else the one holding most
                int best = -1;
                for (int w = 0; w < (int)held_.size(); ++w) {
                    if (busy_[w]) continue;
                    if (best < 0) { best = w; continue; }
                    const bool fits_w = held_[w] >= r->footprint, fits_b = held_[best] >= r->footprint;
                    if (fits_w != fits_b ? fits_w : (fits_w ? held_[w] < held_[best] : held_[w] > held_[best])) best = w;
                }
                if (best < 0) return;  // no free worker
                const uint64_t grow = r->footprint > held_[best] ? r->footprint - held_[best] : 0;
                if (held + grow > budget_) {
                    // idle workers other than `best` give back their buffers, if that makes room
                    uint64_t idle_other = 0;
                    for (int w = 0; w < (int)held_.size(); ++w)
                        if (!busy_[w] && w != best) idle_other += held_[w];
                    if (held - idle_other + grow <= budget_ && idle_other > 0) {
                        // the idle workers give their buffers back on their own threads, outside
                        // the lock; the request started below waits until they have
                        for (int w = 0; w < (int)held_.size(); ++w)
                            if (!busy_[w] && w != best && held_[w]) {
                                if (release_) release_pending_[w] = 1;
                                held_[w] = 0;
                                ++releases_;
                            }
                        held -= idle_other;
                    } else {
                        continue;  // does not fit now; a later request may
                    }
                }
                // start r on `best`
                for (size_t pj = 0; pj < qi; ++pj) queue_[pj]->bypassed++;
                held += grow;
                held_[best] += grow;
                busy_[best] = 1;
                r->status = -2;
                r->worker = best;
                r->start_seq = ++started_;
                assigned_[best] = r;
                queue_.erase(queue_.begin() + (long)qi);
                uint64_t now = 0;
                for (uint64_t h : held_) now += h;
                if (now > peak_held_) peak_held_ = now;
                cv_work_.notify_all();
                started = true;
                break;
            }
        }
    }

    bool releases_pending_locked() const {
        for (uint8_t f : release_pending_)
            if (f) return true;
        return false;
    }

    void worker_loop(int w) {
        const int init_rc = init_ ? init_(w) : 0;
        std::unique_lock<std::mutex> lk(mu_);
        while (true) {
            cv_work_.wait(lk, [&] { return stop_ || assigned_[w] != nullptr || release_pending_[w]; });
            if (release_pending_[w]) {  // give the buffers back without holding the lock
                lk.unlock();
                release_(w);
                lk.lock();
                release_pending_[w] = 0;
                cv_done_.notify_all();
                continue;
            }
            if (assigned_[w] == nullptr) break;  // stopping, nothing assigned
            std::shared_ptr<ServeRequest> r = assigned_[w];
            // the room this request was admitted into must be free before it allocates
            cv_done_.wait(lk, [&] { return !releases_pending_locked(); });
            lk.unlock();
            r->t_start = std::chrono::steady_clock::now();
            const int rc = init_rc ? init_rc : run_(w, *r);
            r->t_done = std::chrono::steady_clock::now();
            lk.lock();
            spans_.emplace_back(r->t_start, r->t_done);
            r->status = rc < 0 ? 1000 : rc;
            assigned_[w] = nullptr;
            busy_[w] = 0;
            cv_done_.notify_all();
            schedule_locked();
        }
        lk.unlock();
        if (fini_) fini_(w);
    }

    mutable std::mutex mu_;
    std::condition_variable cv_work_, cv_done_;
    std::deque<std::shared_ptr<ServeRequest>> queue_;
    std::map<uint64_t, std::shared_ptr<ServeRequest>> all_;
    std::vector<uint64_t> held_;
    std::vector<uint8_t> busy_, release_pending_;
    std::vector<std::shared_ptr<ServeRequest>> assigned_;
    std::vector<std::pair<std::chrono::steady_clock::time_point, std::chrono::steady_clock::time_point>> spans_;
    std::vector<std::thread> threads_;
    uint64_t budget_, next_id_ = 0, peak_held_ = 0, releases_ = 0, started_ = 0;
    uint32_t max_bypass_;
    bool stop_ = false;
    RunFn run_;
    WorkerFn release_, init_, fini_;
};

}  // namespace plan

"""Admission and dispatch of the serving loop, on the CPU with a stand-in executor (no GPU).

plan_gb300/csrc/host/serve_core.hpp decides which submitted snapshot starts on which worker:
arrival order, a device-memory budget over what the workers hold, later requests passing a
blocked one a bounded number of times, idle workers giving their buffers back when a waiting
request needs the room. The harness below drives it with sleeping executors from several
submitting threads and checks every rule while it runs.
"""
from __future__ import annotations

import shutil
import subprocess

import pytest

from conftest import ROOT

HARNESS = r"""
#include <atomic>
#include <cstdio>
#include <random>
#include <thread>
#include <vector>
#include "host/serve_core.hpp"

using namespace plan;

struct Check {
    std::mutex mu;
    std::vector<uint64_t> held;      // what each worker holds, as the executor sees it
    uint64_t budget = 0, worst = 0;  // largest total hold seen at a request's start
    long bad = 0;
};

static int run_case(int workers, uint64_t budget, uint32_t max_bypass, int nreq, int threads, bool fifo_sizes, unsigned seed) {
    Check ck;
    ck.held.assign(workers, 0);
    ck.budget = budget;
    std::atomic<int> inits{0}, finis{0};
    long order_bad = 0;
    ServeQueue q(
        workers, budget, max_bypass, [&](int) { ++inits; return 0; },
        [&](int w, ServeRequest &r) {
            {
                std::lock_guard<std::mutex> lk(ck.mu);
                if (ck.held[w] < r.footprint) ck.held[w] = r.footprint;
                uint64_t s = 0;
                for (uint64_t h : ck.held) s += h;
                if (s > ck.worst) ck.worst = s;
                if (s > ck.budget) ++ck.bad;
            }
            std::this_thread::sleep_for(std::chrono::microseconds(200 + (r.id * 7919) % 1500));
            r.result = reinterpret_cast<void *>(r.id * 3);
            return 0;
        },
        [&](int w) {
            std::lock_guard<std::mutex> lk(ck.mu);
            ck.held[w] = 0;
            return 0;
        },
        [&](int) { ++finis; return 0; });
    std::vector<std::vector<uint64_t>> ids(threads);
    std::vector<std::thread> sub;
    std::atomic<int> rejected{0};
    for (int t = 0; t < threads; ++t)
        sub.emplace_back([&, t] {
            std::mt19937_64 rng(seed + t);
            for (int i = 0; i < nreq / threads; ++i) {
                uint64_t fp = fifo_sizes ? 10 : 1 + rng() % (budget * 3 / 4);
                if (i == 3 && t == 0) {  // one that can never fit
                    if (q.submit(budget + 1, nullptr) == 0) ++rejected;
                }
                uint64_t id = q.submit(fp, nullptr);
                if (id) ids[t].push_back(id);
                if (rng() % 4 == 0) std::this_thread::sleep_for(std::chrono::microseconds(rng() % 500));
            }
        });
    for (auto &th : sub) th.join();
    long done = 0, wrong = 0, bypass_bad = 0;
    for (auto &v : ids)
        for (uint64_t id : v) {
            ServeRequest r;
            if (q.take(id, true, r) != 1) { ++wrong; continue; }
            if (r.status != 0 || r.result != reinterpret_cast<void *>(id * 3)) ++wrong;
            if (r.bypassed > max_bypass) ++bypass_bad;
            if (max_bypass == 0 && r.start_seq != id) ++order_bad;  // strict arrival order
            if (!(r.t_submit <= r.t_start && r.t_start <= r.t_done)) ++wrong;
            ++done;
        }
    ServeRequest r;
    if (q.take(999999, false, r) != -1) ++wrong;
    double busy = 0, both = 0;
    q.overlap(busy, both);
    q.shutdown();
    std::printf("%d %llu %llu %ld %ld %ld %ld %d %d %d %llu %lld %lld\n", workers, (unsigned long long)budget, (unsigned long long)ck.worst, ck.bad,
                done, wrong, bypass_bad + order_bad, rejected.load(), inits.load(), finis.load(), (unsigned long long)q.releases(),
                (long long)(busy * 1000), (long long)(both * 1000));
    return 0;
}

int main() {
    run_case(3, 100, 6, 240, 4, false, 1);
    run_case(4, 1000, 8, 400, 3, false, 2);
    run_case(2, 100, 0, 120, 3, false, 3);   // strict arrival order
    run_case(8, 100, 16, 200, 4, true, 4);   // every request fits: full overlap
    run_case(1, 50, 2, 60, 2, false, 5);
    return 0;
}
"""


def test_serving_admission(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    (tmp_path / "h.cpp").write_text(HARNESS)
    exe = tmp_path / "h"
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-I", str(ROOT / "plan_gb300" / "csrc"), str(tmp_path / "h.cpp"), "-o",
                    str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True, timeout=120).stdout.split("\n")
    rows = [list(map(int, ln.split())) for ln in out if ln.strip()]
    assert len(rows) == 5
    for workers, budget, worst, over, done, wrong, order, rejected, inits, finis, releases, busy_us, both_us in rows:
        assert busy_us > 0 and 0 <= both_us <= busy_us  # run spans: some time busy, overlap within it
        if workers == 1:
            assert both_us == 0                       # one worker never runs two at once
        assert over == 0 and worst <= budget          # the holds never exceed the budget
        assert wrong == 0 and done > 0                # every request ran once, with its own result
        assert order == 0                             # bypass bound and strict order kept
        assert rejected == 1                          # a snapshot larger than the budget is refused
        assert inits == workers and finis == workers  # one context per worker, torn down at the end
    assert any(r[10] > 0 for r in rows)               # idle workers gave buffers back when needed
    assert rows[3][12] > 0                            # eight workers, everything fits: requests overlap

// Command-line front end of the oracle restatement: the reference's find-clumps command
// line (src/global.cpp:247-289) over the CPU restatement. Test infrastructure only.
#include "oracle.hpp"

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <getopt.h>
#include <iomanip>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace orc;

static double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int main(int argc, char **argv) {
    static int f_combined = 0, f_find = 0, f_save = 0, f_noghost = 0, f_basic = 0, f_dvs = 0, f_tmp = 0, f_help = 0, f_dbg = 0, f_verb = 0;
    static struct option opts[] = {
        {"Debug", no_argument, &f_dbg, 1},         {"Verbose", no_argument, &f_verb, 1},
        {"Combined", no_argument, &f_combined, 1}, {"Find_Clumps", no_argument, &f_find, 1},
        {"Save_Clumps", no_argument, &f_save, 1},  {"No_Ghost", no_argument, &f_noghost, 1},
        {"Basic_Analyses", no_argument, &f_basic, 1}, {"Density_Vs_Scale", no_argument, &f_dvs, 1},
        {"Temp_Calculation", no_argument, &f_tmp, 1}, {"Help", no_argument, &f_help, 1},
        {"num_cpus", required_argument, nullptr, 'c'}, {"data_dir", required_argument, nullptr, 'i'},
        {"basename", required_argument, nullptr, 'b'}, {"postname", required_argument, nullptr, 'p'},
        {"file_num", required_argument, nullptr, 'f'}, {"out_file", required_argument, nullptr, 'o'},
        {"in_const", required_argument, nullptr, 't'}, {"sampling", required_argument, nullptr, 's'},
        {"xlim", required_argument, nullptr, 'x'}, {"ylim", required_argument, nullptr, 'y'},
        {"zlim", required_argument, nullptr, 'z'}, {"pow_mode", required_argument, nullptr, 'P'},
        {"threads", required_argument, nullptr, 'T'}, {nullptr, 0, nullptr, 0}};
    int num_cpus = 1, start = 0, end = 0, step = 1, pow_mode = 0, threads = 0;
    unsigned sampling = 1;
    std::string dir, base, post, out, param;
    bool user_box = false;
    double box_lo[3] = {0, 0, 0}, box_hi[3] = {0, 0, 0};
    int o, idx;
    while ((o = getopt_long(argc, argv, ":c:i:b:p:f:o:t:s:x:y:z:hP:T:", opts, &idx)) != -1) {
        switch (o) {
        case 0: break;
        case 'c': num_cpus = std::atoi(optarg); break;
        case 'i': dir = optarg; break;
        case 'b': base = optarg; break;
        case 'p': post = optarg; break;
        case 'f': {
            std::string s(optarg);
            char ch;
            if (s.find_first_of(':') == s.find_last_of(':')) {
                std::istringstream is(s);
                is >> start >> ch >> end;
            } else {
                std::istringstream is(s.substr(0, s.find_last_of(':')));
                is >> start >> ch >> end;
                step = std::atoi(s.substr(s.find_last_of(':') + 1).c_str());
            }
            if (start < 0) start = 0;
            if (end < start) end = start;
            if (step == 0) step = 1;
            break;
        }
        case 'o': out = optarg; break;
        case 't': param = optarg; break;
        case 's': sampling = (unsigned)std::atoi(optarg); if (sampling == 0) sampling = 1; break;
        case 'P': pow_mode = std::atoi(optarg); break;
        case 'T': threads = std::atoi(optarg); break;
        case 'h': f_help = 1; break;
        case 'x': case 'y': case 'z': {  // src/global.cpp:398-440
            const int d = o == 'x' ? 0 : o == 'y' ? 1 : 2;
            std::istringstream is(optarg);
            char sep;
            is >> box_lo[d] >> sep >> box_hi[d];
            if (box_lo[d] > box_hi[d]) std::swap(box_lo[d], box_hi[d]);
            user_box = true;
            break;
        }
        default: std::fprintf(stderr, "Error: Unknown/invalid option\n"); return 2;
        }
    }
    if (f_help || out.empty()) { std::fprintf(stderr, "usage: oracle_plan -c N -i dir -b base -p post -f a:b[:s] -o out -t params [--Combined]\n"); return 0; }
    if (!dir.empty() && dir.back() != '/') dir.push_back('/');
    Params par;
    if (!param.empty()) { int rc = read_param_file(param, par); if (rc) return rc; }
    par.user_box = user_box;
    for (int d = 0; d < 3; ++d) {
        par.user_box_min[d] = box_lo[d];
        par.user_box_max[d] = box_hi[d];
    }
    int nthreads = threads > 0 ? threads : (int)par.num_threads;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#endif
    if (nthreads <= 0) nthreads = 1;
    bool first = true;
    if (!f_find && !f_basic && !f_dvs && !f_tmp) f_find = 1;  // src/global.cpp:498-501
    const std::string ostem = out.substr(0, out.find_last_of('.'));
    // result files in BasicAnalysesPreWork's order (src/analyses.cpp:16-33); with only
    // --Density_Vs_Scale the basic results go to the first open file, the RMPL one
    FILE *rf = nullptr, *pf = nullptr;
    if (f_dvs && !(rf = std::fopen((ostem + "_RMPL.txt").c_str(), "w"))) return 3;
    if (f_find && !(pf = std::fopen((ostem + "_planetesimals.txt").c_str(), "w"))) return 3;
    FILE *basic_file = pf ? pf : rf;
    for (int num = start; num <= end; num += step) {
        std::ostringstream nn;
        nn << std::setw(4) << std::setfill('0') << num;
        std::vector<std::string> files;
        if (f_combined) {
            files.push_back(dir + base + "." + nn.str() + "." + post + ".lis");
        } else {
            files.push_back(dir + "id0/" + base + "." + nn.str() + "." + post + ".lis");
            for (int id = 1; id < num_cpus; ++id)
                files.push_back(dir + "id" + std::to_string(id) + "/" + base + "-id" + std::to_string(id) + "." + nn.str() + "." + post + ".lis");
        }
        double t0 = now();
        Snapshot snap;
        int rc = read_lis_files(files, snap);
        if (rc) return rc;
        finish_read(snap, par, first);
        if (snap.num_particles == 0) {  // the reference has no check and crashes in BuildTree
            std::fprintf(stderr, "Error: the snapshot holds no particles\n");
            return 5;
        }
        if (f_dvs) {  // BasicAnalyses' settings for --Density_Vs_Scale (src/analyses.hpp:29-33)
            par.max_ghost_zone_width = par.max_half_width;
            f_noghost = 1;
        }
        uint32_t nin = snap.num_particles;
        double t1 = now();
        if (!f_noghost) make_ghosts(snap, par);
        Finder f;
        f.par = &par;
        f.threads = nthreads;
        f.pow_mode = pow_mode ? POW_CORRECT : POW_LIBM;
        f.time = snap.time;
        // the shared summary stream is left scientific by an earlier snapshot's basic results
        // or by this snapshot's density-vs-scale lines
        f.window_stats_on = std::getenv("PLAN_ORACLE_WINDOW_STATS") != nullptr;
        f.stream_scientific = !first || f_dvs;
        if (f_dvs) f.tree.max_leaf_size = 64;
        f.tree.build(par, snap.parts, true);
        if (f_dvs) {
            DensityVsScale dv = density_vs_scale(f.tree, par, snap.time);
            const std::string txt = (first ? dv.header : std::string()) + dv.line;
            std::fwrite(txt.data(), 1, txt.size(), rf);
        }
        double t2 = now();
        std::string summary;
        try {
            summary = f.find(nin);
        } catch (const std::domain_error &e) {
            std::fprintf(stderr, "Error: %s\n", e.what());
            return 5;
        }
        double t3 = now();
        std::printf("%s\n", summary.c_str());
        if (f.window_stats_on) {
            const WindowStats &w = f.window_stats;
            static const char *names[kWindowSchemes] = {"first bound, 32 wide", "first bound, 256 wide", "first bound, 1024 wide",
                                                         "speculative windows", "256-wide scan + speculative windows"};
            std::fprintf(stderr, "[oracle] Hill rebinding: %llu calls, %llu candidates, %llu accepted; %llu windows cut short, %llu calls disagreeing\n",
                         (unsigned long long)w.calls, (unsigned long long)w.candidates, (unsigned long long)w.accepted,
                         (unsigned long long)w.mismatch_windows, (unsigned long long)w.disagreements);
            for (int k = 0; k < kWindowSchemes; ++k) {
                uint64_t most = 0, most_acc = 0;
                for (const auto &kv : w.per_clump)
                    if (kv.second.steps[k] > most) {
                        most = kv.second.steps[k];
                        most_acc = kv.second.accepted;
                    }
                std::fprintf(stderr, "[oracle]   %-36s steps %llu, longest call %llu, most for one clump %llu (it accepts %llu)\n", names[k],
                             (unsigned long long)w.steps[k], (unsigned long long)w.longest_call[k], (unsigned long long)most,
                             (unsigned long long)most_acc);
            }
            // a cost model of the longest chain, one clump's calls in a row: a step that
            // accepts costs A cycles in the default loop (3,200 measured); a step or window
            // that accepts nothing costs E; a speculative window that accepts costs W plus C
            // per acceptance for its chain of updates (E, W, C are estimates: the FP32 test
            // and ballot, the test, reciprocals and verification, two dependent FMAs and
            // their operands)
            const double A = 3200, E = 400, W = 1500, Cc = 256;
            double worst_default = 0, worst_spec = 0;
            for (const auto &kv : w.per_clump) {
                const auto &pc = kv.second;
                worst_default = std::max(worst_default, A * pc.accepted + E * (pc.steps[0] - pc.accepted));
                worst_spec = std::max(worst_spec, W * pc.busy_windows + Cc * pc.accepted + E * (pc.steps[3] - pc.busy_windows));
            }
            std::fprintf(stderr, "[oracle] cost model, longest clump chain: default loop %.3g cycles, speculative windows %.3g cycles\n",
                         worst_default, worst_spec);
            // the round model: every clump makes its k-th call in round k, and a round lasts as
            // long as its slowest call
            double round_default = 0, round_spec = 0;
            for (size_t k = 0;; ++k) {
                double md = -1, ms = -1;
                for (const auto &kv : w.per_clump) {
                    if (k >= kv.second.call.size()) continue;
                    const auto &q = kv.second.call[k];
                    md = std::max(md, A * q[0] + E * (q[1] - q[0]));
                    ms = std::max(ms, W * q[3] + Cc * q[0] + E * (q[2] - q[3]));
                }
                if (md < 0) break;
                round_default += md;
                round_spec += ms;
            }
            std::fprintf(stderr, "[oracle] cost model, rounds (one call per clump per round): default loop %.3g cycles, speculative windows %.3g cycles\n",
                         round_default, round_spec);
            uint64_t most_calls = 0, most_grown = 0, grown_of_most_calls = 0;
            for (const auto &kv : w.per_clump) {
                if (kv.second.calls > most_calls) {
                    most_calls = kv.second.calls;
                    grown_of_most_calls = kv.second.grown_members;
                }
                most_grown = std::max(most_grown, kv.second.grown_members);
            }
            std::fprintf(stderr,
                         "[oracle] calls of one clump, at most %llu (members re-sorted over them: %llu); most members re-sorted for one clump %llu\n",
                         (unsigned long long)most_calls, (unsigned long long)grown_of_most_calls, (unsigned long long)most_grown);
            std::fprintf(stderr, "[oracle] accepted per speculative window:");
            for (uint64_t v : w.accepted_per_window) std::fprintf(stderr, " %llu", (unsigned long long)v);
            std::fprintf(stderr, "\n");
        }
        write_peaks_file(peaks_file_name(out, snap.time), f);
        if (f_save) {
            std::ostringstream sid;
            sid << std::setw(4) << std::setfill('0') << num;
            write_parlists("ParList." + sid.str(), f, sampling);
        }
        std::string line = (first ? basic_results_header() : std::string()) + basic_results_line(f, par, snap.time);
        std::fwrite(line.data(), 1, line.size(), basic_file);
        std::fprintf(stderr, "[oracle] read %.4f s, ghost+tree %.4f s, find %.4f s, tree points %u, threads %d\n", t1 - t0, t2 - t1, t3 - t2, f.tree.size(), nthreads);
        first = false;
    }
    if (pf) std::fclose(pf);
    if (rf) std::fclose(rf);
    return 0;
}

// plan_gpu: drop-in for the reference program's find-clumps mode.
//
// Same command line (src/global.cpp:247-289, usage 558-578), same file names
// (src/global.cpp:620-675) and the same outputs: <out-stem>_planetesimals.txt
// (WriteBasicResults), peaks_at_<time>.txt and, with --Save_Clumps, ParList.<NNNN>/.
// -x/-y/-z user boxes restrict the particles read, as in the reference. --Density_Vs_Scale
// writes <out>_RMPL.txt and finds clumps on that run's tree, as the reference does. The grid
// analyses (--Basic_Analyses, --Temp_Calculation) are not part of this program and are rejected
// with exit code 2.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <getopt.h>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "plan_gpu.h"

namespace {

void usage(const char *prog) {
    std::cout << "USAGE: \n" << prog
              << " -c <num_cpus> -i <data_dir> -b <basename> -p <postname>  -f <range(f1:f2)|range_step(f1:f2:step)> -o <output> [-t "
                 "<input_file_for_constants> -s 10 -x -0.1,0.1 -y -0.05,0.05 --flags]\n"
              << "Example: ./plan -c 64 -i ./bin/ -b Par_Strat3d -p ds -f 170:227 -o result.txt -t plan_input.txt --Verbose --Find_Clumps\n"
              << "[...] means optional arguments. Available flags: \n"
              << "Use --Help to obtain this usage information\n"
              << "Use --Verbose to obtain more output during execution\n"
              << "Use --Debug to obtain all possible output during execution\n"
              << "Use --Combined to deal with combined lis files (from all processors)\n"
              << "Use --Find_Clumps to run clump finding functions\n"
              << "Use --Save_Clumps to save all clumps to particle lists\n\t(use '-s N' to sub-sample (1 in N) the particle list for "
                 "outputting to save storage)\n"
              << "Use --No_Ghost to skip making ghost particles\n"
              << "Use --Basic_Analyses to perform basic analyses, which will output max($\\rho_p$) and $H_p$\n"
              << "Use --Density_Vs_Scale to calculate max($\\rho_p$) as a function of length scales\n"
              << "Use --Temp_Calculation to do temporary calculations in TempCalculation()\n"
              << "If you don't specify any flags, then --Find_Clumps will be turned on automatically." << std::endl;
}

int exit_code(int status) {
    switch (status) {
    case 0: return 0;
    case 2: return 2;
    case 3: return 3;
    case 4: return 4;
    default: return 5;
    }
}

}  // namespace

int main(int argc, char **argv) {
    static int f_debug = 0, f_verbose = 0, f_combined = 0, f_find = 0, f_save = 0, f_noghost = 0, f_basic = 0, f_dvs = 0, f_tmp = 0,
               f_help = 0;
    static struct option opts[] = {{"Debug", no_argument, &f_debug, 1},
                                   {"Verbose", no_argument, &f_verbose, 1},
                                   {"Combined", no_argument, &f_combined, 1},
                                   {"Find_Clumps", no_argument, &f_find, 1},
                                   {"Save_Clumps", no_argument, &f_save, 1},
                                   {"No_Ghost", no_argument, &f_noghost, 1},
                                   {"Basic_Analyses", no_argument, &f_basic, 1},
                                   {"Density_Vs_Scale", no_argument, &f_dvs, 1},
                                   {"Temp_Calculation", no_argument, &f_tmp, 1},
                                   {"Help", no_argument, &f_help, 1},
                                   {"num_cpus", required_argument, nullptr, 'c'},
                                   {"data_dir", required_argument, nullptr, 'i'},
                                   {"basename", required_argument, nullptr, 'b'},
                                   {"postname", required_argument, nullptr, 'p'},
                                   {"file_num", required_argument, nullptr, 'f'},
                                   {"out_file", required_argument, nullptr, 'o'},
                                   {"in_const", required_argument, nullptr, 't'},
                                   {"sampling", required_argument, nullptr, 's'},
                                   {"xlim", required_argument, nullptr, 'x'},
                                   {"ylim", required_argument, nullptr, 'y'},
                                   {"zlim", required_argument, nullptr, 'z'},
                                   {nullptr, 0, nullptr, 0}};
    int num_cpus = 0, start_num = 0, end_num = 0, interval = 1, num_files = 0;
    unsigned sampling = 1;
    std::string dir, base, post, out, param;
    bool user_box = false;
    double box_lo[3] = {0, 0, 0}, box_hi[3] = {0, 0, 0};  // user box, 0,0 = not restricted on that axis
    if (argc < 13) {
        usage(argv[0]);
        return 0;
    }
    int o, idx;
    while ((o = getopt_long(argc, argv, ":c:i:b:p:f:o:t:s:x:y:z:h", opts, &idx)) != -1) {
        switch (o) {
        case 0: break;
        case 'c': { std::istringstream is(optarg); is >> num_cpus; break; }
        case 'i': dir = optarg; break;
        case 'b': base = optarg; break;
        case 'p': post = optarg; break;
        case 'f': {
            std::string s(optarg);
            size_t p1 = s.find_first_of(':'), p2 = s.find_last_of(':');
            char ch;
            if (p1 == p2) {
                std::istringstream is(optarg);
                is >> start_num >> ch >> end_num;
                interval = 1;
            } else {
                std::istringstream is(s.substr(0, p2));
                is >> start_num >> ch >> end_num;
                std::istringstream iv(s.substr(p2 + 1));
                iv >> interval;
            }
            if (start_num < 0) { std::cerr << "The start number should be positive (Auto fix to 0)" << std::endl; start_num = 0; }
            if (end_num < start_num) {
                std::cerr << "The end number should be larger or equal than the start number. (Auto fix to start number)." << std::endl;
                end_num = start_num;
            }
            if (interval == 0) { std::cerr << "The interval should be non-zero. (Auto fix to 1)" << std::endl; interval = 1; }
            num_files = (end_num - start_num) / interval + 1;
            break;
        }
        case 'o': out = optarg; break;
        case 't': param = optarg; break;
        case 's': {
            std::string s(optarg);
            if (s.find('-') != std::string::npos) {
                std::cerr << "sub_sampling_rate should be positive. (Auto fix to 1)" << std::endl;
            } else {
                std::istringstream is(optarg);
                is >> sampling;
                if (sampling == 0) sampling = 1;
            }
            break;
        }
        case 'x': case 'y': case 'z': {  // src/global.cpp:398-440
            const int d = o == 'x' ? 0 : o == 'y' ? 1 : 2;
            std::istringstream is(optarg);
            char sep;
            is >> box_lo[d] >> sep >> box_hi[d];
            if (box_lo[d] > box_hi[d]) std::swap(box_lo[d], box_hi[d]);
            user_box = true;
            break;
        }
        case 'h': f_help = 1; break;
        case ':':
            std::cerr << "Error: Option -" << optopt << " requires an arugment.\n";
            return 2;
        default:
            if (!isprint(optopt)) std::cerr << "Error: Unknown/invalid flag, check usage with --Help or -h.\n";
            else std::cerr << "Error: Unknown/invalid option -" << static_cast<char>(optopt) << "\n";
            return 2;
        }
    }
    if (f_help) {
        usage(argv[0]);
        return 0;
    }
    if (!f_find && !f_basic && !f_dvs && !f_tmp) f_find = 1;
    if (optind < argc) {
        std::cerr << "Non-option ARGV-elements: ";
        while (optind < argc) std::cerr << argv[optind++];
        std::cerr << "\nSomething is wrong with the argument list. Check usage by --Help or -h.\n";
        return 2;
    }
    if (f_basic || f_tmp) {
        std::cerr << "Error: only --Find_Clumps and --Density_Vs_Scale are available in this program (the grid analyses are not part of it)."
                  << std::endl;
        return 2;
    }
    if (dir.empty() || *dir.rbegin() != '/') dir.push_back('/');
    plan_params par;
    plan_params_init(&par);
    par.no_ghost = f_noghost;
    par.density_vs_scale = f_dvs ? 1 : 0;
    par.user_box = user_box ? 1 : 0;
    for (int d = 0; d < 3; ++d) {
        par.user_box_min[d] = box_lo[d];
        par.user_box_max[d] = box_hi[d];
    }
    if (!param.empty()) {
        int rc = plan_params_read(param.c_str(), &par);
        if (rc) return exit_code(rc);
    }
    plan_ctx *ctx = nullptr;
    int rc = plan_ctx_create(0, &ctx);
    if (rc) {
        std::cerr << "Error: no usable CUDA device (this program has no CPU path)." << std::endl;
        return exit_code(rc);
    }
    // result files in BasicAnalysesPreWork's order (src/analyses.cpp:16-33): <out>_RMPL.txt for
    // --Density_Vs_Scale, <out>_planetesimals.txt for --Find_Clumps; WriteBasicResults writes to
    // the first open file when only the former is open
    const std::string ostem = out.substr(0, out.find_last_of('.'));
    FILE *rf = nullptr, *pf = nullptr;
    for (int k = 0; k < 2; ++k) {
        if (k == 0 ? !f_dvs : !f_find) continue;
        const std::string name = ostem + (k == 0 ? "_RMPL.txt" : "_planetesimals.txt");
        FILE *fh = std::fopen(name.c_str(), "w");
        if (!fh) {
            std::cerr << "Error: Failed to open file " << name << std::endl;
            if (rf) std::fclose(rf);
            plan_ctx_destroy(ctx);
            return 3;
        }
        (k == 0 ? rf : pf) = fh;
    }
    FILE *basic_file = pf ? pf : rf;
    const char *pd_env = std::getenv("PLAN_PARLIST_DEVICE");
    const bool parlist_device = pd_env && *pd_env == '1';
    std::ostringstream oc;  // keeps its formatting state across snapshots, as the reference's
    bool first = true;
    int status = 0;
    for (int num = start_num; num <= end_num && num_files > 0; num += interval) {  // mpi->loop_begin..loop_end
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
        std::vector<const char *> paths;
        for (auto &f : files) paths.push_back(f.c_str());
        plan_lis *lis = nullptr;
        rc = plan_lis_read(paths.data(), (int)paths.size(), &lis);
        if (rc) { status = rc; break; }
        plan_lis_view view;
        plan_lis_get_view(lis, &view);
        plan_catalogue *cat = nullptr;
        if (f_dvs) {
            // BuildTree, BasicAnalysesWithTree, FindPlanetesimals (src/main.cpp:71-79)
            rc = plan_build_tree(ctx, &view, &par, first ? 1 : 0, nullptr);
            double radii[32], rho[32];
            int nlev = 0;
            if (!rc) rc = plan_density_vs_scale(ctx, &par, view.time, radii, rho, 32, &nlev);
            if (!rc) {
                std::ostringstream rm;  // src/analyses.hpp:258-266, 323-329
                if (first) {
                    rm << std::setw(15) << std::setfill(' ') << "#time";
                    for (int i = 0; i < nlev && i < 32; ++i) rm << std::setw(15) << std::setfill(' ') << std::scientific << radii[i];
                    rm << "\n";
                }
                rm << std::setw(15) << std::setfill(' ') << std::scientific << view.time;
                for (int i = 0; i < nlev && i < 32; ++i) rm << std::setw(15) << std::setfill(' ') << std::scientific << rho[i];
                rm << "\n";
                const std::string t = rm.str();
                std::fwrite(t.data(), 1, t.size(), rf);
                oc << std::scientific;  // the shared stream is left scientific before the summary
                rc = plan_find_planetesimals(ctx, &par, nullptr, &cat);
            }
        } else {
            rc = plan_find_clumps(ctx, &view, &par, first ? 1 : 0, nullptr, &cat);
        }
        if (rc) {
            std::cerr << "Error: " << plan_last_error(ctx) << std::endl;
            plan_lis_free(lis);
            status = rc;
            break;
        }
        // summary line (src/tree.hpp:4269, 4320-4325, 4337-4338)
        plan_clump_info last;
        uint32_t n = plan_catalogue_count(cat);
        oc << "Finish clump finding for t = " << view.time << ", ";
        if (n > 0) {
            double tot = 0.;
            for (uint32_t i = 0; i < n; ++i) { plan_catalogue_get(cat, i, &last); tot = tot + last.total_mass; }
            oc << "found " << n << " clumps; " << " Mp_max = " << last.total_mass << ", Mp_tot = " << tot << "(" << std::fixed
               << tot / par.mass_total_code_units * 100 << "%) in code units.";
        } else {
            oc << "found zero clumps";
        }
        oc << std::endl;
        std::cout << oc.str() << std::flush;
        oc.str(std::string());
        oc.clear();
        oc << std::scientific;  // WriteBasicResults leaves the shared stream in scientific mode
        // member lists formatted on the device with PLAN_PARLIST_DEVICE=1, else on the host
        rc = plan_catalogue_write_peaks(cat, out.c_str(), f_save && !parlist_device, num, sampling);
        if (!rc && f_save && parlist_device) rc = plan_catalogue_write_parlists(ctx, cat, num, sampling);
        if (rc) status = rc;
        char buf[1024];
        int len = plan_catalogue_basic_results(cat, &par, first ? 1 : 0, buf, sizeof(buf));
        if (len > 0) std::fwrite(buf, 1, (size_t)len, basic_file);
        plan_catalogue_free(cat);
        plan_lis_free(lis);
        first = false;
    }
    if (pf) std::fclose(pf);
    if (rf) std::fclose(rf);
    plan_ctx_destroy(ctx);
    return exit_code(status);
}

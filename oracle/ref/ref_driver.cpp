// Find-clumps-only driver for the UNMODIFIED reference sources (test infrastructure).
//
// This file is oracle code: it links src/global.cpp, src/tree.cpp and src/tree.hpp of the
// reference exactly as they are and drives the same per-snapshot sequence as the
// reference's main program for `--Find_Clumps` and `--Density_Vs_Scale`
// (src/main.cpp:39-102). Of src/analyses.hpp it runs BasicAnalysesWithTree as it is; the
// part of BasicAnalyses that --Density_Vs_Scale needs (three settings, src/analyses.hpp:29-33)
// is repeated here because the rest of that function needs a working Boost.MultiArray (the
// grid analyses, which never touch these outputs). Only tests/, bench.py's CPU-baseline leg
// and __graft_entry__.smoke() may run what this builds.
//
// Extra, optional behaviour (never changes the catalogue): when PLAN_REF_DUMP=<dir> is set,
// stage arrays are written as raw little-endian binaries after each public call, using only
// public members of the reference classes:
//   tree.bin      sorted tree points: pos[3], vel[3] f64, mass, ath_density, new_density f64,
//                 original_id u32, sink flag u8 (after BuildTree; densities after Find)
//   keys.bin      96-bit Morton keys of the sorted points recomputed with the public
//                 MortonKey::Morton on the tree's own box (3 x u32, low word first)
//   nodes.bin     TreeNode array: center[3], half_width f64, begin, end, parent,
//                 first_daughter u32, orthant u16, num_daughters u8, level u8
//   knn.bin       for every `PLAN_REF_KNN_STRIDE`-th point: K_d neighbour (idx u32, dr2 f64)
//   hop.bin       densest-neighbour pointer of every point (public KNN + the same argmax rule)
//   clumps.bin    final clump map in key order: peak u32, n u32, M, Hill, com[3], vcom[3],
//                 J[3] f64, then n member tree indices (u32) in `indices` order
#include "global.hpp"
#include "tree.hpp"
#include "analyses.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

MPI_Wrapper *mpi = new MPI_Wrapper;
std::vector<Timer> timer(__time_type_count);
Basic_IO_Operations *progIO = new Basic_IO_Operations;

namespace {

template <class T>
void put(std::ofstream &f, const T &v) { f.write(reinterpret_cast<const char *>(&v), sizeof(T)); }

void dump_tree(const std::string &dir, DataSet<float, dim> &ds) {
    auto &t = ds.tree;
    std::ofstream f(dir + "/tree.bin", std::ios::binary);
    uint64_t n = t.num_particles;
    put(f, n);
    for (uint32_t i = 0; i < t.num_particles; ++i) {
        auto &p = t.particle_list[i];
        for (int d = 0; d < 3; ++d) put(f, p.pos[d]);
        for (int d = 0; d < 3; ++d) put(f, p.vel[d]);
        put(f, p.mass); put(f, p.ath_density); put(f, p.new_density);
        put(f, p.original_id);
        uint8_t s = p.sink_flag ? 1 : 0; put(f, s);
    }
    std::ofstream k(dir + "/keys.bin", std::ios::binary);
    put(k, n);
    for (uint32_t i = 0; i < t.num_particles; ++i) {
        auto key = t.Morton(t.particle_list[i].pos, 0);
        uint32_t w0 = (uint32_t)key, w1 = (uint32_t)(key >> 32), w2 = (uint32_t)(key >> 64);
        put(k, w0); put(k, w1); put(k, w2);
    }
    std::ofstream nf(dir + "/nodes.bin", std::ios::binary);
    uint64_t nn = t.num_nodes;
    put(nf, nn);
    for (int i = 0; i < t.num_nodes; ++i) {
        auto &nd = t.tree[i];
        for (int d = 0; d < 3; ++d) put(nf, nd.center[d]);
        put(nf, nd.half_width); put(nf, nd.begin); put(nf, nd.end); put(nf, nd.parent);
        put(nf, nd.first_daughter); put(nf, nd.orthant); put(nf, nd.num_daughters); put(nf, nd.level);
    }
}

void dump_after_find(const std::string &dir, DataSet<float, dim> &ds) {
    auto &t = ds.tree;
    auto &paras = progIO->numerical_parameters;
    dump_tree(dir, ds);  // refresh with new_density filled in
    unsigned stride = 1;
    if (const char *s = std::getenv("PLAN_REF_KNN_STRIDE")) stride = (unsigned)std::atoi(s);
    if (stride == 0) stride = 1;
    unsigned kd = paras.num_neighbors_in_knn_search, kh = paras.num_neighbors_to_hop;
    std::ofstream kf(dir + "/knn.bin", std::ios::binary);
    uint32_t hdr[3] = {t.num_particles, stride, kd};
    kf.write(reinterpret_cast<char *>(hdr), sizeof(hdr));
    std::vector<uint32_t> idx(std::max(kd, kh));
    std::vector<std::pair<int, double>> heap;
    double r = 0;
    for (uint32_t i = 0; i < t.num_particles; i += stride) {
        t.KNN_Search_OpenMP(t.particle_list[i].pos, kd, r, idx.data(), heap);
        for (unsigned j = 0; j < kd; ++j) { put(kf, (uint32_t)heap[j].first); put(kf, heap[j].second); }
    }
    // Densest-neighbour pointers, recomputed with the public KNN and the argmax rule of
    // src/tree.hpp:3719-3735 (the reference frees its own array inside FindPlanetesimals).
    std::ofstream hf(dir + "/hop.bin", std::ios::binary);
    uint64_t n = t.num_particles;
    put(hf, n);
    double thr = ds.planetesimal_list.density_threshold;
    for (uint32_t i = 0; i < t.num_particles; ++i) {
        uint32_t best = i;
        if (t.particle_list[i].new_density >= thr) {
            t.KNN_Search_OpenMP(t.particle_list[i].pos, kh, r, idx.data(), heap);
            double dmax = t.particle_list[i].new_density;
            for (unsigned j = 0; j < kh; ++j) {
                double dj = t.particle_list[idx[j]].new_density;
                if (dmax < dj) { best = idx[j]; dmax = dj; }
                else if (dmax == dj && best > idx[j]) best = idx[j];
            }
        }
        put(hf, best);
    }
    std::ofstream cf(dir + "/clumps.bin", std::ios::binary);
    uint64_t nc = ds.planetesimal_list.planetesimals.size();
    put(cf, nc);
    for (auto &it : ds.planetesimal_list.planetesimals) {
        auto &c = it.second;
        uint32_t peak = it.first, m = (uint32_t)c.indices.size();
        put(cf, peak); put(cf, m);
        put(cf, c.total_mass); put(cf, c.Hill_radius);
        for (int d = 0; d < 3; ++d) put(cf, c.center_of_mass[d]);
        for (int d = 0; d < 3; ++d) put(cf, c.vel_com[d]);
        for (int d = 0; d < 3; ++d) put(cf, c.J[d]);
        for (auto ix : c.indices) put(cf, ix);
    }
}

}  // namespace

int main(int argc, const char *argv[]) {
    mpi->Initialization(argc, argv);
    progIO->Initialize(argc, argv);
    mpi->DetermineLoop(progIO->num_files);
    const char *dump = std::getenv("PLAN_REF_DUMP");
    DataSet<float, dim> ds;
    const bool dvs = progIO->flags.density_vs_scale_flag != 0;
    // result files in BasicAnalysesPreWork's order (src/analyses.cpp:16-33)
    if (dvs) mpi->OpenFile(progIO->file_name.max_rhop_vs_scale_file);
    if (progIO->flags.find_clumps_flag) mpi->OpenFile(progIO->file_name.planetesimals_file);
    for (int lc = mpi->loop_begin; lc <= mpi->loop_end; lc += mpi->loop_step) {
        double t0 = Timer::GetCurrentTime();
        ds.particle_set.ReadLisFile(lc);
        if (dvs) {  // BasicAnalyses' settings for --Density_Vs_Scale (src/analyses.hpp:29-33)
            progIO->numerical_parameters.max_ghost_zone_width = progIO->numerical_parameters.max_half_width;
            ds.tree.max_leaf_size = std::pow(1U << dim, 2);
            progIO->flags.no_ghost_particle_flag = 1;
        }
        double t1 = Timer::GetCurrentTime();
        ds.particle_set.MakeGhostParticles(progIO->numerical_parameters);
        ds.tree.BuildTree(progIO->numerical_parameters, ds.particle_set);
        if (dvs) BasicAnalysesWithTree(ds, lc);
        double t2 = Timer::GetCurrentTime();
        ds.tree.FindPlanetesimals(ds, lc);
        ds.planetesimal_list.WriteBasicResults(lc);
        double t3 = Timer::GetCurrentTime();
        std::fprintf(stderr, "[ref] read %.4f s, ghost+tree %.4f s, find %.4f s, tree points %u\n",
                     t1 - t0, t2 - t1, t3 - t2, ds.tree.num_particles);
        if (dump) dump_after_find(dump, ds);
    }
    for (auto &f : mpi->result_files) mpi->CloseFile(f);
    return 0;
}

// --Save_Clumps member lists with every line formatted on the device.
//
// OutputSinglePlanetesimal (src/tree.hpp:5191-5222) writes, for each kept member of a clump
// (1 in `sampling`, starting with the first, in the clump's distance order), the member's id
// as setw(16) and its position, velocity and mass as setw(24) scientific with precision 16.
// Every field has a fixed width (an unsigned id fits in 16 columns, "%.16e" of any double in
// 24), so a line is always 185 bytes and line i starts at byte 185 i: one thread per line
// formats it with the exact conversions of fmt_e16.cuh. The host only gathers the members,
// copies them in and the text out, and writes one file per clump.
#include <sys/stat.h>

#include <cstdio>
#include <cstring>
#include <iomanip>
#include <sstream>
#include <string>
#include <vector>

#include "catalogue.h"
#include "fmt_e16.cuh"
#include "pipeline.h"

namespace plan {

namespace {

constexpr size_t kLine = 16 + 7 * 24 + 1;  // id, x y z, vx vy vz, mass, newline

struct ParRec {
    uint32_t orig, pad;
    double v[7];  // x, y, z, vx, vy, vz, mass
};
static_assert(sizeof(ParRec) == 64, "one member record is 64 bytes");

__global__ void k_parlist_lines(const ParRec *rec, uint64_t n, char *out) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ParRec r = rec[i];
    char line[kLine];
    fmt_u32_w16(r.orig, line);
    for (int j = 0; j < 7; ++j) fmt_e16_w24(r.v[j], line + 16 + 24 * j);
    line[kLine - 1] = '\n';
    char *o = out + i * kLine;
    for (size_t b = 0; b < kLine; ++b) o[b] = line[b];
}

}  // namespace

int write_parlists_device(Context &c, const plan_catalogue &cat, int file_number, uint32_t sampling, cudaStream_t s) {
    if (sampling == 0) sampling = 1;
    std::ostringstream sid;
    sid << std::setw(4) << std::setfill('0') << file_number;
    const std::string dir = "ParList." + sid.str();
    mkdir(dir.c_str(), 0755);
    const size_t nc = cat.clumps.size();
    std::vector<uint64_t> first(nc + 1, 0);
    for (size_t k = 0; k < nc; ++k) first[k + 1] = first[k] + (cat.clumps[k].orig.size() + sampling - 1) / sampling;
    const uint64_t L = first[nc];
    ParRec *h_rec = nullptr, *d_rec = nullptr;
    char *h_txt = nullptr, *d_txt = nullptr;
    int rc = kOk;
    if (L) {
        if (cudaMallocHost(&h_rec, L * sizeof(ParRec)) != cudaSuccess || cudaMallocHost(&h_txt, L * kLine) != cudaSuccess ||
            cudaMallocAsync(&d_rec, L * sizeof(ParRec), s) != cudaSuccess || cudaMallocAsync(&d_txt, L * kLine, s) != cudaSuccess) {
            cudaGetLastError();
            rc = kErrOutOfMemory;
        } else {
            for (size_t k = 0; k < nc; ++k) {
                const auto &cl = cat.clumps[k];
                uint64_t at = first[k];
                for (size_t q = 0; q < cl.orig.size(); q += sampling, ++at) {
                    ParRec &r = h_rec[at];
                    r.orig = cl.orig[q];
                    r.pad = 0;
                    for (int d = 0; d < 3; ++d) {
                        r.v[d] = cl.pos[3 * q + d];
                        r.v[3 + d] = cl.vel[3 * q + d];
                    }
                    r.v[6] = cl.mass[q];
                }
            }
            cudaMemcpyAsync(d_rec, h_rec, L * sizeof(ParRec), cudaMemcpyHostToDevice, s);
            k_parlist_lines<<<(unsigned)((L + 127) / 128), 128, 0, s>>>(d_rec, L, d_txt);
            c.launches++;
            cudaMemcpyAsync(h_txt, d_txt, L * kLine, cudaMemcpyDeviceToHost, s);
            if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) rc = kErrDevice;
        }
    }
    if (rc == kOk) {
        for (size_t k = 0; k < nc; ++k) {
            const std::string name = dir + "/" + std::to_string(cat.clumps[k].key) + ".txt";
            FILE *pf = std::fopen(name.c_str(), "w");
            if (!pf) {
                std::fprintf(stderr, "Error: Failed to open file: %s. But we proceed.\n", name.c_str());
                continue;
            }
            const size_t bytes = (size_t)(first[k + 1] - first[k]) * kLine;
            if (bytes && std::fwrite(h_txt + first[k] * kLine, 1, bytes, pf) != bytes) rc = kErrIo;
            std::fclose(pf);
        }
    }
    if (d_rec) cudaFreeAsync(d_rec, s);
    if (d_txt) cudaFreeAsync(d_txt, s);
    cudaStreamSynchronize(s);
    if (h_rec) cudaFreeHost(h_rec);
    if (h_txt) cudaFreeHost(h_txt);
    return rc;
}

}  // namespace plan

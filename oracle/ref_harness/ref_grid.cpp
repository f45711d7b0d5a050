// Runs the reference CPU grid A* (src/pathway/CPU-solver.cpp:80-146) on a
// binary .grid instance and writes the result as JSON.
//
//   ref_grid <instance.grid> <out.json>
//
// The .grid layout is the engine's own instance file: "UAG1", int32 H, W, sx,
// sy, ex, ey, uint64 nwords, then nwords little-endian uint64 words holding
// one bit per cell (bit id&63 of word id>>6, id = x*W+y, 1 = open).  Open
// cells become 0xFF and blocked cells 0x00 in Pathway::m_graph, exactly what
// the reference's `custom` input module stores (src/pathway/input/custom.cpp:14-26).
// The stdin parse is skipped by filling m_graph directly, so the timed region
// is CPUPathwaySolver::solve() alone.
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <queue>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "utils.hpp"
#include "ref_common.hpp"
#define private public
#include "pathway/pathway.hpp"
#include "pathway/CPU-solver.hpp"
#include "pathway/GPU-solver.hpp"
#undef private

// The GPU solver cannot be built here (it needs the absent moderngpu
// submodule and sm_35); Pathway's constructor only news it.
GPUPathwaySolver::GPUPathwaySolver(Pathway *pathway) : p(pathway), d(nullptr) {}
GPUPathwaySolver::~GPUPathwaySolver() {}
void GPUPathwaySolver::initialize() {}
bool GPUPathwaySolver::solve() { return false; }
void GPUPathwaySolver::getSolution(float *, vector<int> *) {}

int main(int argc, char **argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: ref_grid <instance.grid> <out.json>\n");
        return 2;
    }
    std::ifstream in(argv[1], std::ios::binary);
    char magic[4];
    int32_t hdr[6];
    uint64_t nwords = 0;
    in.read(magic, 4);
    in.read(reinterpret_cast<char *>(hdr), sizeof(hdr));
    in.read(reinterpret_cast<char *>(&nwords), 8);
    if (!in || std::memcmp(magic, "UAG1", 4) != 0) {
        std::fprintf(stderr, "bad instance file\n");
        return 2;
    }
    std::vector<uint64_t> words(nwords);
    in.read(reinterpret_cast<char *>(words.data()), nwords * 8);
    const int H = hdr[0], W = hdr[1];

    vm_options.emplace("width", boost::program_options::variable_value(W));
    vm_options.emplace("height", boost::program_options::variable_value(H));
    vm_options.emplace("input-module", boost::program_options::variable_value(std::string("custom")));

    Pathway p;
    p.m_graph.assign((size_t)H * W, 0);
    for (size_t id = 0; id < (size_t)H * W; ++id)
        p.m_graph[id] = (words[id >> 6] >> (id & 63)) & 1 ? 0xFF : 0x00;
    p.m_sx = hdr[2];
    p.m_sy = hdr[3];
    p.m_ex = hdr[4];
    p.m_ey = hdr[5];

    p.cpuSolver->initialize();
    auto t0 = std::chrono::steady_clock::now();
    bool ok = p.cpuSolver->solve();
    auto t1 = std::chrono::steady_clock::now();
    double secs = std::chrono::duration<double>(t1 - t0).count();

    FILE *out = std::fopen(argv[2], "w");
    if (!ok) {
        std::fprintf(out, "{\"solved\": false, \"solve_seconds\": %.6f}\n", secs);
        std::fclose(out);
        return 0;
    }
    float cost = 0;
    std::vector<int> path;
    size_t generated = p.cpuSolver->globalList.size();
    p.cpuSolver->getSolution(&cost, &path);
    std::fprintf(out, "{\"solved\": true, \"cost\": %.9g, \"generated\": %zu, \"solve_seconds\": %.6f, \"path\": [",
                 cost, generated, secs);
    for (size_t i = 0; i < path.size(); ++i)
        std::fprintf(out, i ? ", %d" : "%d", path[i]);
    std::fprintf(out, "]}\n");
    std::fclose(out);
    return 0;
}

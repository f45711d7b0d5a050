// Runs the reference CPU sliding-tile A* (src/puzzle/CPU-solver.hpp:276-493)
// and its pattern-database generator (src/puzzle/database.cpp:37-122).
//
//   ref_puzzle pdb <N> <cache_dir>                  build/cached PDB files only
//   ref_puzzle solve <N> <cache_dir> <in.txt> <out.jsonl>
//
// <in.txt> holds one instance per line: N*N tile numbers, 0 = blank, row-major
// (the order Puzzle::prepare reads from stdin, src/puzzle/puzzle.cu:91-98).
// The PDB files are cached in <cache_dir> under the reference's own names
// (database_<n>_<tiles>.bin, src/puzzle/database.cpp:86-122).
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <queue>
#include <sstream>
#include <string>
#include <unistd.h>
#include <vector>

#include "utils.hpp"
#include "ref_common.hpp"
#include "puzzle/storage.hpp"
#include "puzzle/database.hpp"
#include <boost/unordered_map.hpp>
#define private public
#include "puzzle/puzzle.cuh"
#include "puzzle/CPU-solver.hpp"
#undef private

// Out-of-line members of Puzzle normally compiled from src/puzzle/puzzle.cu,
// which also pulls in the GPU solver and so cannot be built here.
Puzzle::Puzzle() : n(0), d(nullptr) {}
Puzzle::~Puzzle() {}
string Puzzle::problemName() const { return "Tile Puzzle"; }
void Puzzle::prepare() {}
void Puzzle::cpuInitialize() {}
void Puzzle::gpuInitialize() {}
void Puzzle::cpuSolve() {}
void Puzzle::gpuSolve() {}
bool Puzzle::output() { return true; }

template <int N> static int run_solve(const char *in_path, const char *out_path) {
    std::ifstream in(in_path);
    FILE *out = std::fopen(out_path, "w");
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream ss(line);
        std::vector<uint8_t> tiles;
        int t;
        while (ss >> t) tiles.push_back((uint8_t)t);
        if ((int)tiles.size() != N * N) continue;
        Puzzle p;
        p.n = N;
        p.m_initialState = tiles;
        cpusolver::CPUPuzzleSolver<N> solver(&p);
        solver.initialize();
        auto t0 = std::chrono::steady_clock::now();
        bool ok = solver.solve();
        auto t1 = std::chrono::steady_clock::now();
        double secs = std::chrono::duration<double>(t1 - t0).count();
        if (!ok) {
            std::fprintf(out, "{\"solved\": false, \"solve_seconds\": %.6f}\n", secs);
            continue;
        }
        int steps = 0;
        std::vector<int> moves;
        size_t stored = solver.closeList.size();
        solver.getSolution(&steps, &moves);
        std::fprintf(out, "{\"solved\": true, \"steps\": %d, \"stored\": %zu, \"solve_seconds\": %.6f, \"moves\": [",
                     steps, stored, secs);
        for (size_t i = 0; i < moves.size(); ++i) std::fprintf(out, i ? ", %d" : "%d", moves[i]);
        std::fprintf(out, "]}\n");
        std::fflush(out);
    }
    std::fclose(out);
    return 0;
}

template <int N> static int run_pdb() {
    // The same pattern partitions CPUPuzzleSolver<N>::initialize uses
    // (src/puzzle/CPU-solver.hpp:43-102); fetchDatabase builds and caches.
    std::vector<std::vector<int>> tracked;
    if (N == 3) tracked = {{1, 2, 3, 4, 5, 6, 7, 8}};
    if (N == 4) tracked = {{1, 2, 3, 4, 5, 6, 9, 13}, {7, 8, 10, 11, 12, 14, 15}};
    if (N == 5)
        tracked = {{3, 4, 5, 10, 15, 20}, {2, 1, 6, 11, 16, 21}, {7, 8, 9, 12, 17, 22}, {13, 14, 18, 19, 23, 24}};
    for (auto &tr : tracked) {
        PatternDatabase pd(N, tr);
        std::vector<uint8_t> buf(pd.size());
        pd.fetchDatabase(buf.data());
    }
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: ref_puzzle pdb|solve <N> <cache_dir> [in out]\n");
        return 2;
    }
    std::string mode = argv[1];
    int n = std::atoi(argv[2]);
    std::string in_path = argc > 4 ? std::string(argv[4]) : "";
    std::string out_path = argc > 5 ? std::string(argv[5]) : "";
    if (!in_path.empty() && in_path[0] != '/') {
        char cwd[4096];
        if (getcwd(cwd, sizeof cwd)) in_path = std::string(cwd) + "/" + in_path;
    }
    if (!out_path.empty() && out_path[0] != '/') {
        char cwd[4096];
        if (getcwd(cwd, sizeof cwd)) out_path = std::string(cwd) + "/" + out_path;
    }
    if (chdir(argv[3]) != 0) {
        std::fprintf(stderr, "cannot enter %s\n", argv[3]);
        return 2;
    }
    if (mode == "pdb") return n == 3 ? run_pdb<3>() : n == 4 ? run_pdb<4>() : run_pdb<5>();
    if (mode == "solve" && argc == 6)
        return n == 3 ? run_solve<3>(in_path.c_str(), out_path.c_str())
               : n == 4 ? run_solve<4>(in_path.c_str(), out_path.c_str())
                        : run_solve<5>(in_path.c_str(), out_path.c_str());
    std::fprintf(stderr, "bad mode\n");
    return 2;
}

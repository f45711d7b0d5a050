// Solves problems read from stdin through the C++ host classes of
// uastar_solvers.hpp, driven the way the reference's Pathway::gpuSolve /
// Puzzle::gpuSolve drive their GPU solvers (construct, initialize, solve,
// getSolution).  Grids use the reference's custom input format
// (src/pathway/input/custom.cpp:14-26) after a header line:
//   pathway <height> <width>
//   <sx> <sy>
//   <ex> <ey>
//   <height x width ints, nonzero = open>
//   puzzle <n>
//   <n*n ints, 0 = blank>
// For each problem one line: "pathway solved <cost> <n> <ids...>" or
// "puzzle solved <steps> <n> <moves...>", "... unsolved", or "error <status>".
// argv[1]: the pattern-database cache directory ("." when absent, as in the
// reference; "" for none); where each puzzle's tables came from goes to
// stderr as "database cache|gpu".
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "uastar_solvers.hpp"

namespace {

// The reference's Pathway accessors (src/pathway/pathway.hpp:22-32).
struct Pathway {
    int m_sx, m_sy, m_ex, m_ey, m_width, m_height;
    std::vector<uint8_t> m_graph;
    int sx() const { return m_sx; }
    int sy() const { return m_sy; }
    int ex() const { return m_ex; }
    int ey() const { return m_ey; }
    int width() const { return m_width; }
    int height() const { return m_height; }
    const uint8_t *graph() const { return m_graph.data(); }
};

// The reference's Puzzle accessor (src/puzzle/puzzle.cuh:28-30).
struct Puzzle {
    std::vector<uint8_t> m_initialState;
    void initialState(std::vector<uint8_t> &data) { data = m_initialState; }
};

template <int N>
void solve_puzzle(Puzzle &pz, const std::string &cache_dir) {
    uastar_host::GPUPuzzleSolver<N, Puzzle> solver(&pz, 0, nullptr, cache_dir);
    solver.initialize();
    std::fprintf(stderr, "database %s\n", solver.databaseSource());
    if (!solver.solve()) {
        std::printf("puzzle unsolved\n");
        return;
    }
    int steps = 0;
    std::vector<int> moves;
    solver.getSolution(&steps, &moves);
    std::printf("puzzle solved %d %zu", steps, moves.size());
    for (int m : moves) std::printf(" %d", m);
    std::printf("\n");
}

}  // namespace

int main(int argc, char **argv) {
    const std::string cache_dir = argc > 1 ? argv[1] : ".";
    std::string kind;
    while (std::cin >> kind) {
        try {
            if (kind == "pathway") {
                Pathway p;
                std::cin >> p.m_height >> p.m_width >> p.m_sx >> p.m_sy >> p.m_ex >> p.m_ey;
                p.m_graph.resize((size_t)p.m_height * p.m_width);
                for (auto &c : p.m_graph) {
                    int t;
                    std::cin >> t;
                    c = t ? 0xFF : 0;
                }
                uastar_host::GPUPathwaySolver<Pathway> solver(&p);
                solver.initialize();
                if (!solver.solve()) {
                    std::printf("pathway unsolved\n");
                    continue;
                }
                float cost = 0;
                std::vector<int> path;
                solver.getSolution(&cost, &path);
                std::printf("pathway solved %.6f %zu", cost, path.size());
                for (int id : path) std::printf(" %d", id);
                std::printf("\n");
            } else if (kind == "puzzle") {
                int n;
                std::cin >> n;
                Puzzle pz;
                pz.m_initialState.resize((size_t)n * n);
                for (auto &t : pz.m_initialState) {
                    int v;
                    std::cin >> v;
                    t = (uint8_t)v;
                }
                if (n == 3)
                    solve_puzzle<3>(pz, cache_dir);
                else if (n == 4)
                    solve_puzzle<4>(pz, cache_dir);
                else
                    solve_puzzle<5>(pz, cache_dir);
            } else {
                std::printf("error %d\n", (int)UASTAR_BAD_INPUT);
                return 2;
            }
        } catch (const uastar_host::SolverError &e) {
            std::printf("error %d %s\n", (int)e.status(), e.what());
        }
        std::fflush(stdout);
    }
    return 0;
}

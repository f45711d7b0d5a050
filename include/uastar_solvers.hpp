/* C++ host classes over the C ABI (uastar_gpu.h) with the reference's solver
 * names and call sequence: construct from the problem object, initialize(),
 * solve() -> bool, getSolution(...).  They replace
 *   GPUPathwaySolver          (src/pathway/GPU-solver.hpp:20-36, GPU-solver.cu:129-354)
 *   gpusolver::GPUPuzzleSolver<N> (src/puzzle/GPU-solver.cuh:55-294)
 * inside the reference's Pathway::gpuInitialize / gpuSolve / output
 * (src/pathway/pathway.cpp:72-112) and Puzzle::gpu* (src/puzzle/puzzle.cu:115-205).
 *
 * The problem type is a template parameter with the reference's accessors:
 *   Pathway: graph() (H*W bytes, nonzero = open), width(), height(), sx(),
 *            sy(), ex(), ey()                     (src/pathway/pathway.hpp:22-32)
 *   Puzzle:  initialState(std::vector<uint8_t>&)  (src/puzzle/puzzle.cuh:28-30)
 * The device ordinal is a constructor argument (the reference reads
 * vm_options["ordinal"]).
 *
 * Differences from the reference, on purpose: the device is never reset
 * (the reference's initialize() calls cudaDeviceReset); solve() returns false
 * only when no path exists (grid) or the board is unsolvable (puzzle), and
 * every other failure — capacity, device, bad input — throws SolverError with
 * the engine's status and message instead of being ignored. */
#pragma once

#include <cstdint>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "uastar_gpu.h"

namespace uastar_host {

class SolverError : public std::runtime_error {
public:
    SolverError(int32_t status, const std::string &what) : std::runtime_error(what), status_(status) {}
    int32_t status() const { return status_; }

private:
    int32_t status_;
};

namespace detail {
// An engine owned by one solver object.
class Engine {
public:
    Engine(int ordinal, const uastar_config *cfg) : eng_(uastar_create(ordinal, cfg)) {
        if (!eng_) throw SolverError(UASTAR_CUDA_ERROR, "cannot create an engine on device " + std::to_string(ordinal));
    }
    ~Engine() { uastar_destroy(eng_); }
    Engine(const Engine &) = delete;
    Engine &operator=(const Engine &) = delete;
    uastar_engine *get() const { return eng_; }
    void check(int32_t rc, const char *what) const {
        if (rc != UASTAR_OK) throw SolverError(rc, std::string(what) + ": " + uastar_last_error(eng_));
    }

private:
    uastar_engine *eng_;
};
// The reference's disjoint patterns, in its tracked order
// (src/puzzle/CPU-solver.hpp:43-102), and its cache file names
// (src/puzzle/database.cpp:86-91).
inline std::vector<std::vector<int>> partitions(int n) {
    if (n == 3) return {{1, 2, 3, 4, 5, 6, 7, 8}};
    if (n == 4) return {{1, 2, 3, 4, 5, 6, 9, 13}, {7, 8, 10, 11, 12, 14, 15}};
    return {{3, 4, 5, 10, 15, 20}, {2, 1, 6, 11, 16, 21}, {7, 8, 9, 12, 17, 22}, {13, 14, 18, 19, 23, 24}};
}
inline std::string cache_name(int n, const std::vector<int> &tiles) {
    std::string s = "database_" + std::to_string(n);
    for (int t : tiles) s += "_" + std::to_string(t);
    return s + ".bin";
}
// Entries of a table over k tracked tiles: (n*n)! / (n*n - k)!.
inline size_t table_bytes(int n, size_t k) {
    size_t b = 1;
    for (size_t i = 0; i < k; ++i) b *= (size_t)(n * n) - i;
    return b;
}
}  // namespace detail

template <class PathwayT>
class GPUPathwaySolver {
public:
    explicit GPUPathwaySolver(PathwayT *pathway, int ordinal = 0, const uastar_config *cfg = nullptr)
        : p_(pathway), ordinal_(ordinal), has_cfg_(cfg != nullptr) {
        if (cfg) cfg_ = *cfg;
    }

    /* GPU-solver.cu:129-178: device setup and the graph upload (as a 1-bit
     * bitmap: bit id & 63 of word id >> 6, id = x * width + y). */
    void initialize() {
        eng_.reset(new detail::Engine(ordinal_, has_cfg_ ? &cfg_ : nullptr));
        const int32_t H = p_->height(), W = p_->width();
        const size_t cells = (size_t)H * (size_t)W;
        std::vector<uint64_t> words((cells + 63) / 64, 0);
        const uint8_t *g = p_->graph();
        for (size_t id = 0; id < cells; ++id)
            if (g[id]) words[id >> 6] |= 1ull << (id & 63);
        eng_->check(uastar_grid_load(eng_->get(), words.data(), H, W), "grid upload");
    }

    /* GPU-solver.cu:180-328: true iff a path from (sx, sy) to (ex, ey) exists. */
    bool solve() {
        res_ = uastar_grid_result{};
        const int32_t rc = uastar_grid_solve_loaded(engine().get(), p_->sx(), p_->sy(), p_->ex(), p_->ey(), &res_);
        if (rc == UASTAR_NO_SOLUTION) return false;
        engine().check(rc, "grid solve");
        return true;
    }

    /* GPU-solver.cu:330-354: the float32 cost along the path (as the
     * reference accumulates it) and the cell ids start -> goal. */
    void getSolution(float *optimal, std::vector<int> *pathList) {
        const int64_t n = uastar_grid_path(engine().get(), nullptr, 0);
        if (n < 0) throw SolverError((int32_t)-n, "no grid solution to read");
        pathList->resize((size_t)n);
        uastar_grid_path(engine().get(), reinterpret_cast<int32_t *>(pathList->data()), n);
        *optimal = res_.cost;
    }

    /* Beyond the reference: the exact cost (straight + diagonal * sqrt 2) and
     * the search statistics of the last solve. */
    const uastar_grid_result &result() const { return res_; }

private:
    static_assert(sizeof(int) == sizeof(int32_t), "path ids are written as int32");
    detail::Engine &engine() const {
        if (!eng_) throw SolverError(UASTAR_BAD_INPUT, "initialize() has not run");
        return *eng_;
    }
    PathwayT *p_;
    int ordinal_;
    bool has_cfg_;
    uastar_config cfg_{};
    std::unique_ptr<detail::Engine> eng_;
    uastar_grid_result res_{};
};

template <int N, class PuzzleT>
class GPUPuzzleSolver {
    static_assert(N >= 3 && N <= 5, "3x3, 4x4 or 5x5 boards");

public:
    /* `cache_dir`: where the reference's database_<n>_<tiles>.bin cache files
     * are read and written ("." = the working directory, as the reference
     * does; "" = no files). */
    explicit GPUPuzzleSolver(PuzzleT *puzzle, int ordinal = 0, const uastar_config *cfg = nullptr,
                             std::string cache_dir = ".")
        : p_(puzzle), ordinal_(ordinal), has_cfg_(cfg != nullptr), cache_dir_(std::move(cache_dir)) {
        if (cfg) cfg_ = *cfg;
    }

    /* GPU-solver.cuh:64-195: device setup and the disjoint pattern databases,
     * the way the reference's fetchDatabase treats its cache
     * (database.cpp:86-122): with every table's file present they are read
     * (a short file throws, where the reference exits); otherwise the tables
     * are built on the GPU and the missing files written. */
    void initialize() {
        eng_.reset(new detail::Engine(ordinal_, has_cfg_ ? &cfg_ : nullptr));
        const std::vector<std::vector<int>> parts = detail::partitions(N);
        std::vector<std::string> paths;
        bool all = !cache_dir_.empty();
        for (const auto &t : parts) {
            paths.push_back(cache_dir_ + "/" + detail::cache_name(N, t));
            if (all) {
                std::FILE *f = std::fopen(paths.back().c_str(), "rb");
                all = f != nullptr;
                if (f) std::fclose(f);
            }
        }
        const size_t total = (size_t)uastar_pdb_bytes(N);
        if (all) {
            std::vector<uint8_t> tables(total);
            size_t off = 0;
            for (size_t i = 0; i < parts.size(); ++i) {
                const size_t bytes = detail::table_bytes(N, parts[i].size());
                std::FILE *f = std::fopen(paths[i].c_str(), "rb");
                const size_t got = f ? std::fread(tables.data() + off, 1, bytes, f) : 0;
                if (f) std::fclose(f);
                if (got != bytes) throw SolverError(UASTAR_BAD_INPUT, paths[i] + " is not intact");
                off += bytes;
            }
            eng_->check(uastar_pdb_load(eng_->get(), N, tables.data(), (int64_t)total), "database load");
            source_ = "cache";
            return;
        }
        double ms = 0;
        eng_->check(uastar_pdb_build(eng_->get(), N, &ms), "database build");
        source_ = "gpu";
        if (cache_dir_.empty()) return;
        std::vector<uint8_t> tables(total);
        eng_->check(uastar_pdb_fetch(eng_->get(), N, tables.data(), (int64_t)total), "database fetch");
        size_t off = 0;
        for (size_t i = 0; i < parts.size(); ++i) {
            const size_t bytes = detail::table_bytes(N, parts[i].size());
            std::FILE *f = std::fopen(paths[i].c_str(), "rb");
            if (f) {
                std::fclose(f);  // present: the reference keeps its own file
            } else if (!(f = std::fopen(paths[i].c_str(), "wb")) ||
                       std::fwrite(tables.data() + off, 1, bytes, f) != bytes || std::fclose(f) != 0) {
                std::remove(paths[i].c_str());
                throw SolverError(UASTAR_BAD_INPUT, paths[i] + " cannot be written");
            }
            off += bytes;
        }
    }

    /* Where initialize() took the tables from: "cache" or "gpu". */
    const char *databaseSource() const { return source_; }

    /* GPU-solver.cuh:197-274: true iff the board is solvable (the reference
     * would search forever on an unsolvable one). */
    bool solve() {
        std::vector<uint8_t> tiles;
        p_->initialState(tiles);
        if (tiles.size() != (size_t)(N * N))
            throw SolverError(UASTAR_BAD_INPUT, "initial state must hold N*N tiles");
        res_ = uastar_puzzle_result{};
        const int32_t rc = uastar_puzzle_solve(engine().get(), N, tiles.data(), &res_);
        if (rc == UASTAR_NO_SOLUTION) return false;
        engine().check(rc, "puzzle solve");
        return true;
    }

    /* GPU-solver.cuh:276-287: the optimal move count and the moves start ->
     * goal, each 0..3 indexing the reference's DX/DY (GPU-kernel.cuh:494-495). */
    void getSolution(int *optimal, std::vector<int> *pathList) {
        const int64_t n = uastar_puzzle_moves(engine().get(), nullptr, 0);
        if (n < 0) throw SolverError((int32_t)-n, "no puzzle solution to read");
        pathList->resize((size_t)n);
        uastar_puzzle_moves(engine().get(), reinterpret_cast<int32_t *>(pathList->data()), n);
        *optimal = res_.steps;
    }

    const uastar_puzzle_result &result() const { return res_; }

private:
    detail::Engine &engine() const {
        if (!eng_) throw SolverError(UASTAR_BAD_INPUT, "initialize() has not run");
        return *eng_;
    }
    PuzzleT *p_;
    int ordinal_;
    bool has_cfg_;
    std::string cache_dir_;
    const char *source_ = "";
    uastar_config cfg_{};
    std::unique_ptr<detail::Engine> eng_;
    uastar_puzzle_result res_{};
};

}  // namespace uastar_host

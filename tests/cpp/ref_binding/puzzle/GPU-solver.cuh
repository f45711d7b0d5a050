/* The reference-side binding of the puzzle solver: what a maintainer puts in
 * place of the reference's src/puzzle/GPU-solver.cuh (class template
 * gpusolver::GPUPuzzleSolver<N> with a Puzzle* constructor, initialize(),
 * solve() -> bool and getSolution(int*, vector<int>*),
 * src/puzzle/GPU-solver.cuh:55-294).  The template keeps that name and
 * constructor, which src/puzzle/puzzle.cu calls, and runs the GA* engine
 * through include/uastar_solvers.hpp, with the reference's pattern-database
 * cache files in the working directory.  Found before the reference's own
 * header by include order. */
#pragma once
#include "uastar_solvers.hpp"
#include "utils.hpp"

class Puzzle;

namespace gpusolver {
template <int N> class GPUPuzzleSolver : public uastar_host::GPUPuzzleSolver<N, Puzzle> {
public:
    explicit GPUPuzzleSolver(Puzzle *puzzle)
        : uastar_host::GPUPuzzleSolver<N, Puzzle>(
              puzzle, vm_options.count("ordinal") ? vm_options["ordinal"].as<int>() : 0) {}
};
}  // namespace gpusolver

/* Drives the reference's own problem classes -- Pathway
 * (src/pathway/pathway.cpp) and Puzzle (src/puzzle/puzzle.cu), compiled
 * unmodified from the reference's sources -- through the call sequence of
 * the reference's solve_problem (src/main.cpp:60-110): prepare, CPU and GPU
 * initialize, CPU and GPU solve, output (which compares the two results and
 * fails on a mismatch).  The GPU half runs on this repository's engine
 * through the binding headers in tests/cpp/ref_binding/.
 *
 *   ref_problem_driver pathway <H> <W> [--no-cpu|--no-gpu] < custom-format grid
 *   ref_problem_driver puzzle <N> [--no-cpu|--no-gpu] < N*N tiles
 *
 * Exit status: 0 when output() accepts the results, 1 when it reports the
 * CPU and GPU results inconsistent, 3 when the engine raises (e.g. no GPU).
 * Test infrastructure only. */
#include <cstdio>
#include <cstring>
#include <string>

#include "ref_common.hpp"
#include "pathway/pathway.hpp"
#include "puzzle/puzzle.cuh"
#include "uastar_solvers.hpp"

int main(int argc, char **argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: ref_problem_driver pathway <H> <W> | puzzle <N> [--no-cpu|--no-gpu]\n");
        return 2;
    }
    const std::string mode = argv[1];
    int next = 3;
    if (mode == "pathway") {
        if (argc < 4) return 2;
        vm_options["height"] = boost::program_options::variable_value(std::atoi(argv[2]));
        vm_options["width"] = boost::program_options::variable_value(std::atoi(argv[3]));
        vm_options["input-module"] = boost::program_options::variable_value(std::string("custom"));
        next = 4;
    } else if (mode == "puzzle") {
        vm_options["width"] = boost::program_options::variable_value(std::atoi(argv[2]));
    } else {
        return 2;
    }
    bool use_cpu = true, use_gpu = true;
    for (int i = next; i < argc; ++i) {
        if (!std::strcmp(argv[i], "--no-cpu")) use_cpu = false;
        if (!std::strcmp(argv[i], "--no-gpu")) use_gpu = false;
    }
    try {
        Problem *problem = mode == "pathway" ? static_cast<Problem *>(new Pathway()) : new Puzzle();
        problem->prepare();
        if (use_cpu) problem->cpuInitialize();
        if (use_gpu) problem->gpuInitialize();
        if (use_cpu) problem->cpuSolve();
        if (use_gpu) problem->gpuSolve();
        const bool ok = problem->output();
        delete problem;
        if (!ok) {
            std::printf("ERROR: Output of the CPU and GPU is not consistent!\n");
            return 1;
        }
    } catch (const uastar_host::SolverError &e) {
        std::printf("engine error: %s\n", e.what());
        return 3;
    }
    return 0;
}

/* The reference-side binding of the grid solver: what a maintainer puts in
 * place of the reference's src/pathway/GPU-solver.hpp (which declares class
 * GPUPathwaySolver with a Pathway* constructor, initialize(), solve() -> bool
 * and getSolution(float*, vector<int>*), src/pathway/GPU-solver.hpp:20-36).
 * The class keeps that name and constructor, which src/pathway/pathway.cpp
 * calls, and runs the GA* engine through include/uastar_solvers.hpp; the
 * device ordinal comes from the reference's --ordinal option
 * (src/main.cpp:141).  Found before the reference's own header by include
 * order (this directory is searched first). */
#pragma once
#include "uastar_solvers.hpp"
#include "utils.hpp"

class Pathway;

class GPUPathwaySolver : public uastar_host::GPUPathwaySolver<Pathway> {
public:
    explicit GPUPathwaySolver(Pathway *pathway)
        : uastar_host::GPUPathwaySolver<Pathway>(
              pathway, vm_options.count("ordinal") ? vm_options["ordinal"].as<int>() : 0) {}
};

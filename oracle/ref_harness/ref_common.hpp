// Shared globals the reference's sources expect from its CLI driver
// (src/main.cpp:39-48 defines vm_options, random_engine, help, debug).
// Test infrastructure only: this harness links the reference's own CPU
// solvers, compiled unmodified from their source tree, so that the oracle
// restatement under oracle/ can be checked against them.
#pragma once
#include <cstdio>
#include <cstdlib>
#include "utils.hpp"

boost::program_options::variables_map vm_options;
boost::mt19937 random_engine;
bool debug = false;
void help() {
    std::fprintf(stderr, "reference harness: bad options\n");
    std::exit(2);
}

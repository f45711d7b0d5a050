// Parallel iterative-deepening A* (IDA*) passes for the sliding-tile
// puzzles: the exact phase of the memory-bounded mode.
//
// One pass searches every path whose f = g + h stays at or below a threshold
// t, depth-first, with memory proportional to the depth only (no dedup
// table).  The start's tree is cut at a fixed depth on the host into roots
// (move sequences without immediate reversal, as the search itself prunes);
// every thread takes roots from a queue and searches each one's subtree with
// a stack of at most kMaxDepth levels in its own local memory.  A pass that
// finds no goal proves the optimum above t and reports the least f it cut
// off, the next threshold (Korf, "Depth-first iterative-deepening: an optimal
// admissible tree search", 1985).  With an admissible h the first pass that
// finds a goal finds an optimal solution.
#pragma once
#include <cstdint>

#include "ga_device.cuh"
#include "ga_problems.cuh"

namespace uastar {

// A root of the cut tree: its board (narrow keys use lo only), depth, the
// move that reached it (+1, 0 for the start) and the moves from the start,
// 2 bits each, first move in the lowest bits.
struct IdaRoot {
    unsigned long long lo, hi;
    uint32_t g;
    uint32_t last;
    unsigned long long prefix;
};

constexpr uint32_t kIdaMaxMoves = 256;  // longest solution a pass records

// Pass state, zeroed by the host before each pass (min_exceed set to all ones).
struct IdaPass {
    uint32_t next_root;   // root queue
    uint32_t found;       // 1: a goal was reached (the first finder records it)
    uint32_t stopped;     // 1: the time limit cut the pass short; 2: a subtree was deeper than the stack
    uint32_t min_exceed;  // least f above the threshold among the cut-off nodes
    unsigned long long nodes;
    uint32_t found_root;
    uint32_t found_len;   // moves below the root
    uint8_t moves[kIdaMaxMoves];
};

template <class P> __device__ __forceinline__ typename P::Key ida_key(const IdaRoot &r) {
    if constexpr (P::kWide)
        return Key128{r.lo, r.hi};
    else
        return (uint64_t)r.lo;
}

template <class P, int kMaxDepth>
__global__ void __launch_bounds__(128) k_ida_pass(P prob, const IdaRoot *roots, uint32_t nroots, uint32_t t,
                                                  IdaPass *out, unsigned long long budget_ns) {
    using Key = typename P::Key;
    // the pass ends budget_ns after this thread started (the threads of a
    // launch start together: the grid fits the GPU at once)
    const unsigned long long deadline_ns = globaltimer_ns() + budget_ns;
    Key ks[kMaxDepth + 1];
    uint32_t as[kMaxDepth + 1];
    uint8_t rem[kMaxDepth + 1];
    unsigned long long nodes = 0, next_check = 1024;
    uint32_t minx = ~0u;
    bool quit = false;
    while (!quit) {
        if (ldcg_u32(&out->found) || ldcg_u32(&out->stopped)) break;
        if (globaltimer_ns() > deadline_ns) {
            atomicCAS(&out->stopped, 0u, 1u);
            break;
        }
        const uint32_t i = atomicAdd(&out->next_root, 1u);
        if (i >= nroots) break;
        const IdaRoot r = roots[i];
        P q = prob;
        q.start = ida_key<P>(r);
        const uint32_t a0 = q.start_aux() | (r.last << P::kLastMoveShift);
        const uint32_t g0 = r.g;
        const uint32_t f0 = g0 + P::hsum(a0);
        if (f0 > t) {
            minx = min(minx, f0);
            continue;
        }
        ks[0] = q.start;
        as[0] = a0;
        rem[0] = (uint8_t)prob.moves(ks[0], a0);
        int d = 0;
        while (d >= 0) {
            if (rem[d] == 0) {
                --d;
                continue;
            }
            const int mv = __ffs(rem[d]) - 1;
            rem[d] &= (uint8_t)(rem[d] - 1);
            typename P::Succ sc;
            prob.succ_begin(ks[d], g0 + d, as[d], mv, sc);
            uint32_t naux;
            uint64_t nf;
            prob.succ_end(sc, as[d], mv, naux, nf);
            ++nodes;
            if (nf > t) {
                minx = min(minx, (uint32_t)nf);
                continue;
            }
            if (prob.is_goal(sc.key)) {
                if (atomicCAS(&out->found, 0u, 1u) == 0u) {
                    const uint32_t len = (uint32_t)d + 1;
                    out->found_root = i;
                    out->found_len = len;
                    for (int j = 1; j <= d; ++j) out->moves[j - 1] = (uint8_t)((as[j] >> P::kLastMoveShift) - 1);
                    out->moves[d] = (uint8_t)mv;
                }
                quit = true;
                break;
            }
            if (d + 1 >= kMaxDepth) {
                atomicCAS(&out->stopped, 0u, 2u);
                quit = true;
                break;
            }
            ++d;
            ks[d] = sc.key;
            as[d] = naux;
            rem[d] = (uint8_t)prob.moves(ks[d], naux);
            if (nodes >= next_check) {  // another thread's goal, or the time limit
                next_check = nodes + 1024;
                if (ldcg_u32(&out->found)) {
                    quit = true;
                    break;
                }
                if (globaltimer_ns() > deadline_ns) {
                    atomicCAS(&out->stopped, 0u, 1u);
                    quit = true;
                    break;
                }
            }
        }
    }
    if (nodes) atomicAdd(&out->nodes, nodes);
    if (minx != ~0u) atomicMin(&out->min_exceed, minx);
}

}  // namespace uastar

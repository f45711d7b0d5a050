// Host-side engine object shared by the engine's translation units
// (engine.cu: plain solves; pdb.cu: pattern databases; batch.cu: batched
// and serving engines).  Not part of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/uastar_gpu.h"

namespace uastar {

// Grow-only device allocation.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need) {
        if (need <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, need);
        if (e == cudaSuccess)
            bytes = need;
        else
            (void)cudaGetLastError();  // an allocation failure is reported here, not by the next launch check
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T> T *as() const { return static_cast<T *>(p); }
};

// A 3x3 / 4x4 board packed as the search's 64-bit key (cell c in bits 4c..4c+3).
inline uint64_t pack_board(int n, const uint8_t *tiles) {
    uint64_t k = 0;
    for (int i = 0; i < n * n; ++i) k |= (uint64_t)(tiles[i] & 15) << (4 * i);
    return k;
}

// Solvability of a valid board: the goal has no inversions and the blank in
// row n-1.  A horizontal move keeps the inversion parity; a vertical move
// changes it by n-1 and moves the blank one row.  So a board is solvable iff
// inversions are even (n odd), or inversions + blank row has the parity of
// n-1 (n even).
inline bool board_solvable(int n, const uint8_t *tiles) {
    int inv = 0, brow = 0;
    for (int i = 0; i < n * n; ++i) {
        if (!tiles[i]) {
            brow = i / n;
            continue;
        }
        for (int j = i + 1; j < n * n; ++j)
            if (tiles[j] && tiles[j] < tiles[i]) ++inv;
    }
    if (n & 1) return (inv & 1) == 0;
    return ((inv + brow) & 1) == ((n - 1) & 1);
}

struct ServeState;  // batch.cu

}  // namespace uastar

struct uastar_engine {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    uastar_config cfg{};
    int sms = 0;
    std::string err;
    std::atomic<int64_t> launches{0};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    // plain engine buffers
    uastar::DevBuf tab, heaps, heap_size, cand, team, walk, bitmap;
    uastar::DevBuf tab_next, grow_map;  // table growth of a paused search
    // first table of a 3x3 / 4x4 plain solve, log2 slots (0: 2^20 / 2^22);
    // the batched engine raises it for the puzzles it escalates, which have
    // already filled a cluster's partition or round budget
    int puzzle_log2_start = 0;
    uastar::DevBuf sortb;               // per-round successor sort (dedup = 1), uastar_sort_keys
    uastar::DevBuf ida;                 // memory-bounded mode: IDA* roots and pass state
    // launch-configuration queries of the plain engine, made once per shape:
    // the dynamic shared memory limit set per kernel, and co-resident CTAs
    // per SM per (kernel, block, shared memory)
    std::map<const void *, size_t> smem_limit;
    std::map<std::tuple<const void *, uint32_t, size_t>, int> occupancy;
    int32_t gH = 0, gW = 0;
    bool grid_loaded = false;
    // pattern databases, indexed by board side
    uastar::DevBuf pdb[6];
    bool pdb_ready[6] = {false, false, false, false, false, false};

    // last plain solve
    int last_kind = 0;          // UASTAR_KIND_GRID / UASTAR_KIND_PUZZLE
    bool last_ok = false;
    uint32_t last_goal_slot = 0;
    int32_t lsx = 0, lsy = 0, lex = 0, ley = 0;
    int32_t last_n = 0;
    uint8_t last_tiles[25] = {0};
    bool path_cached = false;
    std::vector<int32_t> path;  // grid: cell ids; puzzle: moves

    // batched / serving engines
    uastar::DevBuf b_desc, b_out, b_queue, b_bitmaps, b_tab, b_heaps, b_hsize, b_cand, b_walk,
        b_walklen, b_cstate, b_cnext;
    uastar::ServeState *serve = nullptr;  // owned; released by uastar_serve_stop
    // instantiated launch graphs of the batched engine, one per launch shape
    // (cluster size, CTAs, CTA size, shared memory); each call captures its
    // launch and updates the matching executable graph in place
    std::map<std::tuple<int, int, int, size_t>, cudaGraphExec_t> b_graphs;

    void set_err(const std::string &s) { err = s; }
};

namespace uastar {
// engine.cu
int32_t fail_cuda(uastar_engine *eng, cudaError_t e, const char *what);
// Fill `bytes` (a multiple of 16) at `p` with 0xFF on `stream` using the whole GPU.
int32_t fill_ff_async(uastar_engine *eng, void *p, size_t bytes, cudaStream_t stream);
// pdb.cu
int32_t pdb_build_device(uastar_engine *eng, int n, double *ms);
// batch.cu: the batched engine keeps its team regions, heaps and bitmaps for
// the next batch; a caller that needs the memory (the serving loop, a plain
// solve that cannot get its table) gives them back.
void release_batch_buffers(uastar_engine *eng);
}  // namespace uastar

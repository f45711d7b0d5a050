// Disjoint pattern databases built on the GPU by level-synchronous breadth-
// first search over pattern ranks, and the C-ABI calls that load, build and
// fetch them.
//
// Semantics are those of the reference's generator (src/puzzle/database.cpp:
// 37-84): the blank is not tracked; from the goal abstraction (tile v on cell
// v-1) a tracked tile may slide into any adjacent cell that holds no tracked
// tile, at cost 1; entries are uint8 distances, 0xFF = unreached.  BFS
// distances are unique, so the tables equal the reference's byte for byte.
// The ranking is the reference's mixed-radix partial-permutation code
// (database.cpp:140-199), restated with bit masks: the cell of tracked tile j
// is the v_j-th cell not used by tiles < j.
#include <cuda_runtime.h>

#include <chrono>
#include <cstring>
#include <vector>

#include "engine_internal.h"
#include "ga_problems.cuh"

using namespace uastar;

namespace uastar {

// One BFS level: every entry equal to d expands; unreached neighbours get d+1.
// Threads scan 16 entries each (one 16-byte load), so the level scan runs at
// streaming bandwidth and only the expansions make random accesses.  Racing
// writers of a neighbour all store the same value.
template <int N, int P>
__global__ void __launch_bounds__(256) k_pdb_level(uint8_t *table, uint64_t size, uint32_t d,
                                                   uint32_t *changed) {
    constexpr int NN = N * N;
    constexpr int K = PuzzlePatterns<N>::count(P);
    const uint64_t chunks = (size + 15) / 16;
    bool any = false;
    for (uint64_t cidx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; cidx < chunks;
         cidx += (uint64_t)gridDim.x * blockDim.x) {
        uint4 v;
        const uint64_t r0 = cidx * 16;
        if (r0 + 16 <= size) {
            v = __ldcg(reinterpret_cast<const uint4 *>(table + r0));
        } else {
            uint8_t tmp[16];
            for (int i = 0; i < 16; ++i) tmp[i] = r0 + i < size ? __ldcg(table + r0 + i) : 0xFF;
            memcpy(&v, tmp, 16);
        }
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll 1
        for (int i = 0; i < 16; ++i) {
            if (((w[i >> 2] >> (8 * (i & 3))) & 0xFFu) != d) continue;
            // decode rank -> cells of the K tracked tiles
            uint64_t code = r0 + i;
            uint32_t pos[K];
            uint32_t used = 0;
#pragma unroll
            for (int j = 0; j < K; ++j) {
                const uint32_t m = pattern_mult<N>(P, j + 1);
                const uint32_t vj = (uint32_t)(code / m);
                code -= (uint64_t)vj * m;
                const uint32_t cell = __fns(~used, 0, (int)vj + 1);
                pos[j] = cell;
                used |= 1u << cell;
            }
            // every tracked tile, every direction
#pragma unroll
            for (int j = 0; j < K; ++j) {
                const int c = (int)pos[j], cx = c / N, cy = c % N;
#pragma unroll
                for (int dir = 0; dir < 4; ++dir) {
                    const int nx = cx + (dir == 0 ? 1 : dir == 1 ? -1 : 0);
                    const int ny = cy + (dir == 2 ? 1 : dir == 3 ? -1 : 0);
                    if (nx < 0 || nx >= N || ny < 0 || ny >= N) continue;
                    const uint32_t q = (uint32_t)(nx * N + ny);
                    if (used >> q & 1u) continue;
                    uint32_t u2 = 0, r = 0;
#pragma unroll
                    for (int t = 0; t < K; ++t) {
                        const uint32_t p = t == j ? q : pos[t];
                        r += (p - __popc(u2 & ((1u << p) - 1u))) * pattern_mult<N>(P, t + 1);
                        u2 |= 1u << p;
                    }
                    if (__ldcg(table + r) == 0xFF) {
                        table[r] = (uint8_t)(d + 1);
                        any = true;
                    }
                }
            }
        }
    }
    if (__syncthreads_or(any) && threadIdx.x == 0) *changed = 1u;
    (void)NN;
}

__global__ void k_pdb_set(uint8_t *table, uint64_t idx) { table[idx] = 0; }

}  // namespace uastar

namespace {

struct PatternDesc {
    int n, k;
    int tiles[8];
    uint64_t size, offset;
};

std::vector<PatternDesc> patterns_of(int n) {
    std::vector<PatternDesc> v;
    if (n == 3) {
        PatternDesc p{3, 8, {1, 2, 3, 4, 5, 6, 7, 8}, 362880ull, 0};
        v.push_back(p);
    } else if (n == 4) {
        PatternDesc a{4, 8, {1, 2, 3, 4, 5, 6, 9, 13}, 518918400ull, 0};
        PatternDesc b{4, 7, {7, 8, 10, 11, 12, 14, 15, 0}, 57657600ull, 518918400ull};
        v.push_back(a);
        v.push_back(b);
    } else if (n == 5) {
        // src/puzzle/CPU-solver.hpp:71-102, in its tracked order
        const int t[4][6] = {{3, 4, 5, 10, 15, 20}, {2, 1, 6, 11, 16, 21}, {7, 8, 9, 12, 17, 22},
                             {13, 14, 18, 19, 23, 24}};
        for (int p = 0; p < 4; ++p) {
            PatternDesc d{5, 6, {t[p][0], t[p][1], t[p][2], t[p][3], t[p][4], t[p][5], 0, 0}, 127512000ull,
                          (uint64_t)p * 127512000ull};
            v.push_back(d);
        }
    }
    return v;
}

// Rank of the goal abstraction (tile t on cell t-1), host side.
uint64_t goal_rank(const PatternDesc &p) {
    uint64_t code = 0;
    uint32_t used = 0;
    for (int j = 0; j < p.k; ++j) {
        const uint32_t cell = (uint32_t)(p.tiles[j] - 1);
        uint32_t below = 0;
        for (uint32_t c = 0; c < cell; ++c) below += (used >> c) & 1u;
        uint64_t m = 1;
        for (int i = j + 1; i < p.k; ++i) m *= (uint64_t)(p.n * p.n - i);
        code += (uint64_t)(cell - below) * m;
        used |= 1u << cell;
    }
    return code;
}

__global__ void k_pdb_max(const uint8_t *t, uint64_t n, uint32_t *mx) {
    uint32_t m = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        m = max(m, (uint32_t)t[i]);
    atomicMax(mx, m);
}

// Fails unless every entry is <= limit.
int32_t check_max(uastar_engine *eng, const uint8_t *t, uint64_t n, uint32_t limit) {
    uastar::DevBuf d;
    cudaError_t e;
    if ((e = d.ensure(64)) != cudaSuccess) return fail_cuda(eng, e, "pdb check");
    cudaMemsetAsync(d.p, 0, 4, eng->stream);
    k_pdb_max<<<eng->sms * 4, 256, 0, eng->stream>>>(t, n, d.as<uint32_t>());
    eng->launches++;
    uint32_t mx = 0;
    cudaMemcpyAsync(&mx, d.p, 4, cudaMemcpyDeviceToHost, eng->stream);
    if ((e = cudaStreamSynchronize(eng->stream)) != cudaSuccess) return fail_cuda(eng, e, "pdb check");
    if (mx > limit) {
        eng->set_err("pattern database entry above the search's field width");
        return UASTAR_BAD_INPUT;
    }
    return UASTAR_OK;
}

template <int N, int P>
int32_t build_one(uastar_engine *eng, uint8_t *table, uint64_t size, uint64_t goal) {
    cudaError_t e;
    if ((e = cudaMemsetAsync(table, 0xFF, size, eng->stream)) != cudaSuccess) return fail_cuda(eng, e, "pdb clear");
    k_pdb_set<<<1, 1, 0, eng->stream>>>(table, goal);
    eng->launches++;
    uastar::DevBuf flag;
    if ((e = flag.ensure(64)) != cudaSuccess) return fail_cuda(eng, e, "pdb flag");
    uint32_t *d_changed = flag.as<uint32_t>();
    uint32_t *h_changed = nullptr;
    if ((e = cudaMallocHost(&h_changed, sizeof(uint32_t))) != cudaSuccess) {
        flag.release();
        return fail_cuda(eng, e, "pdb host flag");
    }
    const uint64_t chunks = (size + 15) / 16;
    const int blocks = (int)std::min<uint64_t>((chunks + 255) / 256, (uint64_t)eng->sms * 16);
    int32_t rc = UASTAR_OK;
    for (uint32_t d = 0; d < 254; ++d) {
        cudaMemsetAsync(d_changed, 0, 4, eng->stream);
        k_pdb_level<N, P><<<blocks, 256, 0, eng->stream>>>(table, size, d, d_changed);
        eng->launches++;
        cudaMemcpyAsync(h_changed, d_changed, 4, cudaMemcpyDeviceToHost, eng->stream);
        if ((e = cudaStreamSynchronize(eng->stream)) != cudaSuccess) {
            rc = fail_cuda(eng, e, "pdb level");
            break;
        }
        if (!*h_changed) break;
    }
    cudaFreeHost(h_changed);
    flag.release();
    return rc;
}

}  // namespace

namespace uastar {

int32_t pdb_build_device(uastar_engine *eng, int n, double *ms) {
    const auto pats = patterns_of(n);
    if (pats.empty()) {
        eng->set_err("pattern databases exist for n = 3, 4 and 5");
        return UASTAR_BAD_INPUT;
    }
    const int64_t bytes = uastar_pdb_bytes(n);
    cudaError_t e;
    if ((e = eng->pdb[n].ensure((size_t)bytes + 64)) != cudaSuccess) return fail_cuda(eng, e, "alloc pdb");
    eng->pdb_ready[n] = false;
    uint8_t *base = eng->pdb[n].as<uint8_t>();
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, eng->stream);
    int32_t rc = UASTAR_OK;
    if (n == 3) {
        rc = build_one<3, 0>(eng, base, pats[0].size, goal_rank(pats[0]));
    } else if (n == 4) {
        rc = build_one<4, 0>(eng, base + pats[0].offset, pats[0].size, goal_rank(pats[0]));
        if (!rc) rc = build_one<4, 1>(eng, base + pats[1].offset, pats[1].size, goal_rank(pats[1]));
    } else {
        rc = build_one<5, 0>(eng, base + pats[0].offset, pats[0].size, goal_rank(pats[0]));
        if (!rc) rc = build_one<5, 1>(eng, base + pats[1].offset, pats[1].size, goal_rank(pats[1]));
        if (!rc) rc = build_one<5, 2>(eng, base + pats[2].offset, pats[2].size, goal_rank(pats[2]));
        if (!rc) rc = build_one<5, 3>(eng, base + pats[3].offset, pats[3].size, goal_rank(pats[3]));
        // the 5x5 search keeps each part in 7 bits
        if (!rc) rc = check_max(eng, base, (uint64_t)bytes, 127);
    }
    cudaEventRecord(b, eng->stream);
    cudaEventSynchronize(b);
    float t = 0;
    cudaEventElapsedTime(&t, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (ms) *ms = t;
    if (!rc) eng->pdb_ready[n] = true;
    return rc;
}

}  // namespace uastar

extern "C" {

int64_t uastar_pdb_bytes(int32_t n) {
    if (n == 3) return 362880;
    if (n == 4) return 518918400ll + 57657600ll;
    if (n == 5) return 4ll * 127512000ll;
    return 0;
}

int32_t uastar_pdb_build(uastar_engine *eng, int32_t n, double *build_ms) {
    if (!eng) return UASTAR_BAD_INPUT;
    cudaSetDevice(eng->device);
    return pdb_build_device(eng, n, build_ms);
}

int32_t uastar_pdb_load(uastar_engine *eng, int32_t n, const uint8_t *tables, int64_t bytes) {
    if (!eng) return UASTAR_BAD_INPUT;
    const int64_t need = uastar_pdb_bytes(n);
    if (!need || !tables || bytes != need) {
        eng->set_err("pdb_load: wrong side or byte count");
        return UASTAR_BAD_INPUT;
    }
    cudaSetDevice(eng->device);
    cudaError_t e;
    if ((e = eng->pdb[n].ensure((size_t)need + 64)) != cudaSuccess) return fail_cuda(eng, e, "alloc pdb");
    if ((e = cudaMemcpyAsync(eng->pdb[n].p, tables, (size_t)need, cudaMemcpyHostToDevice, eng->stream)) !=
        cudaSuccess)
        return fail_cuda(eng, e, "pdb upload");
    if ((e = cudaStreamSynchronize(eng->stream)) != cudaSuccess) return fail_cuda(eng, e, "pdb upload");
    eng->pdb_ready[n] = false;
    // the 5x5 search keeps each table's value in 7 bits of the node record
    if (n == 5)
        if (int32_t rc = check_max(eng, eng->pdb[n].as<uint8_t>(), (uint64_t)need, 127)) return rc;
    eng->pdb_ready[n] = true;
    return UASTAR_OK;
}

int32_t uastar_pdb_fetch(uastar_engine *eng, int32_t n, uint8_t *out, int64_t bytes) {
    if (!eng) return UASTAR_BAD_INPUT;
    const int64_t need = uastar_pdb_bytes(n);
    if (!need || !out || bytes != need || !eng->pdb_ready[n]) {
        eng->set_err("pdb_fetch: tables not resident or wrong byte count");
        return UASTAR_BAD_INPUT;
    }
    cudaSetDevice(eng->device);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(out, eng->pdb[n].p, (size_t)need, cudaMemcpyDeviceToHost, eng->stream)) !=
        cudaSuccess)
        return fail_cuda(eng, e, "pdb download");
    if ((e = cudaStreamSynchronize(eng->stream)) != cudaSuccess) return fail_cuda(eng, e, "pdb download");
    return UASTAR_OK;
}

}  // extern "C"

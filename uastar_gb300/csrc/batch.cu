// Batched persistent engine and continuous-batching serving loop.
//
// Both run GA* with one CTA per instance (a BlockTeam: the CTA's threads are
// the instance's heaps and every round barrier is a __syncthreads), so many
// instances of uneven size progress side by side on the 152 SMs.
//
//  - uastar_batch_solve: a persistent kernel whose CTAs take instances from a
//    device work queue (largest estimate first), each with its own dedup
//    partition in one table arena and the CTA's own heap slice; the launch
//    sequence is captured once into a CUDA graph.  Instances that overflow
//    their partition or heaps are re-run in a further wave with 4x the space.
//  - uastar_serve_*: a host thread admits requests by their estimated heap +
//    partition bytes against a budget, gives each a resident slot whose search
//    state (team state, heaps, partition) stays on the device between
//    quanta, launches one persistent kernel per quantum that advances every
//    resident request by a bounded number of rounds, retires finished ones
//    and backfills from the queue.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <numeric>
#include <vector>

#include "engine_internal.h"
#include "ga_device.cuh"
#include "ga_problems.cuh"
#include "ga_search.cuh"
#include "ga_grow.cuh"

using namespace uastar;

namespace uastar {

struct InstDesc {
    int32_t kind, n, H, W, sx, sy, ex, ey;
    uint64_t bm_word;     // first 32-bit word of the bitmap in the bitmap arena
    uint64_t start_key;   // packed board (puzzle)
    uint64_t tab_off;     // first slot of the dedup partition
    uint32_t log2_slots;
    uint32_t fresh;       // serving: state not yet initialised
    uint64_t max_rounds;
    uint64_t heap_off;    // serving: byte offset of this request's heap slice
    uint32_t heap_stride; // serving: entries per heap of that slice
    uint32_t heap_hcap;   // serving: maximum heap size
    uint64_t budget;      // batch: rounds before the instance gives up its team (0: the launch's)
    uint64_t key_off;     // batch: first path key of this instance in the key buffer
    uint64_t key_cap;     // batch: room for path keys
    uint64_t grow_at;     // serving: pause the search when it has claimed this many slots (0: never)
};

struct InstOut {
    uint32_t status, goal_slot;
    unsigned long long goal_best, rounds, expanded, generated, pushed, inserted;
    unsigned long long t_start, t_end;  // device globaltimer around this call's work (ns)
    unsigned long long path_len;        // batch: keys written (goal -> start); key_cap + 1 if cut
};

struct BatchArgs {
    const InstDesc *descs;
    uint32_t count;
    uint32_t *queue;
    const uint32_t *bitmaps;
    const uint8_t *pdb3;
    const uint8_t *pdb4;
    Slot *tab;
    uint8_t *heaps;        // per CTA: H heaps x slice bytes
    uint64_t slice;        // bytes per heap (batch)
    uint32_t *hsize;       // per CTA: H
    Cand *cand;            // per CTA: 2 * (8 H + 1) records (cand_records with 8 moves)
    uint32_t H;            // heaps per instance (CTA)
    uint32_t L_grid, L_puzzle;            // heap levels in shared memory
    uint32_t stride_grid, stride_puzzle;  // batch heap geometry per entry type
    uint32_t hcap_grid, hcap_puzzle;
    uint32_t split_grid, split_puzzle;    // SearchMem::split per entry type
    InstOut *outs;
    TeamState *states;     // serving: per slot persisted team state
    TeamState *cstates;    // cluster teams: per cluster team state
    uint32_t *cnext;       // cluster teams: instance index broadcast per cluster
    double max_load;
    uint64_t budget;       // rounds per call (serving quantum) or ~0
    int serving;           // 1: CTA b serves slot b; 0: work queue
    uint64_t region_slots; // batch: dedup region of each team (reused by the instances it takes)
    uint64_t quantum_ns;   // serving: time slice of the launch, from each team's start (0: rounds only)
    uint64_t walk_inline;  // serving: paths of more cells are walked after the quantum (0: all inline)
    unsigned long long *keys;  // batch: path keys of solved instances
};

// Cells (states) on the path of a solved instance, from its goal cost: a
// grid's straight + diagonal steps, a puzzle's moves, plus the start.
__host__ __device__ inline uint64_t path_cells(uint32_t kind, unsigned long long goal_best) {
    return kind == UASTAR_KIND_GRID ? (goal_best >> 32) + (goal_best & 0xffffffffull) + 1 : goal_best + 1;
}
constexpr unsigned long long kWalkDeferred = ~0ull;  // InstOut::path_len: walk after the quantum

// Writes the keys of the prev chain from `goal_slot` (goal -> start) and
// returns their number, or cap + 1 if the chain is longer than cap.  One
// thread: a pointer chase.
__device__ unsigned long long walk_chain(const Slot *part, uint32_t goal_slot, unsigned long long *out,
                                         uint64_t cap, int link) {
    uint32_t s = goal_slot;
    uint64_t n = 0;
    while (s != kNone && n < cap) {
        uint64_t key;
        uint32_t prev;
        slot_key_prev(part + s, link, key, prev);
        out[n++] = key;
        s = prev;
    }
    return s != kNone ? cap + 1 : n;
}

__device__ void clear_partition(Slot *tab, uint64_t slots) {
    uint4 *p = reinterpret_cast<uint4 *>(tab);
    const uint4 v = make_uint4(~0u, ~0u, ~0u, ~0u);
    for (uint64_t j = threadIdx.x; j < slots * 2; j += blockDim.x) p[j] = v;
}

__device__ void init_state(TeamState *st) { team_state_init(st); }

// Runs one instance on this CTA for up to `budget` rounds.
template <class Team>
__device__ uint32_t run_instance(const BatchArgs &a, const InstDesc &d, Team &team, Slot *tab, uint8_t *heaps,
                                 uint32_t *hs, Cand *cand, unsigned char *smem, uint64_t budget,
                                 uint64_t deadline_ns) {
    const uint64_t slots = 1ull << d.log2_slots;
    const bool own_geo = a.serving != 0;  // serving requests carry their heap geometry
    if (d.kind == UASTAR_KIND_GRID) {
        GridProblem prob;
        prob.bm = a.bitmaps + d.bm_word;
        prob.H = d.H;
        prob.W = d.W;
        prob.sx = d.sx;
        prob.sy = d.sy;
        prob.ex = d.ex;
        prob.ey = d.ey;
        SearchMem<GridEntry> m{tab, slots - 1, (uint64_t)(slots * a.max_load), 4096u,
                               reinterpret_cast<GridEntry *>(heaps),
                               own_geo ? d.heap_stride : a.stride_grid, own_geo ? d.heap_hcap : a.hcap_grid,
                               a.L_grid, hs, cand, d.max_rounds};
        if (d.grow_at) m.grow_at = d.grow_at;
        m.deadline_ns = deadline_ns;
        m.split = a.split_grid;
        return ga_search(prob, team, m, a.H, smem, budget);
    }
    SearchMem<PuzzleEntry> m{tab, slots - 1, (uint64_t)(slots * a.max_load), 4096u,
                             reinterpret_cast<PuzzleEntry *>(heaps),
                             own_geo ? d.heap_stride : a.stride_puzzle, own_geo ? d.heap_hcap : a.hcap_puzzle,
                             a.L_puzzle, hs, cand, d.max_rounds};
    if (d.grow_at) m.grow_at = d.grow_at;
    m.deadline_ns = deadline_ns;
    m.split = a.split_puzzle;
    if (d.n == 4) {
        PuzzleProblem<4> prob;
        prob.pdb = a.pdb4;
        prob.start = d.start_key;
        prob.goal = PuzzleProblem<4>::goal_key();
        return ga_search(prob, team, m, a.H, smem, budget);
    }
    PuzzleProblem<3> prob;
    prob.pdb = a.pdb3;
    prob.start = d.start_key;
    prob.goal = PuzzleProblem<3>::goal_key();
    return ga_search(prob, team, m, a.H, smem, budget);
}

__global__ void __launch_bounds__(512, 1) k_batch(BatchArgs a) {
    __shared__ TeamState st;
    __shared__ uint32_t s_next;
    extern __shared__ __align__(128) unsigned char smem[];
    const uint32_t H = a.H;
    // batch: each CTA owns a heap slice reused by the instances it takes;
    // serving: each request owns a slice named by its descriptor
    uint8_t *heaps = a.heaps + (size_t)blockIdx.x * H * a.slice;
    uint32_t *hs = a.hsize + (size_t)blockIdx.x * H;
    Cand *cand = a.cand + (size_t)blockIdx.x * 2 * (8 * H + 1);
    for (uint32_t iter = 0;; ++iter) {
        if (a.serving) {
            if (iter > 0 || blockIdx.x >= a.count) break;
            if (threadIdx.x == 0) s_next = blockIdx.x;
        } else if (threadIdx.x == 0) {
            s_next = atomicAdd(a.queue, 1u);
        }
        __syncthreads();
        const uint32_t i = s_next;
        if (i >= a.count) break;
        const InstDesc d = a.descs[i];
        if (a.serving && d.kind == 0) break;  // empty serving slot
        const unsigned long long t_start = globaltimer_ns();
        if (a.serving) heaps = a.heaps + d.heap_off;
        // serving: the request's own partition; batch: this CTA's region
        Slot *const tab = a.serving ? a.tab + d.tab_off : a.tab + (size_t)blockIdx.x * a.region_slots;
        if (!a.serving || d.fresh) {
            // serving partitions are cleared by the host at admission (fresh == 2)
            if (d.fresh != 2) clear_partition(tab, 1ull << d.log2_slots);
            for (uint32_t j = threadIdx.x; j < H; j += blockDim.x) hs[j] = 0;
            if (threadIdx.x == 0) init_state(&st);
        } else if (threadIdx.x == 0) {
            st = a.states[i];
        }
        __syncthreads();
        BlockTeam team{&st};
        run_instance(a, d, team, tab, heaps, hs, cand, smem, d.budget ? d.budget : a.budget,
                     a.quantum_ns ? t_start + a.quantum_ns : 0);
        __syncthreads();
        if (threadIdx.x == 0) {
            InstOut o;
            o.path_len = 0;
            o.status = st.status;
            o.goal_slot = st.goal_slot;
            o.goal_best = st.goal_best;
            o.rounds = st.round;
            o.expanded = st.expanded;
            o.generated = st.generated;
            o.pushed = st.pushed;
            o.inserted = st.inserted;
            o.t_start = t_start;
            o.t_end = globaltimer_ns();
            // a phase-2 error of the last round of a quantum is still in error2
            // an error of a parked search is reported by its next decision: report it now
            if (o.status == ST_RUNNING && st.error) o.status = st.error;
            // the path is read out now (a batch region is reused by the
            // team's next instance); a serving request's long path is walked
            // after the quantum instead, so that one thread's pointer chase
            // does not hold the whole launch
            if (o.status == ST_OK) {
                if (a.walk_inline && path_cells(d.kind, o.goal_best) > a.walk_inline)
                    o.path_len = kWalkDeferred;
                else
                    o.path_len = walk_chain(tab, o.goal_slot, a.keys + d.key_off, d.key_cap,
                                            d.kind == UASTAR_KIND_GRID ? GridProblem::kLink : PuzzleProblem<4>::kLink);
            }
            a.outs[i] = o;
            if (a.serving) a.states[i] = st;
        }
        __syncthreads();
    }
}

// A deferred serving walk: one request's chain into out[0 .. cap), its
// length into out[cap].
__global__ void k_serve_walk(const Slot *part, uint32_t goal_slot, unsigned long long *out, uint64_t cap, int link) {
    if (blockIdx.x == 0 && threadIdx.x == 0) out[cap] = walk_chain(part, goal_slot, out, cap, link);
}

__device__ void clear_partition_team(Slot *tab, uint64_t slots, uint32_t rank, uint32_t nranks) {
    uint4 *p = reinterpret_cast<uint4 *>(tab);
    const uint4 v = make_uint4(~0u, ~0u, ~0u, ~0u);
    for (uint64_t j = (uint64_t)rank * blockDim.x + threadIdx.x; j < slots * 2; j += (uint64_t)nranks * blockDim.x)
        p[j] = v;
}

// Batch of large instances: one thread-block cluster per instance.  The
// cluster's CTAs are one GA* team (H heaps each); instances come from the
// device work queue, one per cluster at a time.
__global__ void __launch_bounds__(512, 1) k_batch_cluster(BatchArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const uint32_t crank = ClusterTeam{nullptr}.cta(), csize = ClusterTeam{nullptr}.ctas();
    const uint32_t cid = blockIdx.x / csize;
    const uint32_t H = a.H;
    TeamState *st = a.cstates + cid;
    ClusterTeam team{st};
    uint8_t *heaps = a.heaps + (size_t)cid * csize * H * a.slice;
    uint32_t *hs = a.hsize + (size_t)cid * csize * H;
    Cand *cand = a.cand + (size_t)cid * csize * 2 * (8 * H + 1);
    for (uint32_t iter = 0;; ++iter) {
        uint32_t i;
        if (a.serving) {
            // serving: cluster c advances large-request slot c by one quantum
            if (iter > 0) break;
            i = cid;
        } else {
            if (crank == 0 && threadIdx.x == 0) a.cnext[cid] = atomicAdd(a.queue, 1u);
            team.sync();
            i = ldcg_u32(&a.cnext[cid]);
        }
        if (i >= a.count) break;
        const InstDesc d = a.descs[i];
        if (a.serving && d.kind == 0) break;  // empty slot
        if (a.serving) heaps = a.heaps + d.heap_off;
        const unsigned long long t_start = globaltimer_ns();
        Slot *const tab = a.serving ? a.tab + d.tab_off : a.tab + (size_t)cid * a.region_slots;
        if (!a.serving || d.fresh) {
            // serving partitions are cleared by the host at admission (fresh == 2)
            if (d.fresh != 2) clear_partition_team(tab, 1ull << d.log2_slots, crank, csize);
            for (uint32_t j = threadIdx.x; j < H; j += blockDim.x) hs[crank * H + j] = 0;
            if (crank == 0 && threadIdx.x == 0) init_state(st);
        }
        team.sync();
        run_instance(a, d, team, tab, heaps, hs, cand, smem, d.budget ? d.budget : a.budget,
                     a.quantum_ns ? t_start + a.quantum_ns : 0);
        team.sync();
        if (crank == 0 && threadIdx.x == 0) {
            InstOut o;
            o.path_len = 0;
            o.status = ldcg_u32(&st->status);
            o.goal_slot = ldcg_u32(&st->goal_slot);
            o.goal_best = ldcg_u64(&st->goal_best);
            o.rounds = ldcg_u64(&st->round);
            o.expanded = ldcg_u64(&st->expanded);
            o.generated = ldcg_u64(&st->generated);
            o.pushed = ldcg_u64(&st->pushed);
            o.inserted = ldcg_u64(&st->inserted);
            o.t_start = t_start;
            o.t_end = globaltimer_ns();
            const uint32_t pend = ldcg_u32(&st->error);
            if (o.status == ST_RUNNING && pend) o.status = pend;
            if (o.status == ST_OK) {
                if (a.walk_inline && path_cells(d.kind, o.goal_best) > a.walk_inline)
                    o.path_len = kWalkDeferred;  // walked after the quantum (the CTA kernel's note)
                else
                    o.path_len = walk_chain(tab, o.goal_slot, a.keys + d.key_off, d.key_cap,
                                            d.kind == UASTAR_KIND_GRID ? GridProblem::kLink : PuzzleProblem<4>::kLink);
            }
            a.outs[i] = o;
        }
        team.sync();
    }
}

// One thread per finished instance walks its prev chain (goal -> start).
__global__ void k_batch_walk(const InstDesc *descs, const InstOut *outs, const uint32_t *which,
                             uint32_t nwhich, const Slot *tab, unsigned long long *keys,
                             const uint64_t *key_off, const uint64_t *key_cap, unsigned long long *lens) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nwhich) return;
    const uint32_t i = which[t];
    lens[t] = walk_chain(tab + descs[i].tab_off, outs[i].goal_slot, keys + key_off[t], key_cap[t],
                         descs[i].kind == UASTAR_KIND_GRID ? GridProblem::kLink : PuzzleProblem<4>::kLink);
}

// Move a parked single-CTA search's heaps (hs heaps) onto a cluster slot's
// hd = 8 hs heaps: destination heap j takes every (hd / hs)-th entry of source
// heap j % hs and pushes it into its (empty) heap, one thread per destination
// heap, with the heap's saved top in global memory and its brick scratch in
// shared memory.  The dedup partition and the team state carry over as they
// are, so the search resumes where it stopped.  Sets *err on overflow.
template <class P>
__global__ void __launch_bounds__(128) k_migrate_heaps(const typename P::Entry *src, uint32_t src_stride,
                                                       const uint32_t *src_size, uint32_t hs,
                                                       typename P::Entry *dst, uint32_t dst_stride,
                                                       uint32_t *dst_size, uint32_t hd, uint32_t L, uint32_t hcap,
                                                       uint32_t *err) {
    using E = typename P::Entry;
    __shared__ __align__(16) E scr[128 * 2 * BrickHeap<P>::BE];
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= hd) return;
    const uint32_t topn = (1u << L) - 1u, sh = j % hs, ratio = hd / hs;
    const E *sblock = src + (size_t)sh * src_stride;
    const BrickHeap<P> from{const_cast<E *>(sblock) + top_reserve<P>(L), nullptr, nullptr, L};
    E *dblock = dst + (size_t)j * dst_stride;
    const BrickHeap<P> to{dblock + top_reserve<P>(L), dblock, scr + (size_t)threadIdx.x * 2 * BrickHeap<P>::BE, L};
    const uint32_t n_src = src_size[sh];
    uint32_t n = 0;
    for (uint32_t i = 1 + j / hs; i <= n_src; i += ratio) {
        const E e = i <= topn ? P::load(sblock + i) : P::load(from.g + from.off(i));
        if (n + 1 > hcap) {
            atomicExch(err, 1u);
            break;
        }
        heap_push<P>(to, n, e);
    }
    dst_size[j] = n;
}

}  // namespace uastar

namespace {

// UASTAR_DEBUG=1 in the environment prints the batch engine's wave plan and
// timings to stderr.
bool debug_log() {
    static const bool on = [] {
        const char *v = std::getenv("UASTAR_DEBUG");
        return v && *v && *v != '0';
    }();
    return on;
}

inline double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}
inline uint64_t next_pow2_u64(uint64_t v) {
    uint64_t p = 1;
    while (p < v) p <<= 1;
    return p;
}
inline int log2_u64(uint64_t v) {
    int l = 0;
    while ((1ull << l) < v) ++l;
    return l;
}

// Estimated dedup nodes of an instance (a sizing hint; overflow is retried).
uint64_t est_nodes(const uastar_instance &in) {
    if (in.est_nodes > 0) return (uint64_t)in.est_nodes;
    // Grids: an eighth of the cells (random grids searched corner to corner
    // touch a few percent to ~20 %).  15-puzzles: 2^19 states, what a single
    // CTA team inserts in a 4096-round budget (64 heaps, ~2 new states per
    // expansion), so that a puzzle leaves that tier by running out of rounds
    // rather than out of space.  An instance that fills its partition is
    // re-run in the next wave with 16x the space.
    if (in.kind == UASTAR_KIND_GRID) return std::max<uint64_t>(4096, (uint64_t)in.H * in.W / 8);
    return in.n == 3 ? 65536 : 524288;
}

struct BatchPlan {
    std::vector<InstDesc> descs;
    std::vector<uint64_t> bm_words;  // packed bitmaps of all grid instances (32-bit words)
    uint64_t total_slots = 0;
};

int32_t check_instance(const uastar_instance &in) {
    if (in.kind == UASTAR_KIND_GRID) {
        if (!in.words || in.H <= 0 || in.W <= 0 || (uint64_t)in.H * in.W >= (1ull << 31)) return UASTAR_BAD_INPUT;
        if (in.sx < 0 || in.sx >= in.H || in.sy < 0 || in.sy >= in.W || in.ex < 0 || in.ex >= in.H ||
            in.ey < 0 || in.ey >= in.W)
            return UASTAR_BAD_INPUT;
        return UASTAR_OK;
    }
    if (in.kind == UASTAR_KIND_PUZZLE && (in.n == 3 || in.n == 4)) {
        int seen = 0;
        for (int i = 0; i < in.n * in.n; ++i) {
            if (in.tiles[i] >= in.n * in.n || (seen >> in.tiles[i] & 1)) return UASTAR_BAD_INPUT;
            seen |= 1 << in.tiles[i];
        }
        return UASTAR_OK;
    }
    return UASTAR_BAD_INPUT;
}

struct BatchGeometry {
    int T, ctas;
    int csize = 0;      // > 0: cluster teams of csize CTAs (ctas = clusters * csize)
    uint32_t H, L_grid, L_puzzle;
    uint64_t want;  // requested heap capacity (entries)
    HeapGeometry<GridProblem> hg_grid;
    HeapGeometry<PuzzleProblem<4>> hg_puzzle;
    uint64_t slice;  // bytes per heap
    size_t smem;
    // Split rounds (SearchMem::split) where their push staging fits the
    // shared memory the CTA already has: the puzzles' tops are the smaller,
    // so puzzles get them at every launch shape here, grids not.
    uint32_t split_grid = 0, split_puzzle = 0;
    double load;
    void set_capacity(uint64_t w) {
        want = w;
        hg_grid = heap_geometry<GridProblem>(L_grid, w);
        hg_puzzle = heap_geometry<PuzzleProblem<4>>(L_puzzle, w);
        slice = std::max<uint64_t>((uint64_t)hg_grid.stride * sizeof(GridEntry),
                                   (uint64_t)hg_puzzle.stride * sizeof(PuzzleEntry));
        slice = (slice + 127) & ~127ull;
    }
};

// Largest L (>= 1) whose shared heap tops fit `budget`.
template <class P> uint32_t fit_top(uint32_t H, size_t budget) {
    uint32_t best = 1;
    for (uint32_t L = 1; L <= 10; ++L) {
        if (SearchSmem<P>::bytes(H, L) > budget) break;
        best = L;
    }
    return best;
}

// CTA size, heaps per CTA, shared heap tops sized for two CTAs per SM.
int32_t resolve_block_geometry(uastar_engine *eng, int threads, int tph, BatchGeometry *g) {
    g->T = threads > 0 ? threads : 256;
    g->T = std::max(32, std::min(512, (g->T + 31) / 32 * 32));
    tph = std::max(1, std::min(tph > 0 ? tph : 4, g->T));
    g->H = (uint32_t)std::max(1, g->T / tph);
    int smem_sm = 0;
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, eng->device);
    const size_t per_cta = (size_t)std::max(16 * 1024, smem_sm / 2 - 4 * 1024);
    g->L_grid = fit_top<GridProblem>(g->H, per_cta);
    g->L_puzzle = fit_top<PuzzleProblem<4>>(g->H, per_cta);
    g->smem = std::max(SearchSmem<GridProblem>::bytes(g->H, g->L_grid),
                       SearchSmem<PuzzleProblem<4>>::bytes(g->H, g->L_puzzle));
    g->split_grid = SearchSmem<GridProblem>::bytes_split(g->H, g->L_grid) <= g->smem ? 1u : 0u;
    g->split_puzzle = SearchSmem<PuzzleProblem<4>>::bytes_split(g->H, g->L_puzzle) <= g->smem ? 1u : 0u;
    g->set_capacity(4095);
    cudaError_t e = cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g->smem);
    if (e != cudaSuccess) return fail_cuda(eng, e, "smem attribute");
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batch, g->T, g->smem);
    if (e != cudaSuccess) return fail_cuda(eng, e, "occupancy");
    g->ctas = eng->sms * std::max(1, occ);
    return UASTAR_OK;
}

// Cluster teams: the same CTA geometry, `csize` CTAs per team, as many
// teams as can be co-resident.
int32_t resolve_cluster_geometry(uastar_engine *eng, int csize, BatchGeometry *g) {
    cudaError_t e = cudaFuncSetAttribute(k_batch_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g->smem);
    if (e == cudaSuccess && csize > 8)
        e = cudaFuncSetAttribute(k_batch_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return fail_cuda(eng, e, "cluster attributes");
    cudaLaunchConfig_t lc = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)csize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    lc.gridDim = dim3((unsigned)csize);
    lc.blockDim = dim3((unsigned)g->T);
    lc.dynamicSmemBytes = g->smem;
    lc.attrs = at;
    lc.numAttrs = 1;
    int nclusters = 0;
    e = cudaOccupancyMaxActiveClusters(&nclusters, k_batch_cluster, &lc);
    if (e != cudaSuccess || nclusters < 1) {
        eng->set_err("no cluster of the requested size fits this GPU");
        return UASTAR_BAD_INPUT;
    }
    g->csize = csize;
    g->ctas = nclusters * csize;
    return UASTAR_OK;
}

int32_t resolve_geometry(uastar_engine *eng, const uastar_batch_config *cfg, BatchGeometry *g) {
    int32_t rc = resolve_block_geometry(eng, cfg ? cfg->threads_per_instance : 0, cfg ? cfg->threads_per_heap : 0, g);
    if (rc) return rc;
    g->set_capacity(cfg && cfg->heap_capacity > 0 ? (uint64_t)cfg->heap_capacity : 4095);
    g->load = cfg && cfg->load_factor > 0 && cfg->load_factor < 1 ? cfg->load_factor : 0.5;
    if (cfg && cfg->ctas > 0) g->ctas = std::min(g->ctas, cfg->ctas);
    return UASTAR_OK;
}

// Runs `idx` (indices into insts) as one wave; fills results for them.
// Each team (CTA or cluster) owns one dedup region, sized for the largest
// partition of the wave and reused by every instance the team takes, so the
// wave's table memory is teams x region, not the sum over instances.
// `puzzle_budget` (0: none) is a round budget for puzzle instances only.
int32_t run_wave(uastar_engine *eng, const uastar_instance *insts, const std::vector<int> &idx,
                 const BatchGeometry &g, const std::vector<int> &space_mult, bool use_graph, uint64_t budget,
                 uint64_t puzzle_budget, uastar_instance_result *results, uastar_batch_stats *stats,
                 std::vector<int> *retry) {
    cudaError_t e;
    const int cnt = (int)idx.size();
    // plan: order largest estimate first (longest-processing-time first)
    std::vector<int> order(cnt);
    std::iota(order.begin(), order.end(), 0);
    std::vector<uint64_t> est(cnt);
    for (int j = 0; j < cnt; ++j) est[j] = est_nodes(insts[idx[j]]) * (uint64_t)space_mult[j];
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return est[a] > est[b]; });

    std::vector<InstDesc> descs(cnt);
    std::vector<int> slot_of(cnt);  // position of wave instance j in descs
    uint64_t bm_words = 0, region_slots = 1u << 12, ktot = 0;
    for (int p = 0; p < cnt; ++p) {
        const int j = order[p];
        const uastar_instance &in = insts[idx[j]];
        InstDesc d;
        std::memset(&d, 0, sizeof d);
        d.kind = in.kind;
        d.n = in.n;
        d.max_rounds = eng->cfg.max_rounds;
        uint64_t slots = next_pow2_u64((uint64_t)((double)est[j] / g.load));
        slots = std::max<uint64_t>(slots, 1u << 12);
        d.log2_slots = (uint32_t)log2_u64(slots);
        region_slots = std::max(region_slots, slots);
        // path keys: a longer path (a maze) goes to the plain engine
        d.key_off = ktot;
        d.key_cap = in.kind == UASTAR_KIND_GRID ? 2ull * ((uint64_t)in.H + in.W) + 64 : 256;
        ktot += d.key_cap;
        d.budget = in.kind == UASTAR_KIND_PUZZLE ? puzzle_budget : 0;
        if (in.kind == UASTAR_KIND_GRID) {
            d.H = in.H;
            d.W = in.W;
            d.sx = in.sx;
            d.sy = in.sy;
            d.ex = in.ex;
            d.ey = in.ey;
            d.bm_word = bm_words * 2;
            bm_words += ((uint64_t)in.H * in.W + 63) / 64 + 2;
        } else {
            d.start_key = pack_board(in.n, in.tiles);
        }
        descs[p] = d;
        slot_of[j] = p;
    }
    // device buffers
    const int teams = g.csize > 0 ? std::min(g.ctas / g.csize, cnt) : std::min(g.ctas, cnt);
    const size_t tab_b = (size_t)teams * region_slots * sizeof(Slot);
    const size_t heap_b = (size_t)g.ctas * g.H * g.slice;
    if (debug_log())
        std::fprintf(stderr, "[uastar] wave: %d instances, %d %s teams of %d CTAs x %d threads, %d heaps each, "
                             "budget %llu rounds (puzzles %llu), regions %.2f GB (2^%d slots each), heap slices "
                             "%.2f GB (%llu B/heap)\n",
                     cnt, teams, g.csize > 0 ? "cluster" : "CTA", g.csize > 0 ? g.csize : 1, g.T, (int)g.H,
                     (unsigned long long)budget, (unsigned long long)puzzle_budget, tab_b / 1e9,
                     (int)log2_u64(region_slots), heap_b / 1e9, (unsigned long long)g.slice);
    if ((e = eng->b_tab.ensure(tab_b)) != cudaSuccess) return fail_cuda(eng, e, "alloc partitions");
    if ((e = eng->b_heaps.ensure(heap_b)) != cudaSuccess) return fail_cuda(eng, e, "alloc heap slices");
    if ((e = eng->b_hsize.ensure((size_t)g.ctas * g.H * 4)) != cudaSuccess) return fail_cuda(eng, e, "alloc");
    if ((e = eng->b_cand.ensure((size_t)g.ctas * 2 * (8 * g.H + 1) * sizeof(Cand))) != cudaSuccess)
        return fail_cuda(eng, e, "alloc");
    if ((e = eng->b_desc.ensure(cnt * sizeof(InstDesc))) != cudaSuccess) return fail_cuda(eng, e, "alloc");
    if ((e = eng->b_out.ensure(cnt * sizeof(InstOut))) != cudaSuccess) return fail_cuda(eng, e, "alloc");
    if ((e = eng->b_queue.ensure(64)) != cudaSuccess) return fail_cuda(eng, e, "alloc");
    if ((e = eng->b_bitmaps.ensure(std::max<size_t>(16, bm_words * 8))) != cudaSuccess)
        return fail_cuda(eng, e, "alloc bitmaps");
    if ((e = eng->b_walk.ensure(std::max<size_t>(64, ktot * 8))) != cudaSuccess) return fail_cuda(eng, e, "alloc keys");
    // bitmaps H2D (one copy per grid)
    for (int p = 0; p < cnt; ++p) {
        const int j = order[p];
        const uastar_instance &in = insts[idx[j]];
        if (in.kind != UASTAR_KIND_GRID) continue;
        const size_t nb = (((uint64_t)in.H * in.W + 63) / 64) * 8;
        e = cudaMemcpyAsync(eng->b_bitmaps.as<uint32_t>() + descs[p].bm_word, in.words, nb,
                            cudaMemcpyHostToDevice, eng->stream);
        if (e != cudaSuccess) return fail_cuda(eng, e, "bitmap upload");
    }
    if ((e = cudaMemcpyAsync(eng->b_desc.p, descs.data(), cnt * sizeof(InstDesc), cudaMemcpyHostToDevice,
                             eng->stream)) != cudaSuccess)
        return fail_cuda(eng, e, "desc upload");

    BatchArgs a;
    std::memset(&a, 0, sizeof a);
    a.descs = eng->b_desc.as<InstDesc>();
    a.count = (uint32_t)cnt;
    a.queue = eng->b_queue.as<uint32_t>();
    a.bitmaps = eng->b_bitmaps.as<uint32_t>();
    a.pdb3 = eng->pdb[3].as<uint8_t>();
    a.pdb4 = eng->pdb[4].as<uint8_t>();
    a.tab = eng->b_tab.as<Slot>();
    a.heaps = eng->b_heaps.as<uint8_t>();
    a.slice = g.slice;
    a.hsize = eng->b_hsize.as<uint32_t>();
    a.cand = eng->b_cand.as<Cand>();
    a.outs = eng->b_out.as<InstOut>();
    a.max_load = 0.75;
    a.budget = ~0ull;
    a.serving = 0;
    a.H = g.H;
    a.L_grid = g.L_grid;
    a.L_puzzle = g.L_puzzle;
    a.stride_grid = g.hg_grid.stride;
    a.stride_puzzle = g.hg_puzzle.stride;
    a.hcap_grid = g.hg_grid.hcap;
    a.hcap_puzzle = g.hg_puzzle.hcap;
    a.split_grid = g.split_grid;
    a.split_puzzle = g.split_puzzle;
    a.budget = budget;
    a.region_slots = region_slots;
    a.keys = eng->b_walk.as<unsigned long long>();
    int ctas = std::min(g.ctas, cnt);
    cudaLaunchConfig_t lc = {};
    cudaLaunchAttribute lat[1];
    if (g.csize > 0) {
        const int nclusters = std::min(g.ctas / g.csize, cnt);
        ctas = nclusters * g.csize;
        if ((e = eng->b_cstate.ensure((size_t)nclusters * sizeof(TeamState))) != cudaSuccess ||
            (e = eng->b_cnext.ensure((size_t)nclusters * 4 + 64)) != cudaSuccess)
            return fail_cuda(eng, e, "alloc cluster state");
        a.cstates = eng->b_cstate.as<TeamState>();
        a.cnext = eng->b_cnext.as<uint32_t>();
        lat[0].id = cudaLaunchAttributeClusterDimension;
        lat[0].val.clusterDim.x = (unsigned)g.csize;
        lat[0].val.clusterDim.y = 1;
        lat[0].val.clusterDim.z = 1;
        lc.gridDim = dim3((unsigned)ctas);
        lc.blockDim = dim3((unsigned)g.T);
        lc.dynamicSmemBytes = g.smem;
        lc.stream = eng->stream;
        lc.attrs = lat;
        lc.numAttrs = 1;
    }

    cudaEvent_t k0, k1;
    cudaEventCreate(&k0);
    cudaEventCreate(&k1);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    auto enqueue = [&]() {
        cudaMemsetAsync(eng->b_queue.p, 0, 4, eng->stream);
        if (g.csize > 0)
            cudaLaunchKernelEx(&lc, k_batch_cluster, a);
        else
            k_batch<<<ctas, g.T, g.smem, eng->stream>>>(a);
    };
    cudaEventRecord(k0, eng->stream);
    if (use_graph) {
        // The launch is captured every call (its arguments change) and the
        // executable graph of this launch shape, instantiated once, is
        // updated in place; a shape seen for the first time, or an update
        // the driver refuses, instantiates a new one.
        e = cudaStreamBeginCapture(eng->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            enqueue();
            e = cudaStreamEndCapture(eng->stream, &graph);
        }
        const auto key = std::make_tuple(g.csize, ctas, g.T, g.smem);
        auto it = eng->b_graphs.find(key);
        if (e == cudaSuccess && it != eng->b_graphs.end()) {
            cudaGraphExecUpdateResultInfo info;
            if (cudaGraphExecUpdate(it->second, graph, &info) == cudaSuccess) {
                exec = it->second;
            } else {
                cudaGetLastError();  // the refused update is not an error of the launch
                cudaGraphExecDestroy(it->second);
                eng->b_graphs.erase(it);
            }
        }
        if (e == cudaSuccess && !exec) {
            e = cudaGraphInstantiate(&exec, graph, 0);
            if (e == cudaSuccess) eng->b_graphs[key] = exec;
        }
        if (e == cudaSuccess) e = cudaGraphLaunch(exec, eng->stream);
    } else {
        enqueue();
        e = cudaGetLastError();
    }
    eng->launches++;
    cudaEventRecord(k1, eng->stream);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail_cuda(eng, e, "batch launch");
    std::vector<InstOut> outs(cnt);
    e = cudaMemcpyAsync(outs.data(), eng->b_out.p, cnt * sizeof(InstOut), cudaMemcpyDeviceToHost, eng->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(eng->stream);
    if (e != cudaSuccess) return fail_cuda(eng, e, "batch kernel");
    float kms = 0;
    cudaEventElapsedTime(&kms, k0, k1);
    cudaEventDestroy(k0);
    cudaEventDestroy(k1);
    if (stats) stats->kernel_ms += kms;
    if (debug_log()) {
        int hist[16] = {0};
        for (int p = 0; p < cnt; ++p) hist[std::min<uint32_t>(outs[p].status, 15)]++;
        std::fprintf(stderr, "[uastar]   kernel %.1f ms; status counts:", kms);
        for (int q = 0; q < 16; ++q)
            if (hist[q]) std::fprintf(stderr, " %d:%d", q, hist[q]);
        std::fprintf(stderr, "\n");
    }

    // paths of solved instances, walked by their teams (goal -> start)
    std::vector<unsigned long long> keys(ktot);
    if (ktot && (e = cudaMemcpyAsync(keys.data(), eng->b_walk.p, ktot * 8, cudaMemcpyDeviceToHost, eng->stream)) !=
                    cudaSuccess)
        return fail_cuda(eng, e, "path keys");
    if ((e = cudaStreamSynchronize(eng->stream)) != cudaSuccess) return fail_cuda(eng, e, "path keys");
    unsigned long long t_first = ~0ull;
    for (int p = 0; p < cnt; ++p) t_first = std::min(t_first, outs[p].t_start);

    for (int j = 0; j < cnt; ++j) {
        const int p = slot_of[j];
        const InstOut &o = outs[p];
        const uastar_instance &in = insts[idx[j]];
        uastar_instance_result &r = results[idx[j]];
        r.attempts += 1;
        r.device_ms = (double)(o.t_end - o.t_start) * 1e-6;
        r.start_ms = (double)(o.t_start - t_first) * 1e-6;
        r.status = (int32_t)o.status;
        r.expanded += (int64_t)o.expanded;
        r.generated += (int64_t)o.generated;
        r.rounds += (int64_t)o.rounds;
        if (stats) {
            stats->expanded += (int64_t)o.expanded;
            stats->generated += (int64_t)o.generated;
        }
        const bool long_path = o.status == ST_OK && o.path_len > descs[p].key_cap;
        if ((o.status == ST_HASH_FULL || o.status == ST_HEAP_OVERFLOW || o.status == ST_RUNNING || long_path) &&
            retry) {
            retry->push_back(idx[j]);
            continue;
        }
        if (o.status != ST_OK) continue;
        const uint64_t len = o.path_len;
        if (long_path) {
            r.status = UASTAR_ARENA_FULL;
            continue;
        }
        // keys are goal -> start
        const unsigned long long *kk = keys.data() + descs[p].key_off;
        if (in.kind == UASTAR_KIND_GRID) {
            r.straight = (int64_t)(o.goal_best >> 32);
            r.diagonal = (int64_t)(o.goal_best & 0xffffffffu);
            std::vector<int32_t> path(len);
            for (uint64_t t = 0; t < len; ++t) path[t] = (int32_t)kk[len - 1 - t];
            int64_t a2 = 0, b2 = 0;
            float fc = 0;
            if (uastar_validate_grid_path(in.words, in.H, in.W, in.sx, in.sy, in.ex, in.ey, path.data(),
                                          (int64_t)len, &a2, &b2, &fc) != UASTAR_OK ||
                a2 != r.straight || b2 != r.diagonal) {
                r.status = UASTAR_CUDA_ERROR;
                eng->set_err("batched engine returned a path that fails host validation");
                continue;
            }
            r.cost = fc;
        } else {
            r.steps = (int32_t)o.goal_best;
            std::vector<int32_t> moves;
            auto blank = [&](uint64_t k) {
                for (int c = 0; c < in.n * in.n; ++c)
                    if (((k >> (4 * c)) & 15) == 0) return c;
                return -1;
            };
            for (uint64_t t = len - 1; t >= 1; --t) {
                const int pb = blank(kk[t]), cb = blank(kk[t - 1]);
                moves.push_back(cb - pb == in.n ? 0 : cb - pb == -in.n ? 1 : cb - pb == 1 ? 2 : 3);
            }
            if ((int64_t)moves.size() != r.steps ||
                uastar_validate_puzzle_moves(in.n, in.tiles, moves.data(), (int64_t)moves.size()) != UASTAR_OK) {
                r.status = UASTAR_CUDA_ERROR;
                eng->set_err("batched engine returned moves that fail host validation");
                continue;
            }
        }
    }
    if (stats) {
        stats->waves += 1;
        stats->partition_bytes = std::max<int64_t>(stats->partition_bytes, (int64_t)tab_b);
    }
    return UASTAR_OK;
}

}  // namespace

namespace uastar {
void release_batch_buffers(uastar_engine *eng) {
    for (DevBuf *b : {&eng->b_tab, &eng->b_heaps, &eng->b_bitmaps, &eng->b_cand, &eng->b_hsize, &eng->b_walk})
        b->release();
}
}  // namespace uastar

extern "C" {

int32_t uastar_batch_solve(uastar_engine *eng, const uastar_instance *insts, int32_t count,
                           const uastar_batch_config *cfg, uastar_instance_result *results,
                           uastar_batch_stats *stats) {
    if (!eng || !insts || count < 0 || !results) return UASTAR_BAD_INPUT;
    cudaSetDevice(eng->device);
    const double t0 = now_ms();
    if (stats) std::memset(stats, 0, sizeof(*stats));
    std::memset(results, 0, sizeof(uastar_instance_result) * (size_t)count);
    BatchGeometry g;
    int32_t rc = resolve_geometry(eng, cfg, &g);
    if (rc) return rc;
    std::vector<int> todo;
    for (int i = 0; i < count; ++i) {
        const uastar_instance &in = insts[i];
        if (check_instance(in) != UASTAR_OK) {
            results[i].status = UASTAR_BAD_INPUT;
            continue;
        }
        if (in.kind == UASTAR_KIND_PUZZLE) {
            if (!eng->pdb_ready[in.n]) {
                results[i].status = UASTAR_BAD_INPUT;
                eng->set_err("pattern database not resident for a puzzle instance");
                continue;
            }
            if (!board_solvable(in.n, in.tiles)) {
                results[i].status = UASTAR_NO_SOLUTION;
                continue;
            }
        }
        todo.push_back(i);
    }
    // Tiers: single-CTA teams for small instances (with a round budget, so
    // that an unexpectedly large one moves on instead of holding a CTA),
    // cluster teams of 8 CTAs for large grids, for instances that ran out of
    // rounds and for those that overflowed (with 16x the space); whatever
    // overflows a cluster team or outlasts its round budget goes to the plain
    // engine (the whole GPU).
    std::vector<int> mult(count, 1);
    const bool use_graph = !cfg || cfg->use_graph != 0 || cfg->threads_per_instance == 0;
    const uint64_t big_cells = 2048ull * 2048ull;
    std::vector<int> tier1, tier2, retry;
    for (int i : todo) {
        const uastar_instance &in = insts[i];
        if (in.kind == UASTAR_KIND_GRID && (uint64_t)in.H * in.W > big_cells)
            tier2.push_back(i);
        else
            tier1.push_back(i);
    }
    if (!tier1.empty()) {
        std::vector<int> m(tier1.size(), 1);
        const uint64_t b1 = cfg && cfg->tier1_rounds > 0 ? (uint64_t)cfg->tier1_rounds : 2048;
        rc = run_wave(eng, insts, tier1, g, m, use_graph, b1, 0, results, stats, &retry);
        if (rc) return rc;
        // running out of rounds proves an instance large just as an overflow does
        for (int i : retry) {
            mult[i] = 16;
            tier2.push_back(i);
        }
    }
    todo.clear();
    if (!tier2.empty()) {
        BatchGeometry gc = g;
        bool heap_over = false;
        for (int i : tier2) heap_over |= results[i].status == UASTAR_HEAP_OVERFLOW;
        if (heap_over) gc.set_capacity(g.want * 16 + 15);
        const int csize = cfg && cfg->cluster_size >= 2 && cfg->cluster_size <= 16 ? cfg->cluster_size : 8;
        rc = resolve_cluster_geometry(eng, csize, &gc);
        if (rc) return rc;
        std::vector<int> m(tier2.size());
        for (size_t j = 0; j < tier2.size(); ++j) m[j] = mult[tier2[j]] * 2;
        retry.clear();
        // Puzzles get a round budget here too: one that needs more is better
        // off with the whole GPU than holding a cluster for the batch's tail.
        // Grids do not: their rounds are bounded by the path length, which
        // costs a cluster no more rounds than the whole GPU.
        const uint64_t b2 = cfg && cfg->tier2_puzzle_rounds > 0 ? (uint64_t)cfg->tier2_puzzle_rounds : 16384;
        rc = run_wave(eng, insts, tier2, gc, m, use_graph, ~0ull, b2, results, stats, &retry);
        if (rc) return rc;
        todo = retry;
    }
    // The team regions are kept for the next batch (teams x region, tens of
    // GB at most); only a plain-engine escalation that finds too little free
    // memory for its table gets them back.
    if (!todo.empty()) {
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        if (free_b < (32ull << 30)) {
            eng->b_tab.release();
            eng->b_bitmaps.release();
        }
    }
    for (int i : todo) {
        const uastar_instance &in = insts[i];
        uastar_instance_result &r = results[i];
        r.attempts += 1;
        const double te = now_ms();
        if (in.kind == UASTAR_KIND_GRID) {
            uastar_grid_result gr;
            rc = uastar_grid_solve(eng, in.words, in.H, in.W, in.sx, in.sy, in.ex, in.ey, &gr);
            r.status = gr.status;
            r.straight = gr.straight;
            r.diagonal = gr.diagonal;
            r.cost = gr.cost;
            r.expanded += gr.expanded;
            r.generated += gr.generated;
            r.rounds += gr.rounds;
            if (stats) {
                stats->expanded += gr.expanded;
                stats->generated += gr.generated;
            }
        } else {
            // the plain engine starts this puzzle's table at 2^26 slots: it
            // filled a cluster's partition or ran out of its round budget
            // there, and every 4x growth on the way up pauses the search
            uastar_puzzle_result pr;
            eng->puzzle_log2_start = 26;
            rc = uastar_puzzle_solve(eng, in.n, in.tiles, &pr);
            eng->puzzle_log2_start = 0;
            r.status = pr.status;
            r.steps = pr.steps;
            r.expanded += pr.expanded;
            r.generated += pr.generated;
            r.rounds += pr.rounds;
            if (stats) {
                stats->expanded += pr.expanded;
                stats->generated += pr.generated;
            }
        }
        if (stats) stats->escalated += 1;
        if (debug_log())
            std::fprintf(stderr, "[uastar] escalated instance %d (%s) to the plain engine: status %d, %.1f ms\n", i,
                         in.kind == UASTAR_KIND_GRID ? "grid" : "puzzle", r.status, now_ms() - te);
    }
    if (stats) {
        stats->wall_ms = now_ms() - t0;
        stats->ctas = g.ctas;
        stats->threads_per_instance = g.T;
        stats->heap_capacity = (int32_t)g.hg_puzzle.hcap;
        stats->load_factor = g.load;
    }
    for (int i = 0; i < count; ++i) results[i].latency_ms = now_ms() - t0;
    return UASTAR_OK;
}

int32_t uastar_autotune(uastar_engine *eng, const uastar_instance *sample, int32_t count,
                        uastar_batch_config *best) {
    if (!eng || !sample || count <= 0 || !best) return UASTAR_BAD_INPUT;
    // Coordinate descent over the batch geometry, one pass: starting from the
    // defaults, each knob in turn takes the value that solves the sample in
    // the least wall time with the others held.  Knobs: CTA size per
    // instance, threads per heap (together: heaps per instance), entries per
    // heap, dedup-partition load factor, CTAs per cluster team, the
    // single-CTA tier's round budget and the cluster tier's puzzle budget.
    struct Knob {
        int32_t uastar_batch_config::*i;
        double uastar_batch_config::*d;
        std::vector<double> values;
    };
    const std::vector<Knob> knobs = {
        {&uastar_batch_config::threads_per_instance, nullptr, {128, 256, 512}},
        {&uastar_batch_config::threads_per_heap, nullptr, {2, 4, 8}},
        {&uastar_batch_config::heap_capacity, nullptr, {1023, 4095, 16383}},
        {nullptr, &uastar_batch_config::load_factor, {0.35, 0.5, 0.7}},
        {&uastar_batch_config::cluster_size, nullptr, {4, 8, 16}},
        {&uastar_batch_config::tier1_rounds, nullptr, {1024, 2048, 4096}},
        {&uastar_batch_config::tier2_puzzle_rounds, nullptr, {4096, 16384, 65536}},
    };
    uastar_batch_config cur{};
    cur.threads_per_instance = 256;
    cur.threads_per_heap = 4;
    cur.heap_capacity = 4095;
    cur.load_factor = 0.5;
    cur.cluster_size = 8;
    cur.tier1_rounds = 2048;
    cur.tier2_puzzle_rounds = 16384;
    cur.use_graph = 1;
    std::vector<uastar_instance_result> res(count);
    auto time_of = [&](const uastar_batch_config &c) -> double {
        uastar_batch_stats s;
        if (uastar_batch_solve(eng, sample, count, &c, res.data(), &s) != UASTAR_OK) return 1e300;
        for (auto &r : res)
            if (r.status != UASTAR_OK && r.status != UASTAR_NO_SOLUTION) return 1e300;
        return s.wall_ms;
    };
    double best_ms = time_of(cur);
    int tried = 1;
    for (const Knob &k : knobs) {
        uastar_batch_config keep = cur;
        for (double v : k.values) {
            uastar_batch_config c = cur;
            if (k.i) {
                if (c.*k.i == (int32_t)v) continue;
                c.*k.i = (int32_t)v;
            } else {
                if (c.*k.d == v) continue;
                c.*k.d = v;
            }
            const double ms = time_of(c);
            ++tried;
            if (ms < best_ms) {
                best_ms = ms;
                keep = c;
            }
        }
        cur = keep;
    }
    if (best_ms >= 1e300) {
        eng->set_err("autotune: no configuration solved the sample");
        return UASTAR_CUDA_ERROR;
    }
    *best = cur;
    best->reserved = tried;
    return UASTAR_OK;
}

}  // extern "C"

// ===================================================================== serving
namespace uastar {

// First-fit allocator over [0, capacity) units, for the dedup-partition and
// bitmap arenas of the serving loop.  Host-side bookkeeping only.
class RangeAlloc {
public:
    void reset(uint64_t capacity) {
        free_.clear();
        if (capacity) free_[0] = capacity;
        cap_ = capacity;
        used_ = 0;
    }
    bool alloc(uint64_t n, uint64_t align, uint64_t *off) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            const uint64_t start = (it->first + align - 1) / align * align;
            const uint64_t end = it->first + it->second;
            if (start + n > end) continue;
            const uint64_t s0 = it->first;
            free_.erase(it);
            if (start > s0) free_[s0] = start - s0;
            if (end > start + n) free_[start + n] = end - (start + n);
            *off = start;
            used_ += n;
            return true;
        }
        return false;
    }
    void release(uint64_t off, uint64_t n) {
        used_ -= n;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    uint64_t used() const { return used_; }
    uint64_t capacity() const { return cap_; }

private:
    std::map<uint64_t, uint64_t> free_;
    uint64_t cap_ = 0, used_ = 0;
};

struct ServeReq {
    int64_t id = 0;
    uastar_instance inst{};
    std::vector<uint64_t> words;  // owned copy of the grid bitmap
    double arrival_s = 0;
    uint64_t mult = 1;            // dedup partition growth (overflow, promotion)
    uint32_t heap_mult = 1;       // heap slice growth after HEAP_OVERFLOW
    int attempts = 0;
    uastar_instance_result acc{};
};

struct ServeSlot {
    bool busy = false;
    ServeReq req;
    uint64_t tab_off = 0, tab_n = 0, bm_off = 0, bm_n = 0, heap_off = 0, heap_n = 0;
};

// A solved request whose path is being walked after its quantum: its
// partition stays allocated until the walk's keys are on the host.
struct ServeWalk {
    ServeReq req;
    InstOut o{};
    uint64_t tab_off = 0, tab_n = 0;
    uint64_t ring_off = 0, n = 0;  // n path cells at ring_off (and their count after them)
    cudaEvent_t ev = nullptr;
};

// One kind of resident slot: single CTAs (puzzles, small grids) or 8-CTA
// clusters (large grids, and requests that outgrew a CTA).  Each tier has its
// own quantum kernel and stream and is relaunched as soon as its previous
// quantum has been retired, independently of the other tier.
struct ServeTier {
    bool large = false;
    int nslots = 0;
    BatchGeometry geo{};
    std::vector<ServeSlot> slots;
    std::vector<InstDesc> descs;
    std::vector<InstOut> outs;
    DevBuf d_descs, d_outs, d_states, d_hsize, d_cand, d_keys, d_walk, d_map;
    // pinned mirrors of descs / outs for the launch's copies: with pageable
    // memory the device-to-host copy of the outs would hold the host thread
    // until the quantum ends, and the other tier could not be launched beside it
    InstDesc *h_descs = nullptr;
    InstOut *h_outs = nullptr;
    int launched_n = 0;  // slots the quantum in flight covers
    uint64_t kcap = 0;  // path keys per slot (walked in the kernel)
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr, done = nullptr;
    bool inflight = false;
    std::vector<char> launched;  // slots that are part of the quantum in flight
    // dedup ranges left by growths queued on this tier's stream: released
    // when its next quantum has finished, which the growth kernels precede
    std::vector<std::pair<uint64_t, uint64_t>> release_after;
    int resident() const {
        int n = 0;
        for (auto &sl : slots) n += sl.busy;
        return n;
    }
    int free_slot() const {
        for (int q = 0; q < nslots; ++q)
            if (!slots[q].busy) return q;
        return -1;
    }
    int extent() const {  // slots a launch must cover
        int n = 0;
        for (int q = 0; q < nslots; ++q)
            if (slots[q].busy) n = q + 1;
        return n;
    }
};

struct ServeState {
    uastar_engine *eng = nullptr;
    uastar_serve_config cfg{};
    ServeTier tier[2];  // 0 = CTA slots, 1 = cluster slots
    int capacity = 0;   // co-resident CTAs shared by both tiers' resident requests
    uint64_t heap_bytes = 0;
    std::thread th;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<ServeReq> incoming;
    std::vector<int64_t> cancels;
    std::deque<uastar_serve_completion> done;
    bool draining = false, abort_now = false;
    int64_t next_id = 0;
    int64_t outstanding = 0;  // submitted and not yet completed
    uastar_serve_stats stats{};
    int32_t loop_error = UASTAR_OK;
    // device arenas shared by both tiers
    DevBuf tab, bitmaps, heaps;
    RangeAlloc tab_alloc, bm_alloc, heap_alloc;  // units: slots, 8-byte words, 16-byte heap units
    // Deferred path walks (long paths), on their own stream after the
    // quantum that solved them: a ring of key room on the device and in
    // pinned host memory, used in the order the walks were issued.
    cudaStream_t walk_stream = nullptr;
    DevBuf walk_ring;
    unsigned long long *h_walk_ring = nullptr;
    uint64_t walk_ring_keys = 0;
    std::deque<ServeWalk> walking;
    // Pinned staging for bitmap uploads at admission (a copy from pageable
    // memory may wait for the tier's running quantum): ranges in the order
    // they were staged, each free again once its copy has run.
    unsigned char *h_stage = nullptr;
    uint64_t stage_bytes = 0;
    struct Staged {
        uint64_t off, n;
        cudaEvent_t ev;
    };
    std::deque<Staged> staged;
};

static void serve_complete(ServeState *S, ServeReq &r, int32_t status) {
    uastar_serve_completion c;
    c.id = r.id;
    c.result = r.acc;
    c.result.status = status;
    c.result.attempts = r.attempts;
    c.result.latency_ms = (uastar_now_s() - r.arrival_s) * 1e3;
    std::lock_guard<std::mutex> lk(S->mu);
    S->done.push_back(c);
    S->outstanding -= 1;
    S->stats.completed += 1;
    if (status == UASTAR_CANCELLED) S->stats.cancelled += 1;
    if (status == UASTAR_REJECTED) S->stats.rejected += 1;
}

// A request's first dedup partition: its estimate, but at most 2^20 slots
// times its growth multiplier; the search grows it 4x in place whenever it
// is half full (serve_grow), so admission reserves what a request has shown
// it needs rather than what the largest like it might.
static uint64_t serve_partition_slots(const ServeState *S, const ServeReq &r) {
    const double load = S->cfg.load_factor > 0 && S->cfg.load_factor < 1 ? S->cfg.load_factor : 0.5;
    uint64_t slots = next_pow2_u64((uint64_t)((double)est_nodes(r.inst) / load));
    slots = std::min<uint64_t>(slots, 1ull << 20) * r.mult;
    return std::max<uint64_t>(slots, 1u << 12);
}

static void serve_release(ServeState *S, ServeSlot &sl) {
    S->tab_alloc.release(sl.tab_off, sl.tab_n);
    if (sl.bm_n) S->bm_alloc.release(sl.bm_off, sl.bm_n);
    S->heap_alloc.release(sl.heap_off, sl.heap_n);
}

// Copy n host bytes to dst on t's stream through the pinned staging ring
// (a plain pageable copy where the ring has no room).
static cudaError_t serve_upload(ServeState *S, ServeTier &t, void *dst, const void *src, uint64_t n) {
    while (!S->staged.empty() && cudaEventQuery(S->staged.front().ev) == cudaSuccess) {
        cudaEventDestroy(S->staged.front().ev);
        S->staged.pop_front();
    }
    const uint64_t need = (n + 255) & ~255ull, R = S->stage_bytes;
    uint64_t off = 0;
    bool room = need <= R;
    if (room && !S->staged.empty()) {
        const uint64_t tail = S->staged.front().off, head = S->staged.back().off + S->staged.back().n;
        if (head > tail) {  // in use: [tail, head)
            if (head + need <= R)
                off = head;
            else if (need <= tail)
                off = 0;  // wrap to the start
            else
                room = false;
        } else {  // in use: [tail, R) and [0, head)
            if (head + need <= tail)
                off = head;
            else
                room = false;
        }
    }
    cudaEvent_t ev = nullptr;
    if (room && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) room = false;
    if (!room) return cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, t.stream);
    std::memcpy(S->h_stage + off, src, n);
    cudaError_t e = cudaMemcpyAsync(dst, S->h_stage + off, n, cudaMemcpyHostToDevice, t.stream);
    if (e == cudaSuccess) e = cudaEventRecord(ev, t.stream);
    S->staged.push_back({off, need, ev});
    return e;
}

// Try to place `r` in a free slot of tier `t`.  Returns 1 placed, 0 no room
// now, -1 can never fit (completed as REJECTED by the caller).  A free slot
// is not part of a running quantum, so this may run while the tier's kernel
// is in flight: the partition clear and the bitmap copy queue behind it on
// the tier's stream, and the descriptor is uploaded with the next launch.
static int serve_admit(ServeState *S, ServeTier &t, ServeReq &r) {
    uastar_engine *eng = S->eng;
    const int q = t.free_slot();
    if (q < 0) return 0;
    // both tiers' resident requests share the GPU's co-resident CTAs
    if (S->tier[0].resident() + 8 * S->tier[1].resident() + (t.large ? 8 : 1) > S->capacity) return 0;
    const uint64_t tn = serve_partition_slots(S, r);
    const uint64_t bn = r.inst.kind == UASTAR_KIND_GRID ? r.words.size() + 2 : 0;
    BatchGeometry hgeo = t.geo;
    hgeo.set_capacity((t.geo.want + 1) * r.heap_mult - 1);
    const bool grid = r.inst.kind == UASTAR_KIND_GRID;
    const uint32_t hstride = grid ? hgeo.hg_grid.stride : hgeo.hg_puzzle.stride;
    const uint32_t hhcap = grid ? hgeo.hg_grid.hcap : hgeo.hg_puzzle.hcap;
    const uint64_t heaps_per_req = (uint64_t)t.geo.H * (t.large ? 8 : 1);
    const uint64_t hn = (heaps_per_req * hstride * (grid ? 16 : 8) + 127) / 128 * 8;  // 16-byte units
    if (tn > S->tab_alloc.capacity() || bn > S->bm_alloc.capacity() || hn > S->heap_alloc.capacity()) return -1;
    uint64_t toff = 0, boff = 0, hoff = 0;
    if (!S->tab_alloc.alloc(tn, 4, &toff)) return 0;
    if (bn && !S->bm_alloc.alloc(bn, 2, &boff)) {
        S->tab_alloc.release(toff, tn);
        return 0;
    }
    if (!S->heap_alloc.alloc(hn, 8, &hoff)) {
        S->tab_alloc.release(toff, tn);
        if (bn) S->bm_alloc.release(boff, bn);
        return 0;
    }
    ServeSlot &sl = t.slots[q];
    sl.busy = true;
    sl.tab_off = toff;
    sl.tab_n = tn;
    sl.bm_off = boff;
    sl.bm_n = bn;
    sl.heap_off = hoff;
    sl.heap_n = hn;
    sl.req = std::move(r);
    sl.req.attempts += 1;
    InstDesc d;
    std::memset(&d, 0, sizeof d);
    d.kind = sl.req.inst.kind;
    d.n = sl.req.inst.n;
    d.max_rounds = eng->cfg.max_rounds;
    d.tab_off = toff;
    d.log2_slots = (uint32_t)log2_u64(tn);
    d.fresh = 2;  // cleared here, at admission, by a full-GPU fill
    d.heap_off = hoff * 16;
    d.heap_stride = hstride;
    d.heap_hcap = hhcap;
    d.key_off = (uint64_t)q * t.kcap;
    d.key_cap = t.kcap;
    d.grow_at = tn / 2;
    if (fill_ff_async(eng, S->tab.as<Slot>() + toff, tn * sizeof(Slot), t.stream) != UASTAR_OK) {
        S->loop_error = UASTAR_CUDA_ERROR;
        return 0;
    }
    if (d.kind == UASTAR_KIND_GRID) {
        d.H = sl.req.inst.H;
        d.W = sl.req.inst.W;
        d.sx = sl.req.inst.sx;
        d.sy = sl.req.inst.sy;
        d.ex = sl.req.inst.ex;
        d.ey = sl.req.inst.ey;
        d.bm_word = boff * 2;
        if (serve_upload(S, t, S->bitmaps.as<uint64_t>() + boff, sl.req.words.data(), sl.req.words.size() * 8) !=
            cudaSuccess)
            S->loop_error = UASTAR_CUDA_ERROR;
    } else {
        d.start_key = pack_board(d.n, sl.req.inst.tiles);
    }
    t.descs[q] = d;
    return 1;
}

static BatchArgs serve_args(ServeState *S, ServeTier &t) {
    BatchArgs a;
    std::memset(&a, 0, sizeof a);
    a.descs = t.d_descs.as<InstDesc>();
    a.count = (uint32_t)t.nslots;
    a.bitmaps = S->bitmaps.as<uint32_t>();
    a.pdb3 = S->eng->pdb[3].as<uint8_t>();
    a.pdb4 = S->eng->pdb[4].as<uint8_t>();
    a.tab = S->tab.as<Slot>();
    a.heaps = S->heaps.as<uint8_t>();
    a.slice = t.geo.slice;
    a.hsize = t.d_hsize.as<uint32_t>();
    a.cand = t.d_cand.as<Cand>();
    a.outs = t.d_outs.as<InstOut>();
    if (t.large)
        a.cstates = t.d_states.as<TeamState>();
    else
        a.states = t.d_states.as<TeamState>();
    a.max_load = 0.75;
    a.H = t.geo.H;
    a.L_grid = t.geo.L_grid;
    a.L_puzzle = t.geo.L_puzzle;
    a.split_grid = t.geo.split_grid;
    a.split_puzzle = t.geo.split_puzzle;
    // a time slice per launch (every resident search runs until it has
    // passed), capped by a round count; or, without a slice, the round count.
    // 8 ms by default: the first 4000 requests of the 20000-request stream at
    // 1000/s served at 193 / 225 / 231-257 / 252 / 250 solves/s with 2 / 4 /
    // 8 / 12 / 16 ms slices (a launch's fixed costs against the wait of a
    // finished request for its slice's end).
    const bool sliced = S->cfg.quantum_us >= 0;
    a.quantum_ns = sliced ? (uint64_t)(S->cfg.quantum_us > 0 ? S->cfg.quantum_us : 8000) * 1000ull : 0;
    // paths beyond 1024 cells (~0.5 ms of pointer chase) are walked after
    // the quantum, on the walk stream (serve_walk_issue)
    a.walk_inline = 1024;
    a.budget = (uint64_t)(S->cfg.rounds_per_quantum > 0 ? S->cfg.rounds_per_quantum : sliced ? 65536 : 256);
    a.serving = 1;
    a.keys = t.d_keys.as<unsigned long long>();
    return a;
}

// One quantum of tier t: descriptors up, kernel, results down; `done` marks
// the end.
static cudaError_t serve_launch(ServeState *S, ServeTier &t) {
    cudaError_t e;
    const int n = t.extent();
    std::memcpy(t.h_descs, t.descs.data(), n * sizeof(InstDesc));
    if ((e = cudaMemcpyAsync(t.d_descs.p, t.h_descs, n * sizeof(InstDesc), cudaMemcpyHostToDevice,
                             t.stream)) != cudaSuccess)
        return e;
    BatchArgs a = serve_args(S, t);
    cudaEventRecord(t.e0, t.stream);
    if (t.large) {
        cudaLaunchConfig_t lc = {};
        cudaLaunchAttribute lat[1];
        lat[0].id = cudaLaunchAttributeClusterDimension;
        lat[0].val.clusterDim.x = 8;
        lat[0].val.clusterDim.y = 1;
        lat[0].val.clusterDim.z = 1;
        lc.gridDim = dim3((unsigned)(n * 8));
        lc.blockDim = dim3((unsigned)t.geo.T);
        lc.dynamicSmemBytes = t.geo.smem;
        lc.stream = t.stream;
        lc.attrs = lat;
        lc.numAttrs = 1;
        e = cudaLaunchKernelEx(&lc, k_batch_cluster, a);
    } else {
        k_batch<<<n, t.geo.T, t.geo.smem, t.stream>>>(a);
        e = cudaGetLastError();
    }
    S->eng->launches++;
    if (e != cudaSuccess) return e;
    cudaEventRecord(t.e1, t.stream);
    t.launched_n = n;
    if ((e = cudaMemcpyAsync(t.h_outs, t.d_outs.p, n * sizeof(InstOut), cudaMemcpyDeviceToHost,
                             t.stream)) != cudaSuccess)
        return e;
    if ((e = cudaEventRecord(t.done, t.stream)) != cudaSuccess) return e;
    t.inflight = true;
    t.launched.assign(t.nslots, 0);
    for (int q = 0; q < t.nslots; ++q) t.launched[q] = t.slots[q].busy;
    return cudaSuccess;
}

// Reads a solved slot's path (goal -> start keys) into `keys`.
static cudaError_t serve_path(ServeState *S, ServeTier &t, int q, std::vector<unsigned long long> &keys) {
    const InstOut &o = t.outs[q];
    const ServeSlot &sl = t.slots[q];
    cudaError_t e;
    if (o.path_len <= t.kcap) {
        keys.resize(o.path_len);
        if (o.path_len && (e = cudaMemcpyAsync(keys.data(), t.d_keys.as<unsigned long long>() + (size_t)q * t.kcap,
                                               o.path_len * 8, cudaMemcpyDeviceToHost, t.stream)) != cudaSuccess)
            return e;
        return cudaStreamSynchronize(t.stream);
    }
    // longer than a slot's key room (a maze): walk it again into a buffer
    // sized for the whole grid
    const uint64_t cap = sl.req.inst.kind == UASTAR_KIND_GRID ? (uint64_t)sl.req.inst.H * sl.req.inst.W + 1 : 4096;
    if ((e = t.d_walk.ensure(cap * 8 + 64)) != cudaSuccess) return e;
    unsigned long long *d_keys = t.d_walk.as<unsigned long long>();
    uint64_t *d_off = reinterpret_cast<uint64_t *>(d_keys + cap);
    uint64_t *d_cap = d_off + 1;
    unsigned long long *d_len = reinterpret_cast<unsigned long long *>(d_cap + 1);
    uint32_t *d_which = reinterpret_cast<uint32_t *>(d_len + 1);
    const uint64_t zero = 0;
    const uint32_t which = (uint32_t)q;
    cudaMemcpyAsync(d_off, &zero, 8, cudaMemcpyHostToDevice, t.stream);
    cudaMemcpyAsync(d_cap, &cap, 8, cudaMemcpyHostToDevice, t.stream);
    cudaMemcpyAsync(d_which, &which, 4, cudaMemcpyHostToDevice, t.stream);
    k_batch_walk<<<1, 32, 0, t.stream>>>(t.d_descs.as<InstDesc>(), t.d_outs.as<InstOut>(), d_which, 1u,
                                         S->tab.as<Slot>(), d_keys, d_off, d_cap, d_len);
    S->eng->launches++;
    unsigned long long len = 0;
    cudaMemcpyAsync(&len, d_len, 8, cudaMemcpyDeviceToHost, t.stream);
    if ((e = cudaStreamSynchronize(t.stream)) != cudaSuccess) return e;
    if (len > cap) len = 0;
    keys.resize(len);
    if (len && (e = cudaMemcpyAsync(keys.data(), d_keys, len * 8, cudaMemcpyDeviceToHost, t.stream)) != cudaSuccess)
        return e;
    return cudaStreamSynchronize(t.stream);
}

// Checks a solved request's path on the host and fills its cost fields;
// returns the status to report.
static int32_t serve_finish_ok(ServeReq &r, const InstOut &o, const std::vector<unsigned long long> &kk) {
    const auto &in = r.inst;
    const uint64_t len = kk.size();
    if (len == 0) return UASTAR_ARENA_FULL;
    if (in.kind == UASTAR_KIND_GRID) {
        r.acc.straight = (int64_t)(o.goal_best >> 32);
        r.acc.diagonal = (int64_t)(o.goal_best & 0xffffffffu);
        std::vector<int32_t> path(len);
        for (uint64_t u = 0; u < len; ++u) path[u] = (int32_t)kk[len - 1 - u];
        int64_t a2 = 0, b2 = 0;
        float fc = 0;
        if (uastar_validate_grid_path(r.words.data(), in.H, in.W, in.sx, in.sy, in.ex, in.ey, path.data(),
                                      (int64_t)len, &a2, &b2, &fc) != UASTAR_OK ||
            a2 != r.acc.straight || b2 != r.acc.diagonal)
            return UASTAR_CUDA_ERROR;
        r.acc.cost = fc;
        return UASTAR_OK;
    }
    r.acc.steps = (int32_t)o.goal_best;
    std::vector<int32_t> moves;
    auto blank = [&](uint64_t k) {
        for (int c = 0; c < in.n * in.n; ++c)
            if (((k >> (4 * c)) & 15) == 0) return c;
        return -1;
    };
    for (uint64_t u = len - 1; u >= 1; --u) {
        const int pb = blank(kk[u]), cb = blank(kk[u - 1]);
        moves.push_back(cb - pb == in.n ? 0 : cb - pb == -in.n ? 1 : cb - pb == 1 ? 2 : 3);
    }
    if ((int64_t)moves.size() != r.acc.steps ||
        uastar_validate_puzzle_moves(in.n, in.tiles, moves.data(), (int64_t)moves.size()) != UASTAR_OK)
        return UASTAR_CUDA_ERROR;
    return UASTAR_OK;
}

// Room for n keys in the walk ring, used first in, first out.
static bool walk_ring_alloc(ServeState *S, uint64_t n, uint64_t *off) {
    const uint64_t R = S->walk_ring_keys;
    if (n > R) return false;
    if (S->walking.empty()) {
        *off = 0;
        return true;
    }
    const uint64_t tail = S->walking.front().ring_off;
    const uint64_t head = S->walking.back().ring_off + S->walking.back().n + 1;
    if (head > tail) {  // in use: [tail, head)
        if (head + n <= R) {
            *off = head;
            return true;
        }
        if (n <= tail) {  // wrap to the start
            *off = 0;
            return true;
        }
        return false;
    }
    if (head + n <= tail) {  // in use: [tail, R) and [0, head)
        *off = head;
        return true;
    }
    return false;
}

// Walk slot q's solved request (a path longer than the in-quantum limit)
// on the walk stream behind the quantum that solved it, into the ring, and
// copy the keys to the pinned ring; the request completes when they are on
// the host (serve_walk_finish).  Its heap slice and bitmap are released now,
// its partition then.  False: no ring room (the caller walks it now).
static bool serve_walk_issue(ServeState *S, ServeTier &t, int q) {
    const InstOut &o = t.outs[q];
    ServeSlot &sl = t.slots[q];
    const uint64_t n = path_cells(sl.req.inst.kind, o.goal_best);
    uint64_t off = 0;
    if (!walk_ring_alloc(S, n + 1, &off)) return false;
    ServeWalk w;
    if (cudaEventCreateWithFlags(&w.ev, cudaEventDisableTiming) != cudaSuccess) return false;
    unsigned long long *d = S->walk_ring.as<unsigned long long>() + off;
    cudaStreamWaitEvent(S->walk_stream, t.done, 0);
    k_serve_walk<<<1, 32, 0, S->walk_stream>>>(
        S->tab.as<Slot>() + sl.tab_off, o.goal_slot, d, n,
        sl.req.inst.kind == UASTAR_KIND_GRID ? GridProblem::kLink : PuzzleProblem<4>::kLink);
    S->eng->launches++;
    cudaMemcpyAsync(S->h_walk_ring + off, d, (n + 1) * 8, cudaMemcpyDeviceToHost, S->walk_stream);
    cudaEventRecord(w.ev, S->walk_stream);
    if (cudaGetLastError() != cudaSuccess) {
        S->loop_error = UASTAR_CUDA_ERROR;
        cudaEventDestroy(w.ev);
        return false;
    }
    w.o = o;
    w.tab_off = sl.tab_off;
    w.tab_n = sl.tab_n;
    w.ring_off = off;
    w.n = n;
    if (sl.bm_n) S->bm_alloc.release(sl.bm_off, sl.bm_n);
    S->heap_alloc.release(sl.heap_off, sl.heap_n);
    w.req = std::move(sl.req);
    S->walking.push_back(std::move(w));
    return true;
}

// A deferred walk's keys are on the host: validate and complete.
static void serve_walk_finish(ServeState *S, ServeWalk &w) {
    const unsigned long long *h = S->h_walk_ring + w.ring_off;
    const uint64_t len = h[w.n];
    int32_t status = UASTAR_CUDA_ERROR;
    if (len == w.n) {
        std::vector<unsigned long long> keys(h, h + len);
        status = serve_finish_ok(w.req, w.o, keys);
    }
    S->tab_alloc.release(w.tab_off, w.tab_n);
    cudaEventDestroy(w.ev);
    serve_complete(S, w.req, status);
}

// Move slot q's paused search (it passed grow_at) to a partition 4x larger:
// the old one is rehashed into the new on the tier's stream (slots, prev
// links, heap entries, goal slot), then released.  Without room it carries
// on in place up to the table's load limit.
static void serve_grow(ServeState *S, ServeTier &t, int q) {
    uastar_engine *eng = S->eng;
    ServeSlot &sl = t.slots[q];
    InstDesc &d = t.descs[q];
    const uint64_t old_n = 1ull << d.log2_slots, new_n = old_n * 4;
    uint64_t noff = 0;
    if (new_n > (1ull << 31) || !S->tab_alloc.alloc(new_n, 4, &noff)) {
        d.grow_at = 0;
        return;
    }
    // a larger map replaces the one that growths queued earlier may still read
    if (old_n * 4 > t.d_map.bytes && cudaStreamSynchronize(t.stream) != cudaSuccess) {
        S->loop_error = UASTAR_CUDA_ERROR;
        return;
    }
    if (t.d_map.ensure(old_n * 4) != cudaSuccess) {
        S->tab_alloc.release(noff, new_n);
        d.grow_at = 0;
        return;
    }
    Slot *src = S->tab.as<Slot>() + d.tab_off, *dst = S->tab.as<Slot>() + noff;
    uint32_t *map = t.d_map.as<uint32_t>();
    const int blocks = std::max(1, eng->sms * 4);
    const uint32_t per = t.large ? 8u : 1u;
    const uint32_t k = t.geo.H * per;
    uint32_t *hsize = t.d_hsize.as<uint32_t>() + (size_t)q * k;
    TeamState *st = t.d_states.as<TeamState>() + q;
    fill_ff_async(eng, dst, new_n * sizeof(Slot), t.stream);
    if (d.kind == UASTAR_KIND_GRID) {
        k_grow_move<false, GridProblem::kPrevInKey><<<blocks, 256, 0, t.stream>>>(src, old_n, dst, new_n - 1, map);
        k_grow_links<false, GridProblem::kLink><<<blocks, 256, 0, t.stream>>>(src, old_n, dst, map);
    } else {
        k_grow_move<false, false><<<blocks, 256, 0, t.stream>>>(src, old_n, dst, new_n - 1, map);
        k_grow_links<false, PuzzleProblem<4>::kLink><<<blocks, 256, 0, t.stream>>>(src, old_n, dst, map);
    }
    if (d.kind == UASTAR_KIND_GRID)
        k_grow_heaps<GridProblem><<<blocks, 256, 0, t.stream>>>(
            reinterpret_cast<GridEntry *>(S->heaps.as<uint8_t>() + d.heap_off), d.heap_stride, t.geo.L_grid, hsize,
            k, map, st);
    else
        k_grow_heaps<PuzzleProblem<4>><<<blocks, 256, 0, t.stream>>>(
            reinterpret_cast<PuzzleEntry *>(S->heaps.as<uint8_t>() + d.heap_off), d.heap_stride, t.geo.L_puzzle,
            hsize, k, map, st);
    eng->launches += 4;
    if (cudaGetLastError() != cudaSuccess) {
        S->loop_error = UASTAR_CUDA_ERROR;
        return;
    }
    // The old range may be handed out (and cleared on another stream) only
    // once the growth kernels have read it: it is released when this tier's
    // next quantum, queued behind them, has finished (no host wait here).
    t.release_after.emplace_back(sl.tab_off, sl.tab_n);
    sl.tab_off = noff;
    sl.tab_n = new_n;
    d.tab_off = noff;
    d.log2_slots += 2;
    d.grow_at = new_n / 2;
}

// Move CTA slot q's parked request onto a free cluster slot without
// restarting it (k_migrate_heaps; the team state is copied, the partition and
// bitmap stay).  Returns false, changing nothing, when no cluster slot, CTA
// share or heap space is free.
static bool serve_migrate(ServeState *S, int q) {
    ServeTier &small = S->tier[0], &large = S->tier[1];
    const int q2 = large.free_slot();
    if (q2 < 0 || small.resident() - 1 + 8 * (large.resident() + 1) > S->capacity) return false;
    ServeSlot &from = small.slots[q];
    InstDesc d = small.descs[q];
    const bool grid = d.kind == UASTAR_KIND_GRID;
    const uint64_t hd = (uint64_t)large.geo.H * 8;
    const uint64_t hn = (hd * d.heap_stride * (grid ? 16 : 8) + 127) / 128 * 8;  // 16-byte units
    uint64_t hoff = 0;
    if (!S->heap_alloc.alloc(hn, 8, &hoff)) return false;
    uastar_engine *eng = S->eng;
    if (small.d_map.ensure(64) != cudaSuccess) {
        S->heap_alloc.release(hoff, hn);
        return false;
    }
    uint32_t *d_err = small.d_map.as<uint32_t>();
    cudaMemsetAsync(d_err, 0, 4, small.stream);
    const uint32_t hs = small.geo.H;
    const uint32_t *src_size = small.d_hsize.as<uint32_t>() + (size_t)q * hs;
    uint32_t *dst_size = large.d_hsize.as<uint32_t>() + (size_t)q2 * hd;
    const unsigned blocks = (unsigned)((hd + 127) / 128);
    if (grid)
        k_migrate_heaps<GridProblem><<<blocks, 128, 0, small.stream>>>(
            reinterpret_cast<const GridEntry *>(S->heaps.as<uint8_t>() + d.heap_off), d.heap_stride, src_size, hs,
            reinterpret_cast<GridEntry *>(S->heaps.as<uint8_t>() + hoff * 16), d.heap_stride, dst_size, (uint32_t)hd,
            small.geo.L_grid, d.heap_hcap, d_err);
    else
        k_migrate_heaps<PuzzleProblem<4>><<<blocks, 128, 0, small.stream>>>(
            reinterpret_cast<const PuzzleEntry *>(S->heaps.as<uint8_t>() + d.heap_off), d.heap_stride, src_size, hs,
            reinterpret_cast<PuzzleEntry *>(S->heaps.as<uint8_t>() + hoff * 16), d.heap_stride, dst_size,
            (uint32_t)hd, small.geo.L_puzzle, d.heap_hcap, d_err);
    eng->launches++;
    cudaMemcpyAsync(large.d_states.as<TeamState>() + q2, small.d_states.as<TeamState>() + q, sizeof(TeamState),
                    cudaMemcpyDeviceToDevice, small.stream);
    uint32_t err = 0;
    cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, small.stream);
    if (cudaStreamSynchronize(small.stream) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
        S->loop_error = UASTAR_CUDA_ERROR;
        return false;
    }
    if (err) {  // the per-heap capacity is the same: spread over 8x the heaps this cannot overflow
        S->heap_alloc.release(hoff, hn);
        return false;
    }
    // the request now lives on cluster slot q2
    S->heap_alloc.release(from.heap_off, from.heap_n);
    ServeSlot &to = large.slots[q2];
    to = std::move(from);
    to.req.acc.migrations += 1;
    to.heap_off = hoff;
    to.heap_n = hn;
    from = ServeSlot();
    small.descs[q].kind = 0;
    d.heap_off = hoff * 16;
    d.key_off = (uint64_t)q2 * large.kcap;
    d.key_cap = large.kcap;
    d.fresh = 0;
    large.descs[q2] = d;
    return true;
}

// Retire tier t's finished quantum: completed requests report; one that
// overflows its CTA slot restarts on a cluster slot with more space, one that
// overflows a cluster slot retries there with more.  A request that keeps its
// CTA's heaps saturated (a wide frontier, which more heaps cover in fewer
// rounds) moves to a cluster slot with its search state (serve_migrate) when
// the GPU has spare CTAs and nothing waits (`spare`: latency), or once it has
// taken 4M expansions (a request that large would otherwise be the stream's
// tail); other requests stay on one CTA, the most work per CTA.  A grid with
// a thin frontier never moves: its rounds are bounded by its path length,
// which a cluster would not shorten.
static void serve_retire(ServeState *S, ServeTier &t, std::deque<ServeReq> &to_large, bool spare) {
    ServeTier &large = S->tier[1];
    std::memcpy(t.outs.data(), t.h_outs, (size_t)t.launched_n * sizeof(InstOut));
    for (const auto &r : t.release_after) S->tab_alloc.release(r.first, r.second);
    t.release_after.clear();
    float ms = 0;
    cudaEventElapsedTime(&ms, t.e0, t.e1);
    S->stats.quanta += 1;
    S->stats.busy_ms += ms;
    std::vector<unsigned long long> keys;
    for (int q = 0; q < t.nslots; ++q) {
        ServeSlot &sl = t.slots[q];
        if (!sl.busy || !t.launched[q]) continue;  // admitted while the quantum ran
        t.descs[q].fresh = 0;
        const InstOut &o = t.outs[q];
        ServeReq &r = sl.req;
        if (o.status == ST_RUNNING) {
            if (t.descs[q].grow_at && o.inserted > t.descs[q].grow_at) {
                serve_grow(S, t, q);
                if (S->loop_error) return;
            }
            // a wide frontier that has already taken 4M expansions (or any, when
            // the GPU has spare CTAs) moves to a cluster slot, search state and all
            const bool saturated = o.rounds >= 1024 && (double)o.expanded >= 0.5 * t.geo.H * (double)o.rounds;
            if (!t.large && saturated && large.nslots > 0 && to_large.empty() && (spare || o.expanded >= 4000000ull)) {
                if (serve_migrate(S, q)) continue;
                if (S->loop_error) return;
            }
            continue;
        }
        r.acc.device_ms = (double)(o.t_end - o.t_start) * 1e-6;
        r.acc.expanded += (int64_t)o.expanded;
        r.acc.generated += (int64_t)o.generated;
        r.acc.rounds += (int64_t)o.rounds;
        int32_t status = (int32_t)o.status;
        if (status == ST_OK && o.path_len == kWalkDeferred && serve_walk_issue(S, t, q)) {
            t.descs[q].kind = 0;
            sl = ServeSlot();
            continue;
        }
        if (S->loop_error) return;
        if (status == ST_OK) {
            if (serve_path(S, t, q, keys) != cudaSuccess) {
                S->loop_error = UASTAR_CUDA_ERROR;
                return;
            }
            status = serve_finish_ok(r, o, keys);
        }
        serve_release(S, sl);
        t.descs[q].kind = 0;
        if ((status == ST_HASH_FULL || status == ST_HEAP_OVERFLOW) && r.attempts < 8) {
            if (status == ST_HASH_FULL) r.mult = std::max<uint64_t>(r.mult * (t.large ? 4 : 16), 16);
            if (status == ST_HEAP_OVERFLOW) r.heap_mult *= t.large ? 16 : 4;
            if (large.nslots > 0) {
                if (t.large)
                    to_large.push_front(std::move(r));
                else
                    to_large.push_back(std::move(r));
                sl = ServeSlot();
                continue;
            }
        }
        if ((status == ST_HASH_FULL || status == ST_HEAP_OVERFLOW) && r.attempts < 8 && large.nslots == 0) {
            // no cluster tier: retry on a CTA slot with the larger space
            std::lock_guard<std::mutex> lk(S->mu);
            S->incoming.push_front(std::move(r));
            sl = ServeSlot();
            continue;
        }
        serve_complete(S, r, status);
        sl = ServeSlot();
    }
}

static void serve_loop(ServeState *S) {
    uastar_engine *eng = S->eng;
    cudaSetDevice(eng->device);
    // UASTAR_DEBUG: one line per second (quanta and kernel time per tier,
    // residency, queues)
    double log_t = uastar_now_s();
    int64_t log_q[2] = {0, 0};
    double log_ms[2] = {0, 0};
    std::vector<ServeReq> pending;   // arrived or future requests, sorted by arrival
    std::deque<ServeReq> to_large;   // requests waiting for a cluster slot
    ServeTier &small = S->tier[0], &large = S->tier[1];
    cudaError_t e;
    auto fail = [&](cudaError_t err, const char *what) {
        fail_cuda(eng, err, what);
        S->loop_error = UASTAR_CUDA_ERROR;
    };
    for (;;) {
        // 1. intake and cancellation
        {
            std::unique_lock<std::mutex> lk(S->mu);
            bool got = false;
            while (!S->incoming.empty()) {
                pending.push_back(std::move(S->incoming.front()));
                S->incoming.pop_front();
                got = true;
            }
            std::vector<int64_t> cancels;
            cancels.swap(S->cancels);
            lk.unlock();
            if (got)
                std::stable_sort(pending.begin(), pending.end(),
                                 [](const ServeReq &a, const ServeReq &b) { return a.arrival_s < b.arrival_s; });
            for (int64_t cid : cancels) {
                for (size_t i = 0; i < pending.size(); ++i)
                    if (pending[i].id == cid) {
                        serve_complete(S, pending[i], UASTAR_CANCELLED);
                        pending.erase(pending.begin() + i);
                        break;
                    }
                for (size_t i = 0; i < to_large.size(); ++i)
                    if (to_large[i].id == cid) {
                        serve_complete(S, to_large[i], UASTAR_CANCELLED);
                        to_large.erase(to_large.begin() + i);
                        break;
                    }
                // resident: only between quanta (its slot is not in a running kernel)
                for (auto &t : S->tier) {
                    if (t.inflight) {
                        std::lock_guard<std::mutex> lk2(S->mu);
                        S->cancels.push_back(cid);  // retry after this tier's quantum
                        continue;
                    }
                    for (int q = 0; q < t.nslots; ++q)
                        if (t.slots[q].busy && t.slots[q].req.id == cid) {
                            serve_complete(S, t.slots[q].req, UASTAR_CANCELLED);
                            serve_release(S, t.slots[q]);
                            t.slots[q] = ServeSlot();
                            t.descs[q].kind = 0;
                        }
                }
            }
        }
        if (S->loop_error) break;
        // 2. retire finished quanta
        for (auto &t : S->tier) {
            if (!t.inflight) continue;
            e = cudaEventQuery(t.done);
            if (e == cudaErrorNotReady) continue;
            if (e != cudaSuccess) {
                fail(e, "serve quantum");
                break;
            }
            t.inflight = false;
            if (debug_log()) {
                float ms = 0;
                cudaEventElapsedTime(&ms, t.e0, t.e1);
                log_q[t.large] += 1;
                log_ms[t.large] += ms;
            }
            const bool spare = pending.empty() &&
                               S->tier[0].resident() + 8 * (S->tier[1].resident() + 1) <= S->capacity;
            serve_retire(S, t, to_large, spare);
        }
        if (S->loop_error) break;
        // 2b. deferred walks whose keys are on the host complete
        while (!S->walking.empty()) {
            e = cudaEventQuery(S->walking.front().ev);
            if (e == cudaErrorNotReady) break;
            if (e != cudaSuccess) {
                fail(e, "serve walk");
                break;
            }
            serve_walk_finish(S, S->walking.front());
            S->walking.pop_front();
        }
        if (S->loop_error) break;
        // 3. admission: promoted requests take cluster slots, then arrived
        //    requests take CTA slots in arrival order
        while (!to_large.empty()) {
            const int r = serve_admit(S, large, to_large.front());
            if (r == 0) break;
            if (r < 0) serve_complete(S, to_large.front(), UASTAR_REJECTED);
            to_large.pop_front();
        }
        const double now = uastar_now_s();
        {
            std::vector<ServeReq> keep;
            bool small_full = false;
            for (auto &r : pending) {
                if (r.arrival_s > now) {
                    keep.push_back(std::move(r));
                    continue;
                }
                if (small_full) {
                    keep.push_back(std::move(r));
                    continue;
                }
                const int a = serve_admit(S, small, r);
                if (a == 0) {
                    small_full = true;
                    keep.push_back(std::move(r));
                } else if (a < 0) {
                    serve_complete(S, r, UASTAR_REJECTED);
                }
            }
            pending.swap(keep);
        }
        const int rs = small.resident(), rl = large.resident();
        if (debug_log() && uastar_now_s() - log_t >= 1.0) {
            std::fprintf(stderr,
                         "[uastar serve] CTA tier %lld quanta %.2f ms avg, %d/%d resident; cluster tier %lld quanta "
                         "%.2f ms avg, %d/%d resident; waiting %zu (cluster queue %zu); completed %lld\n",
                         (long long)log_q[0], log_q[0] ? log_ms[0] / log_q[0] : 0.0, rs, small.nslots,
                         (long long)log_q[1], log_q[1] ? log_ms[1] / log_q[1] : 0.0, rl, large.nslots,
                         pending.size(), to_large.size(), (long long)S->stats.completed);
            log_t = uastar_now_s();
            log_q[0] = log_q[1] = 0;
            log_ms[0] = log_ms[1] = 0;
        }
        S->stats.peak_resident = std::max(S->stats.peak_resident, rs + rl);
        S->stats.peak_budget_gb =
            std::max(S->stats.peak_budget_gb, ((double)S->tab_alloc.used() * sizeof(Slot) +
                                               (double)S->bm_alloc.used() * 8 + (double)S->heap_alloc.used() * 16) /
                                                  1e9);
        if (S->loop_error) break;
        // 4. launch the tiers that have work, together and the cluster tier
        //    first, once neither is in flight: a cluster's 8 CTAs need room
        //    in one GPC at once, which a CTA-tier launch spread over every SM
        //    does not leave, so launched apart the two kernels would take
        //    turns on the GPU instead of sharing it
        const bool idle = !small.inflight && !large.inflight;
        for (int ti = 1; ti >= 0 && idle; --ti) {
            ServeTier &t = S->tier[ti];
            if (!t.nslots || !t.resident()) continue;
            if ((e = serve_launch(S, t)) != cudaSuccess) {
                fail(e, "serve launch");
                break;
            }
        }
        if (S->loop_error) break;
        if (!small.inflight && !large.inflight) {
            std::unique_lock<std::mutex> lk(S->mu);
            if (S->abort_now || (S->draining && S->outstanding == 0)) break;
            double wait_s = 0.002;
            if (!pending.empty()) wait_s = std::max(0.0, std::min(wait_s, pending.front().arrival_s - now));
            if (S->incoming.empty() && S->cancels.empty())
                S->cv.wait_for(lk, std::chrono::duration<double>(wait_s));
            continue;
        }
        {
            std::lock_guard<std::mutex> lk(S->mu);
            if (S->abort_now) break;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    for (auto &t : S->tier)
        if (t.stream) cudaStreamSynchronize(t.stream);
    // solved requests still being walked complete as solved
    if (S->walk_stream) cudaStreamSynchronize(S->walk_stream);
    while (!S->walking.empty()) {
        serve_walk_finish(S, S->walking.front());
        S->walking.pop_front();
    }
    // drain: anything left is reported as cancelled
    for (auto &r : pending) serve_complete(S, r, UASTAR_CANCELLED);
    for (auto &r : to_large) serve_complete(S, r, UASTAR_CANCELLED);
    for (auto &t : S->tier)
        for (auto &sl : t.slots)
            if (sl.busy) serve_complete(S, sl.req, UASTAR_CANCELLED);
    std::deque<ServeReq> rest;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        rest.swap(S->incoming);
    }
    for (auto &r : rest) serve_complete(S, r, UASTAR_CANCELLED);
}

static void serve_free(ServeState *S) {
    for (auto &t : S->tier) {
        for (DevBuf *b : {&t.d_descs, &t.d_outs, &t.d_states, &t.d_hsize, &t.d_cand, &t.d_keys, &t.d_walk, &t.d_map})
            b->release();
        if (t.e0) cudaEventDestroy(t.e0);
        if (t.e1) cudaEventDestroy(t.e1);
        if (t.done) cudaEventDestroy(t.done);
        if (t.stream) cudaStreamDestroy(t.stream);
        if (t.h_descs) cudaFreeHost(t.h_descs);
        if (t.h_outs) cudaFreeHost(t.h_outs);
        t.h_descs = nullptr;
        t.h_outs = nullptr;
    }
    for (DevBuf *b : {&S->tab, &S->bitmaps, &S->heaps, &S->walk_ring}) b->release();
    if (S->h_walk_ring) cudaFreeHost(S->h_walk_ring);
    S->h_walk_ring = nullptr;
    for (auto &st : S->staged) cudaEventDestroy(st.ev);
    S->staged.clear();
    if (S->h_stage) cudaFreeHost(S->h_stage);
    S->h_stage = nullptr;
    if (S->walk_stream) cudaStreamDestroy(S->walk_stream);
    S->walk_stream = nullptr;
}

}  // namespace uastar

extern "C" {

double uastar_now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int32_t uastar_serve_start(uastar_engine *eng, const uastar_serve_config *cfg) {
    if (!eng) return UASTAR_BAD_INPUT;
    if (eng->serve) {
        eng->set_err("serving loop already running");
        return UASTAR_BAD_INPUT;
    }
    cudaSetDevice(eng->device);
    // the serving arenas take the budget: the batched engine's cached
    // buffers go back first (a later batch call allocates them again)
    release_batch_buffers(eng);
    auto *S = new ServeState();
    S->eng = eng;
    if (cfg) S->cfg = *cfg;
    if (!(S->cfg.hbm_budget_gb > 0)) S->cfg.hbm_budget_gb = 120.0;
    ServeTier &small = S->tier[0], &large = S->tier[1];
    // Two threads per heap: a resident search's latency is its rounds, and
    // 128 heaps per CTA pop twice as many entries per round as 64 (the
    // 20000-request stream's first 4000 at 1000/s: 219-227 solves/s against
    // 154 with 4 threads per heap, 175-186 with 1).
    const int tph = S->cfg.threads_per_heap > 0 ? S->cfg.threads_per_heap : 2;
    int32_t grc = resolve_block_geometry(eng, S->cfg.threads_per_instance, tph, &small.geo);
    if (grc) {
        delete S;
        return grc;
    }
    // resident searches keep their heaps across quanta: a request that
    // overflows restarts, so the default leaves room (16383 entries per heap)
    small.geo.set_capacity(S->cfg.heap_capacity > 0 ? (uint64_t)S->cfg.heap_capacity : 16383);
    large.geo = small.geo;
    large.large = true;
    const int capacity = small.geo.ctas;  // co-resident CTAs of the quantum kernels
    S->capacity = capacity;
    // Both tiers can hold up to the whole GPU; admission keeps their resident
    // requests within the co-resident CTAs together.
    int nlarge = 0;
    if (S->cfg.cluster_slots >= 0 && resolve_cluster_geometry(eng, 8, &large.geo) == UASTAR_OK) {
        nlarge = std::max(1, large.geo.ctas / 8);
        if (S->cfg.cluster_slots > 0) nlarge = std::min(nlarge, S->cfg.cluster_slots);
    }
    int nsmall = capacity;
    if (S->cfg.slots > 0) {
        nsmall = std::min(nsmall, S->cfg.slots);
        if (S->cfg.slots < 8 && S->cfg.cluster_slots <= 0) nlarge = 0;
    }
    small.nslots = std::max(1, nsmall);
    large.nslots = nlarge;
    // The budget is split into three arenas that requests draw from:
    // heap slices (20 %), grid bitmaps (5 %) and dedup partitions (75 %).
    const double budget_b = S->cfg.hbm_budget_gb * 1e9;
    const uint64_t heap_units = (uint64_t)(budget_b * 0.20 / 16);
    const uint64_t bm_words = (uint64_t)(budget_b * 0.05 / 8);
    const double tab_b = budget_b * 0.75;
    S->heap_bytes = heap_units * 16;
    if (S->cfg.heap_capacity <= 0 && heap_units * 16 < (uint64_t)small.geo.H * small.geo.slice) {
        // a small budget: the default heaps shrink to what one slot's share allows
        small.geo.set_capacity(4095);
        large.geo.set_capacity(4095);
    }
    if (tab_b < (double)(1u << 20) * sizeof(Slot) || heap_units * 16 < (uint64_t)small.geo.H * small.geo.slice) {
        delete S;
        eng->set_err("serving budget too small");
        return UASTAR_BAD_INPUT;
    }
    const uint64_t tab_slots = (uint64_t)(tab_b / sizeof(Slot));
    S->tab_alloc.reset(tab_slots);
    S->bm_alloc.reset(bm_words);
    S->heap_alloc.reset(heap_units);
    cudaError_t e = cudaSuccess;
    if ((e = S->tab.ensure(tab_slots * sizeof(Slot))) == cudaSuccess)
        e = S->bitmaps.ensure(bm_words * 8 + 64);
    if (e == cudaSuccess) e = S->heaps.ensure(S->heap_bytes);
    // deferred walks: 4 M keys of ring (32 MB here and pinned on the host)
    S->walk_ring_keys = 1ull << 22;
    if (e == cudaSuccess) e = S->walk_ring.ensure(S->walk_ring_keys * 8);
    if (e == cudaSuccess) e = cudaMallocHost(&S->h_walk_ring, S->walk_ring_keys * 8);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S->walk_stream, cudaStreamNonBlocking);
    // bitmap uploads: 128 MB of pinned staging
    S->stage_bytes = 128ull << 20;
    if (e == cudaSuccess) e = cudaMallocHost(&S->h_stage, S->stage_bytes);
    for (auto &t : S->tier) {
        if (e != cudaSuccess) break;
        const size_t ctas = (size_t)t.nslots * (t.large ? 8 : 1);
        t.slots.assign(t.nslots, ServeSlot());
        t.descs.assign(t.nslots, InstDesc());
        std::memset(t.descs.data(), 0, t.descs.size() * sizeof(InstDesc));
        t.outs.assign(t.nslots, InstOut());
        if ((e = cudaMallocHost(&t.h_descs, std::max(1, t.nslots) * sizeof(InstDesc))) != cudaSuccess ||
            (e = cudaMallocHost(&t.h_outs, std::max(1, t.nslots) * sizeof(InstOut))) != cudaSuccess)
            break;
        if (!t.nslots) continue;
        t.kcap = 65600;  // path keys per slot (2 (H + W) + 64 for grids up to 16384 x 16384)
        if ((e = t.d_keys.ensure((size_t)t.nslots * t.kcap * 8)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&t.done, cudaEventDisableTiming)) != cudaSuccess ||
            (e = t.d_descs.ensure((size_t)t.nslots * sizeof(InstDesc))) != cudaSuccess ||
            (e = t.d_outs.ensure((size_t)t.nslots * sizeof(InstOut))) != cudaSuccess ||
            (e = t.d_states.ensure((size_t)t.nslots * sizeof(TeamState))) != cudaSuccess ||
            (e = t.d_hsize.ensure(ctas * t.geo.H * 4)) != cudaSuccess ||
            (e = t.d_cand.ensure(ctas * 2 * (8 * t.geo.H + 1) * sizeof(Cand))) != cudaSuccess ||
            (e = cudaStreamCreateWithFlags(&t.stream, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaEventCreate(&t.e0)) != cudaSuccess || (e = cudaEventCreate(&t.e1)) != cudaSuccess)
            break;
    }
    if (e != cudaSuccess) {
        serve_free(S);
        delete S;
        return fail_cuda(eng, e, "serving allocation");
    }
    eng->serve = S;
    S->th = std::thread(serve_loop, S);
    return UASTAR_OK;
}

int64_t uastar_serve_submit(uastar_engine *eng, const uastar_instance *inst, double arrival_s) {
    if (!eng || !eng->serve || !inst) return -UASTAR_BAD_INPUT;
    ServeState *S = eng->serve;
    if (check_instance(*inst) != UASTAR_OK) return -UASTAR_BAD_INPUT;
    if (inst->kind == UASTAR_KIND_PUZZLE && !eng->pdb_ready[inst->n]) return -UASTAR_BAD_INPUT;
    ServeReq r;
    r.inst = *inst;
    r.arrival_s = arrival_s > 0 ? arrival_s : uastar_now_s();
    if (inst->kind == UASTAR_KIND_GRID) {
        const size_t nw = ((uint64_t)inst->H * inst->W + 63) / 64;
        r.words.assign(inst->words, inst->words + nw);
        r.inst.words = nullptr;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->draining) return -UASTAR_BAD_INPUT;
    r.id = S->next_id++;
    S->stats.submitted += 1;
    S->outstanding += 1;
    const int64_t id = r.id;
    if (inst->kind == UASTAR_KIND_PUZZLE && !board_solvable(inst->n, inst->tiles)) {
        uastar_serve_completion c;
        std::memset(&c, 0, sizeof c);
        c.id = id;
        c.result.status = UASTAR_NO_SOLUTION;
        S->done.push_back(c);
        S->outstanding -= 1;
        S->stats.completed += 1;
        return id;
    }
    S->incoming.push_back(std::move(r));
    S->cv.notify_one();
    return id;
}

int32_t uastar_serve_poll(uastar_engine *eng, uastar_serve_completion *out, int32_t cap) {
    if (!eng || !eng->serve || (!out && cap > 0)) return -UASTAR_BAD_INPUT;
    ServeState *S = eng->serve;
    std::lock_guard<std::mutex> lk(S->mu);
    int32_t n = 0;
    while (n < cap && !S->done.empty()) {
        out[n++] = S->done.front();
        S->done.pop_front();
    }
    return n;
}

int32_t uastar_serve_cancel(uastar_engine *eng, int64_t id) {
    if (!eng || !eng->serve) return UASTAR_BAD_INPUT;
    ServeState *S = eng->serve;
    std::lock_guard<std::mutex> lk(S->mu);
    for (size_t i = 0; i < S->incoming.size(); ++i)
        if (S->incoming[i].id == id) {
            ServeReq r = std::move(S->incoming[i]);
            S->incoming.erase(S->incoming.begin() + i);
            uastar_serve_completion c;
            std::memset(&c, 0, sizeof c);
            c.id = id;
            c.result.status = UASTAR_CANCELLED;
            S->done.push_back(c);
            S->outstanding -= 1;
            S->stats.completed += 1;
            S->stats.cancelled += 1;
            return UASTAR_OK;
        }
    S->cancels.push_back(id);
    S->cv.notify_one();
    return UASTAR_OK;
}

int32_t uastar_serve_stop(uastar_engine *eng, double timeout_s, uastar_serve_stats *stats) {
    if (!eng || !eng->serve) return UASTAR_BAD_INPUT;
    ServeState *S = eng->serve;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->draining = true;
        if (!(timeout_s > 0)) S->abort_now = true;
        S->cv.notify_one();
    }
    if (timeout_s > 0) {
        const double deadline = uastar_now_s() + timeout_s;
        for (;;) {
            {
                std::lock_guard<std::mutex> lk(S->mu);
                if (S->outstanding == 0) break;
            }
            if (uastar_now_s() > deadline) {
                std::lock_guard<std::mutex> lk(S->mu);
                S->abort_now = true;
                S->cv.notify_one();
                break;
            }
            std::this_thread::sleep_for(std::chrono::milliseconds(1));
        }
    }
    if (S->th.joinable()) S->th.join();
    const int32_t rc = S->loop_error;
    if (stats) *stats = S->stats;
    for (auto &t : S->tier)
        if (t.stream) cudaStreamSynchronize(t.stream);
    serve_free(S);
    delete S;
    eng->serve = nullptr;
    return rc;
}

}  // extern "C"

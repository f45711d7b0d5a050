/*
 * uastar_gpu.h — C ABI of the GB300 (sm_103a) GA*-style parallel A* engine.
 *
 * This is the drop-in boundary for uAstar's GPU solve path.  In the reference
 * that path sits behind class Problem (src/problem.hpp:6-24) and is reached
 * through GPUPathwaySolver (src/pathway/GPU-solver.hpp:20-36) and
 * gpusolver::GPUPuzzleSolver<N> (src/puzzle/GPU-solver.cuh:55-294), each with
 * initialize() / solve() -> bool / getSolution(cost*, vector<int>*).  Every
 * entry point below names the reference call it replaces.
 *
 * Conventions
 *  - Plain C types only: host pointers and sizes.  Inputs are caller-owned
 *    host buffers (copied to the device); all device memory is engine-owned.
 *  - Every int-returning call returns a UASTAR_* status; UASTAR_OK == 0.
 *    The reference ignores CUDA errors and calls exit(1); this ABI reports.
 *  - One engine per host thread.  The engine never resets the device (the
 *    reference's cudaDeviceReset() in initialize(), GPU-solver.cu:129-132,
 *    would destroy other users' state in a shared process).
 *  - Grid bitmaps: one bit per cell, row-major, cell id = x*W + y (the
 *    reference's toID, src/pathway/pathway.hpp:99-102), bit (id & 63) of
 *    little-endian word id >> 6, 1 = open.  An open cell may move in all 8
 *    directions, a blocked cell in none; the target of a move may be blocked
 *    (src/pathway/CPU-solver.cpp:98-104).  Straight moves cost 1, diagonal
 *    moves sqrt(2) (src/utils.hpp:119-122).
 *  - Puzzle boards: n*n bytes row-major, 0 = blank, goal = 1..n*n-1 with the
 *    blank last (src/puzzle/CPU-solver.hpp:145-151).  Moves are blank moves
 *    0..3 = (+1,0), (-1,0), (0,+1), (0,-1) in (row, column), the reference's
 *    DX/DY[0..3] (src/utils.hpp:120-121).
 */
#ifndef UASTAR_GPU_H
#define UASTAR_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
enum {
    UASTAR_OK = 0,
    UASTAR_NO_SOLUTION = 1,   /* open list exhausted: goal unreachable        */
    UASTAR_HEAP_OVERFLOW = 2, /* a per-thread heap is full                     */
    UASTAR_ARENA_FULL = 3,    /* path / node buffer too small                  */
    UASTAR_HASH_FULL = 4,     /* dedup table over its load limit / probe limit */
    UASTAR_ITER_LIMIT = 5,    /* round limit reached                           */
    UASTAR_CUDA_ERROR = 6,    /* a CUDA runtime call failed                    */
    UASTAR_BAD_INPUT = 7,     /* invalid argument                              */
    UASTAR_TIMEOUT = 8,       /* a bounded device-side wait expired            */
    UASTAR_RUNNING = 9,       /* (serving) request still in flight             */
    UASTAR_CANCELLED = 10,    /* (serving) request cancelled                   */
    UASTAR_REJECTED = 11      /* (serving) request exceeds the memory budget   */
};

/* ---- engine ---------------------------------------------------------- */
typedef struct uastar_engine uastar_engine;

typedef struct {
    int32_t heaps;           /* k parallel binary heaps of the plain engine (0 -> 8192 grid, 16384 puzzle) */
    int32_t block_threads;   /* CTA size of the plain engine's persistent kernel (0 -> 256) */
    int32_t heap_capacity;   /* entries per heap (0 -> auto, grown on overflow) */
    int32_t hash_log2_slots; /* dedup table = 2^n slots of 32 B, n <= 31 (0 -> sized from the instance and
                              grown 4x in place whenever it is half full) */
    double max_load;         /* dedup table load limit in (0,1) (0 -> 0.8) */
    int64_t max_rounds;      /* GA* round limit per solve (0 -> 2^31) */
    double wait_timeout_s;   /* bound on any device-side barrier wait (0 -> 10 s) */
    int32_t threads_per_heap; /* threads that share one heap's successors (0 -> 4) */
    int32_t heap_top_levels;  /* heap levels kept in shared memory (0 -> as many as fit, -1 -> none) */
    int32_t dedup;            /* removal of a round's duplicate grid successors: 0 -> the dedup
                                 table keeps the minimum g with a CAS loop (default); 1 -> the
                                 reference's order (src/pathway/GPU-solver.cu:218-235): the round's
                                 successors are radix-sorted by cell on the device and each cell's
                                 least-g record is relaxed once.  Same results; puzzles always use 0
                                 (the reference's puzzle kernel probes its table per successor) */
    int32_t exact_ms;         /* memory-bounded mode: time for its exact (IDA*) passes after the
                                 segments (0 -> 3000 ms, < 0 -> none) */
} uastar_config;

/* Replaces GPUPathwaySolver/GPUPuzzleSolver construction + initialize()'s
 * device setup (src/pathway/GPU-solver.cu:129-140, src/puzzle/GPU-solver.cuh:140-142);
 * `ordinal` is the reference's --ordinal flag (src/main.cpp:141).  cfg may be NULL. */
uastar_engine *uastar_create(int32_t ordinal, const uastar_config *cfg);
/* Replaces the solver destructors (GPU-solver.cu:106-127). */
void uastar_destroy(uastar_engine *eng);
/* Human-readable description of the last failure on this engine. */
const char *uastar_last_error(const uastar_engine *eng);
/* Launch the engine's work on an external CUDA stream (a cudaStream_t passed
 * as void*; NULL restores the engine's own stream). */
int32_t uastar_set_stream(uastar_engine *eng, void *cuda_stream);
/* Kernel launches this engine has issued so far (its own kernels only). */
int64_t uastar_kernel_launches(const uastar_engine *eng);
/* Name of this library build (architecture it was compiled for). */
const char *uastar_build_info(void);

/* Measurement aid (no counterpart in the reference): the latency floor of one
 * round of the plain engine's persistent kernel on its launch geometry (the
 * engine's heaps, block_threads and threads_per_heap).  us_barrier: rounds
 * of one team barrier only; us_cas_barrier: rounds of one 16-byte atomicCAS
 * per thread on a pseudo-random slot of a dedup table larger than L2 (values
 * left as they are; each thread's next slot depends on the CAS's result)
 * followed by the barrier.  Runs `rounds` (1 .. 2^20) rounds of each. */
int32_t uastar_round_floor(uastar_engine *eng, int32_t rounds, double *us_barrier, double *us_cas_barrier);

/* ---- grid pathfinding (--pathway) ------------------------------------- */
typedef struct {
    int32_t status;
    int32_t table_grows;  /* times the auto-sized dedup table grew in place */
    int64_t straight;     /* exact optimal cost = straight + diagonal*sqrt(2) */
    int64_t diagonal;
    float cost;           /* float32 g accumulated along the path in order, as the
                             reference computes it (CPU-solver.cpp:105) */
    float pad;
    double cost_exact;    /* straight + diagonal*sqrt(2) in double */
    int64_t expanded;     /* pops that were neither stale nor the goal */
    int64_t generated;    /* successors generated (dedup probes) */
    int64_t pushed;       /* heap pushes (new or improved nodes) */
    int64_t rounds;       /* GA* rounds */
    int64_t table_used;   /* dedup-table slots in use */
    int64_t path_len;     /* cells on the optimal path, start and goal included */
    double kernel_ms;     /* device time of the search kernel (CUDA events) */
    double solve_ms;      /* host wall time of the whole call */
} uastar_grid_result;

/* Upload a grid bitmap and keep it resident (replaces the graph H2D copy,
 * GPU-solver.cu:140).  words holds ceil(H*W/64) words; H*W < 2^31 (path
 * cell ids are int32, like the reference's vector<int>). */
int32_t uastar_grid_load(uastar_engine *eng, const uint64_t *words, int32_t H, int32_t W);
/* Solve on the resident grid (replaces GPUPathwaySolver::solve, GPU-solver.cu:180-328,
 * plus its kInitialize seeding, GPU-kernel.cuh:141-164). */
int32_t uastar_grid_solve_loaded(uastar_engine *eng, int32_t sx, int32_t sy, int32_t ex,
                                 int32_t ey, uastar_grid_result *out);
/* uastar_grid_load + uastar_grid_solve_loaded + path extraction in one call. */
int32_t uastar_grid_solve(uastar_engine *eng, const uint64_t *words, int32_t H, int32_t W,
                          int32_t sx, int32_t sy, int32_t ex, int32_t ey,
                          uastar_grid_result *out);
/* Path of the last successful grid solve, start -> goal (replaces
 * GPUPathwaySolver::getSolution + kFetchAnswer, GPU-solver.cu:330-354,
 * GPU-kernel.cuh:546-569).  Returns the path length (>= 0, may exceed cap,
 * only cap ids are written) or -status on failure. */
int64_t uastar_grid_path(uastar_engine *eng, int32_t *ids, int64_t cap);

/* The device sort of the sorted dedup mode (uastar_config.dedup = 1), which
 * replaces the reference's per-round MergesortPairs of the successor list
 * (src/pathway/GPU-solver.cu:218), run on its own: a stable LSD radix sort of
 * n 32-bit keys on key bits [0, key_bits) (0 -> 32; every key must be below
 * 2^key_bits) by the whole GPU as one team.  perm[j] = position of the j-th
 * smallest key, equal keys in position order.  0 <= n <= 2048 x SMs. */
int32_t uastar_sort_keys(uastar_engine *eng, const uint32_t *keys, int64_t n, int32_t key_bits,
                         uint32_t *perm);

/* ---- sliding-tile puzzle (--puzzle) ----------------------------------- */
typedef struct {
    int32_t status;
    int32_t steps;        /* optimal move count */
    int64_t expanded;
    int64_t generated;
    int64_t pushed;
    int64_t rounds;
    int64_t table_used;
    double kernel_ms;
    double solve_ms;
    int32_t table_grows;  /* times the auto-sized dedup table grew in place */
    int32_t reserved;
} uastar_puzzle_result;

/* Build the disjoint pattern databases of the n x n puzzle on the GPU by
 * backward breadth-first search and keep them resident (replaces
 * PatternDatabase::genDatabase, src/puzzle/database.cpp:37-84, called from
 * GPUPuzzleSolver::initialize, GPU-solver.cuh:130-138).  n = 3, 4 or 5.
 * Partitions: n=3 {1..8}; n=4 {1,2,3,4,5,6,9,13} + {7,8,10,11,12,14,15};
 * n=5 {3,4,5,10,15,20} + {2,1,6,11,16,21} + {7,8,9,12,17,22} +
 * {13,14,18,19,23,24} (src/puzzle/CPU-solver.hpp:43-102).  build_ms
 * (optional) gets the time. */
int32_t uastar_pdb_build(uastar_engine *eng, int32_t n, double *build_ms);
/* Bytes of the concatenated tables for n (362,880 for n=3; 576,576,000 for
 * n=4; 510,048,000 for n=5). */
int64_t uastar_pdb_bytes(int32_t n);
/* Upload tables from the host in the reference's concatenated layout (table
 * t at the sum of the sizes of tables < t, GPU-solver.cuh:130-138) — e.g. the
 * reference's database_<n>_<tiles>.bin cache files one after the other.
 * UASTAR_BAD_INPUT for a wrong size, or (n = 5) an entry above 127, the
 * largest value the 5x5 search carries per table (the reference's largest is 39). */
int32_t uastar_pdb_load(uastar_engine *eng, int32_t n, const uint8_t *tables, int64_t bytes);
/* Copy the resident tables back (for the on-disk cache and byte checks). */
int32_t uastar_pdb_fetch(uastar_engine *eng, int32_t n, uint8_t *out, int64_t bytes);
/* Solve one board (replaces GPUPuzzleSolver<N>::solve, GPU-solver.cuh:197-274).
 * n = 3, 4 or 5 (n*n bytes at tiles); the tables for n must be resident
 * (uastar_pdb_build or uastar_pdb_load).  5x5 boards use 16-byte state keys
 * (the reference's PuzzleStorage<5>, src/puzzle/storage.hpp:141-217, holds
 * one in two words too); the batched and serving engines take 3x3 and 4x4. */
int32_t uastar_puzzle_solve(uastar_engine *eng, int32_t n, const uint8_t *tiles,
                            uastar_puzzle_result *out);
/* Blank moves of the last puzzle solve, start -> goal (replaces
 * GPUPuzzleSolver::getSolution + kFetchAnswer, GPU-solver.cuh:276-287,
 * GPU-kernel.cuh:462-509).  Returns the move count or -status. */
int64_t uastar_puzzle_moves(uastar_engine *eng, int32_t *moves, int64_t cap);

/* Memory-bounded solve for puzzles too large for the dedup table (the
 * reference's README.md:30-34 describes such a mode; it has no code for it).
 * Phase 1 runs segments of exact GA* with the table capped at
 * 2^max_log2_slots slots (32 B each).  A segment that fills the table pauses;
 * the open list's minimum f is then a lower bound on the remaining optimum,
 * the search commits to the open node holding it and the next segment starts
 * there; one segment means the solution is optimal.  Phase 2, when phase 1
 * took more than one segment, runs iterative-deepening A* passes (depth-first
 * search below a threshold on f, memory proportional to the depth, not to the
 * table) from the first segment's bound upward, for at most uastar_config.
 * exact_ms: a pass that finds a goal returns an optimal solution (steps =
 * lower_bound, exact_optimal = 1); a pass that completes without one raises
 * the bound; reaching phase 1's length proves that solution optimal.  The
 * heuristic stays admissible throughout.  Moves via uastar_puzzle_moves. */
typedef struct {
    int32_t status;
    int32_t steps;            /* moves of the returned solution */
    int32_t lower_bound;      /* proven lower bound on the optimal move count (= steps: optimal) */
    int32_t segments;         /* table-capped GA* segments run; 1 = that solution is optimal */
    int64_t expanded;
    int64_t generated;
    double kernel_ms;
    double solve_ms;
    int32_t exact_passes;     /* IDA* threshold passes run after the segments */
    int32_t exact_optimal;    /* 1 if the passes proved the returned solution optimal */
    int64_t exact_nodes;      /* nodes the passes generated */
    double exact_ms;          /* their time */
} uastar_bounded_result;

int32_t uastar_puzzle_solve_bounded(uastar_engine *eng, int32_t n, const uint8_t *tiles, int32_t max_log2_slots,
                                    uastar_bounded_result *out);

/* ---- batched persistent engine (many instances per launch) ----------- */
enum { UASTAR_KIND_GRID = 1, UASTAR_KIND_PUZZLE = 2 };

typedef struct {
    int32_t kind;             /* UASTAR_KIND_GRID or UASTAR_KIND_PUZZLE */
    int32_t n;                /* puzzle side (3 or 4) */
    int32_t H, W, sx, sy, ex, ey; /* grid */
    const uint64_t *words;    /* grid bitmap (host, caller-owned) */
    uint8_t tiles[16];        /* puzzle board */
    int64_t est_nodes;        /* optional size hint for the dedup partition (0 = auto) */
} uastar_instance;

typedef struct {
    int32_t status;
    int32_t steps;            /* puzzle: optimal move count */
    int64_t straight;         /* grid: exact optimal cost pair */
    int64_t diagonal;
    float cost;               /* grid float cost (straight + diagonal*sqrt2 in float) */
    float pad;
    int64_t expanded;
    int64_t generated;
    int64_t rounds;
    int32_t attempts;         /* 1 + retries with a larger partition */
    int32_t migrations;       /* serving: moves to a cluster slot with the search state kept */
    double latency_ms;        /* serving: completion - arrival; batch: completion - launch */
    double device_ms;         /* device time of the last attempt's search (CTA team) */
    double start_ms;          /* batch: device start of the last attempt, from its wave's first start */
} uastar_instance_result;

typedef struct {
    int32_t threads_per_instance; /* CTA size per instance (0 -> 256) */
    int32_t threads_per_heap;     /* heaps per instance = threads_per_instance / this (0 -> 4) */
    int32_t heap_capacity;        /* entries per heap (0 -> 4095; uastar_autotune picks one) */
    double load_factor;           /* target dedup-partition load (0 -> 0.5; uastar_autotune picks one) */
    int32_t ctas;                 /* persistent CTAs (0 -> all SMs x occupancy) */
    int32_t use_graph;            /* launch through a captured CUDA graph (default 1) */
    int32_t tier1_rounds;         /* round budget of a single-CTA team (0 -> 2048) */
    int32_t tier2_puzzle_rounds;  /* round budget of a puzzle on a cluster team (0 -> 16384) */
    int32_t cluster_size;         /* CTAs per cluster team (0 -> 8; 2..16) */
    int32_t reserved;
} uastar_batch_config;

typedef struct {
    double wall_ms;           /* whole batch, host wall clock */
    double kernel_ms;         /* device time of the persistent kernel(s) */
    int64_t expanded;
    int64_t generated;
    int32_t waves;            /* launches (1 + retry waves) */
    int32_t escalated;        /* instances re-solved by the plain engine */
    int32_t ctas;
    int32_t threads_per_instance;
    int32_t heap_capacity;
    double load_factor;
    int64_t partition_bytes;  /* device bytes of all dedup partitions */
} uastar_batch_stats;

/* Solve `count` instances of mixed kinds with persistent launches: in the
 * first wave each CTA takes instances from a device work queue and runs GA*
 * on one with its own heap slice and dedup partition, under a round budget
 * (tier1_rounds); grids above 2048^2 and the instances that ran out of rounds
 * or space go to a second wave of 8-CTA cluster teams with 16x the
 * partition (puzzles under tier2_puzzle_rounds), and what fails there is
 * solved by the plain engine, one instance at a time.  No counterpart in the
 * reference, which solves one instance per process through
 * GPUPathwaySolver / GPUPuzzleSolver. */
int32_t uastar_batch_solve(uastar_engine *eng, const uastar_instance *insts, int32_t count,
                           const uastar_batch_config *cfg, uastar_instance_result *results,
                           uastar_batch_stats *stats);
/* Pick the batch geometry for a workload by timing configurations on a
 * sample of it: one pass of coordinate descent from the defaults over
 * threads_per_instance {128, 256, 512}, threads_per_heap {2, 4, 8} (heaps per
 * instance = their quotient), heap_capacity {1023, 4095, 16383},
 * load_factor {0.35, 0.5, 0.7}, cluster_size {4, 8, 16}, tier1_rounds
 * {1024, 2048, 4096} and tier2_puzzle_rounds {4096, 16384, 65536}, each knob
 * taking the value of least wall time with
 * the others held.  Writes the choice; best->reserved = configurations timed.
 * Replaces the reference's compile-time sizes (src/pathway/GPU-solver.hpp:6-17,
 * src/puzzle/GPU-solver.cuh:11-20). */
int32_t uastar_autotune(uastar_engine *eng, const uastar_instance *sample, int32_t count,
                        uastar_batch_config *best);

/* ---- serving loop (continuous batching) ------------------------------- */
typedef struct {
    double hbm_budget_gb;     /* admission budget for heaps + dedup partitions (default 120) */
    int32_t slots;            /* max concurrently resident requests (0 -> all CTAs) */
    int32_t threads_per_instance; /* threads of a CTA slot (0 -> 256) */
    int32_t threads_per_heap; /* 0 -> 2: 128 heaps per CTA slot (a resident search's rounds are
                                 its latency; more pops per round shorten it) */
    int32_t heap_capacity;    /* entries per heap of a CTA slot (0 -> 16383, 4095 where the budget's
                                 heap share cannot hold one slot of those; 4x on overflow) */
    int32_t rounds_per_quantum; /* cap on GA* rounds per persistent-kernel launch (0 -> 65536 with
                                   a time slice, 256 without) */
    double load_factor;
    int32_t cluster_slots;    /* cap on 8-CTA slots for requests whose search outgrows one CTA
                                 (0 -> as many as fit, -1 -> none) */
    int32_t quantum_us;       /* time slice of a persistent-kernel launch: every resident search
                                 runs rounds until this many microseconds have passed since the
                                 launch began, so that fast and slow searches share the GPU's time
                                 rather than a round count (0 -> 8000; < 0 -> none, rounds only) */
} uastar_serve_config;

typedef struct {
    int64_t id;
    uastar_instance_result result;
} uastar_serve_completion;

typedef struct {
    int64_t submitted, completed, rejected, cancelled;
    int64_t quanta;           /* persistent-kernel launches */
    double busy_ms;           /* device time spent in quanta */
    double peak_budget_gb;    /* peak admitted device bytes */
    int32_t peak_resident;
    int32_t reserved;
} uastar_serve_stats;

/* Start the serving loop: a host thread that admits submitted requests by
 * their estimated heap + dedup-partition bytes against the budget, keeps each
 * request's search state resident on the device between persistent-kernel
 * quanta, retires finished requests and backfills new ones. */
int32_t uastar_serve_start(uastar_engine *eng, const uastar_serve_config *cfg);
/* Queue a request (the bitmap is copied before return).  arrival_s is the
 * request's arrival time on the CLOCK_MONOTONIC clock in seconds (0 = now),
 * used for latency.  Returns a request id >= 0 or -status. */
int64_t uastar_serve_submit(uastar_engine *eng, const uastar_instance *inst, double arrival_s);
/* Retrieve up to cap completions (non-blocking).  Returns the count. */
int32_t uastar_serve_poll(uastar_engine *eng, uastar_serve_completion *out, int32_t cap);
/* Cancel a queued or resident request. */
int32_t uastar_serve_cancel(uastar_engine *eng, int64_t id);
/* Wait until every submitted request completed (timeout_s bound), then stop. */
int32_t uastar_serve_stop(uastar_engine *eng, double timeout_s, uastar_serve_stats *stats);
/* CLOCK_MONOTONIC now, seconds (the clock serve_submit's arrival_s uses). */
double uastar_now_s(void);

/* ---- allocation-free grid solve ---------------------------------------- */
/* No counterpart in the reference.  For callers that may not allocate device
 * memory while they run (a plugin inside another framework's memory pool, a
 * real-time or graph-replayed loop, an allocator-free service): the same GA*
 * search as uastar_grid_solve, run out of one fixed device array the library
 * reserves at load time (about 53 MB on every GPU that loads it, held until
 * the process exits), so the call allocates nothing.  The caller passes device
 * buffers: the bitmap (layout as above), a path buffer of path_cap cell ids
 * and a result record; the call is asynchronous on `stream` (a cudaStream_t
 * as void*, NULL = the default stream) and the result is valid once the
 * stream has finished.  The first call on a device looks up the array's
 * device address: make it outside any stream capture.  Grids above 2^22
 * cells are rejected with UASTAR_BAD_INPUT; a search that outgrows the array
 * (2^20 dedup slots at 80 % load, 256 heaps of 4095 entries) reports
 * UASTAR_HASH_FULL or UASTAR_HEAP_OVERFLOW in the result, a path longer than
 * path_cap UASTAR_ARENA_FULL (path_len 0), and a team-barrier wait that
 * exceeds 10 s UASTAR_TIMEOUT.  A return value other than UASTAR_OK means
 * nothing was queued that writes the result record; an error still pending
 * from the caller's earlier CUDA work is returned as UASTAR_CUDA_ERROR and
 * left pending.  The array's address is looked up once per device and kept:
 * do not call this again in a process after cudaDeviceReset.  All calls share
 * the array: calls that overlap on the GPU race, so serialize them. */
typedef struct {
    int32_t status;
    int32_t reserved;
    int64_t straight;
    int64_t diagonal;
    int64_t expanded;
    int64_t generated;
    int64_t rounds;
    int64_t path_len;         /* cells written to the path buffer, start -> goal */
} uastar_noalloc_grid_result;

int32_t uastar_grid_solve_noalloc(const uint64_t *d_words, int32_t H, int32_t W, int32_t sx, int32_t sy,
                                  int32_t ex, int32_t ey, int32_t *d_path, int64_t path_cap,
                                  uastar_noalloc_grid_result *d_result, void *stream);

/* ---- host utilities: instance generators and path validation ---------- */
/* Seeded Bernoulli grid: cell id is blocked iff the top 32 bits of output #id
 * of the splitmix64 stream seeded with `seed` fall below
 * floor(block_rate * 2^32); the cells (sx,sy) and (ex,ey) are forced open.
 * Writes ceil(H*W/64) words. */
int32_t uastar_gen_grid(uint64_t seed, int32_t H, int32_t W, double block_rate, int32_t sx,
                        int32_t sy, int32_t ex, int32_t ey, uint64_t *words);
/* Seeded random walk of walk_len blank moves from the goal, never undoing
 * the previous move: step i picks candidate floor(r * c / 2^32) of the c
 * legal moves in 0..3 order, r = top 32 bits of splitmix64 output #i.
 * Writes n*n tiles (n = 2..4). */
int32_t uastar_gen_puzzle(uint64_t seed, int32_t n, int32_t walk_len, uint8_t *tiles);
/* Zig-zag maze of the reference's `zigzag` input module
 * (src/pathway/input/zigzag.cpp:14-40); writes words and the endpoints. */
int32_t uastar_gen_zigzag(int32_t H, int32_t W, int32_t height_gap, uint64_t *words,
                          int32_t *sx, int32_t *sy, int32_t *ex, int32_t *ey);
/* 1 if the goal is reachable under the move rules above, 0 if not. */
int32_t uastar_grid_reachable(const uint64_t *words, int32_t H, int32_t W, int32_t sx,
                              int32_t sy, int32_t ex, int32_t ey);
/* Cheap screen for large seeded grids: a forward search from the start and a
 * backward search from the goal, each bounded to `limit` cells.  Returns 1 if
 * the goal is proven reachable, 0 if proven unreachable (one side exhausted
 * its component), 2 if both searches outgrew the bound (presumed reachable). */
int32_t uastar_grid_screen(const uint64_t *words, int32_t H, int32_t W, int32_t sx, int32_t sy,
                           int32_t ex, int32_t ey, int64_t limit);
/* Re-validate a grid path on the host: consecutive cells are 8-neighbours,
 * every move leaves an open cell, the path runs start -> goal.  Writes the
 * replayed straight/diagonal counts and the float32 cost accumulated in
 * path order.  Returns UASTAR_OK or UASTAR_BAD_INPUT. */
int32_t uastar_validate_grid_path(const uint64_t *words, int32_t H, int32_t W, int32_t sx,
                                  int32_t sy, int32_t ex, int32_t ey, const int32_t *ids,
                                  int64_t len, int64_t *straight, int64_t *diagonal,
                                  float *cost);
/* Re-validate puzzle moves: every move is legal and the board ends at the
 * goal.  Returns UASTAR_OK or UASTAR_BAD_INPUT. */
int32_t uastar_validate_puzzle_moves(int32_t n, const uint8_t *tiles, const int32_t *moves,
                                     int64_t len);

#ifdef __cplusplus
}
#endif
#endif /* UASTAR_GPU_H */

// Device-side building blocks of the GA* engine (sm_103a):
//   - the dedup-table slot and successor-candidate records,
//   - the per-search team state,
//   - L2-coherent loads, 64-bit hashing, open-addressed find-or-insert with
//     atomicCAS, CAS-based minimum of a cost word,
//   - a grid-wide barrier whose every wait is bounded in time.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace uastar {

constexpr uint64_t kEmptyKey = ~0ull;   // free dedup slot (no valid state packs to all ones)
constexpr uint64_t kInfCost = ~0ull;    // "no cost yet"
constexpr uint32_t kNone = 0xFFFFFFFFu; // null slot index
constexpr unsigned kFull = 0xFFFFFFFFu; // full warp mask

// Status codes (mirror UASTAR_* in include/uastar_gpu.h).
enum : uint32_t {
    ST_OK = 0,
    ST_NO_SOLUTION = 1,
    ST_HEAP_OVERFLOW = 2,
    ST_ARENA_FULL = 3,
    ST_HASH_FULL = 4,
    ST_ITER_LIMIT = 5,
    ST_CUDA_ERROR = 6,
    ST_BAD_INPUT = 7,
    ST_TIMEOUT = 8,
    ST_RUNNING = 9,
};

// One dedup-table slot: exactly one 32-byte sector, so a probe, the g update
// and the pop-time read of a node each touch a single sector.
struct __align__(32) Slot {
    unsigned long long key;  // state key (grid cell id / packed board); kEmptyKey = free
    unsigned long long g;    // cost from the start (problem-specific packing)
    uint32_t aux;            // problem data (puzzle: PDB parts and last move)
    uint32_t prev;           // parent slot, kNone for the root
    uint32_t pad0, pad1;
};
static_assert(sizeof(Slot) == 32, "slot must be one sector");

// Slot access by key width.  Narrow keys (grid cells, boards of up to 16
// cells in 4-bit fields) use the layout above; wide keys (a 5x5 board: 24
// cells in 5-bit fields, the 25th implied) read the same 32 bytes as
// {key lo, key hi, g, aux, prev}: the 16-byte key is claimed with one
// 16-byte CAS and g is lowered with its own 8-byte CAS.
struct Key128 {
    unsigned long long lo, hi;
};
struct __align__(32) WideSlot {
    unsigned long long lo, hi, g;
    uint32_t aux, prev;
};
static_assert(sizeof(WideSlot) == 32, "wide slot must be one sector");

// Where a slot keeps its parent link: its own field, written after the
// round's barrier by the candidate that won the slot; the key word (grids:
// cell | prev << 32); or the g word (narrow puzzle keys: g << 40 | (last
// move + 1) << 32 | prev).  In the key or the g word the link is set by the
// same 16-byte CAS that sets g, so the push phase checks no winner.
enum SlotLink : int { LINK_FIELD = 0, LINK_IN_KEY = 1, LINK_IN_G = 2 };

struct NarrowSlots {
    using Key = uint64_t;
    static constexpr bool kWide = false;
    static constexpr bool kPrevInKey = false;  // see GridProblem
    static constexpr int kLink = LINK_FIELD;
    // the g word that the relax CAS installs, and its cost
    __device__ static uint64_t g_word(uint64_t g, uint32_t, int) { return g; }
    __device__ static uint64_t word_g(uint64_t w) { return w; }
    __device__ static uint64_t slot_g(const Slot *s) { return __ldcg(&s->g); }
    __device__ static uint32_t slot_prev(const Slot *s) { return __ldcg(&s->prev); }
    __device__ static void set_link(Slot *s, uint32_t prev, uint32_t aux) {
        s->prev = prev;
        s->aux = aux;
    }
};
struct WideSlots {
    using Key = Key128;
    static constexpr bool kWide = true;
    static constexpr bool kPrevInKey = false;
    static constexpr int kLink = LINK_FIELD;
    __device__ static const WideSlot *w(const Slot *s) { return reinterpret_cast<const WideSlot *>(s); }
    __device__ static WideSlot *w(Slot *s) { return reinterpret_cast<WideSlot *>(s); }
    __device__ static uint64_t slot_g(const Slot *s) { return __ldcg(&w(s)->g); }
    __device__ static uint32_t slot_prev(const Slot *s) { return __ldcg(&w(s)->prev); }
    __device__ static void set_link(Slot *s, uint32_t prev, uint32_t aux) {
        w(s)->prev = prev;
        w(s)->aux = aux;
    }
};

// Key and parent link of a narrow slot (`link`: a SlotLink).  For the path
// walkers.
__device__ __forceinline__ void slot_key_prev(const Slot *s, int link, uint64_t &key, uint32_t &prev) {
    const uint64_t w = __ldcg(&s->key);
    if (link == LINK_IN_KEY) {
        key = w & 0xffffffffull;
        prev = (uint32_t)(w >> 32);
    } else {
        key = w;
        prev = link == LINK_IN_G ? (uint32_t)__ldcg(&s->g) : __ldcg(&s->prev);
    }
}

// A successor whose g strictly improved its slot this round.
struct __align__(16) Cand {
    uint32_t slot;
    uint32_t parent;
    unsigned long long g;
    unsigned long long f;
    uint32_t aux;
    uint32_t pad;
};
static_assert(sizeof(Cand) == 32, "candidate record");

// Search state shared by the threads of one GA* team (the whole grid for the
// plain engine, one CTA or cluster for the batched engine).  A round has one
// team barrier, between its relax phase and its decision; the push phase of
// round r may still run on one CTA while another is in round r + 1.  So the
// per-round fields are indexed by round % 3: round r writes its own entry,
// every CTA reads it after round r's barrier, and CTA 0 clears the entry of
// round r + 2 during round r's push phase (by then every CTA has read round
// r - 1's entry, and round r + 2 cannot start before CTA 0 finishes).
struct __align__(16) TeamState {
    unsigned long long round_min[3];  // min popped f of the round (cost word)
    unsigned long long goal_min[3];   // min goal f popped in the round
    unsigned long long ins[3];        // dedup slots claimed in the round
    uint32_t err[3];                  // first error of the round's relax phase
    uint32_t pad0_;
    uint32_t quit[3];                 // the round ended past the search's time slice (SearchMem::deadline_ns)
    uint32_t pad1_;
    // totals, stored by CTA 0 when the search stops or pauses
    unsigned long long goal_best;     // best goal f popped so far
    unsigned long long round;         // rounds completed
    unsigned long long inserted;      // dedup slots in use
    unsigned long long expanded, generated, pushed;
    uint32_t goal_slot;
    uint32_t error;                   // fatal error: barrier timeout, start node not inserted,
                                      // heap overflow while parking the insertion buffers
    uint32_t status;                  // final status (ST_RUNNING while active)
    uint32_t base;                    // heap rotation for pushes
    uint32_t started;                 // start node seeded
    uint32_t barrier;                 // grid-barrier arrival counter
};

// A fresh team: nothing popped, no goal, no errors.
__host__ __device__ inline void team_state_init(TeamState *s) {
    unsigned char *b = reinterpret_cast<unsigned char *>(s);
    for (unsigned i = 0; i < sizeof(TeamState); ++i) b[i] = 0;
    for (int i = 0; i < 3; ++i) s->round_min[i] = s->goal_min[i] = kInfCost;
    s->goal_best = kInfCost;
    s->goal_slot = kNone;
    s->status = ST_RUNNING;
}

// ---------------------------------------------------------------- loads ---
// Cross-SM mutable data is read through L2 (ld.global.cg): L1 is not coherent
// across SMs, and the table, heaps and candidates move between SMs every round.
__device__ __forceinline__ unsigned long long ldcg_u64(const unsigned long long *p) {
    return __ldcg(p);
}
__device__ __forceinline__ uint32_t ldcg_u32(const uint32_t *p) { return __ldcg(p); }

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void set_error(uint32_t *err, uint32_t code) {
    atomicCAS(err, 0u, code);
}

// ------------------------------------------------------------- hashing ---
// 64-bit finalizer of MurmurHash3 (Appleby, public domain): a bijective mix
// whose low bits depend on every key bit.
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

__host__ __device__ __forceinline__ uint64_t key_hash(uint64_t k) { return mix64(k); }
__host__ __device__ __forceinline__ uint64_t key_hash(const Key128 &k) { return mix64(k.lo ^ mix64(k.hi)); }

enum : int { FIND_FOUND = 0, FIND_INSERTED = 1, FIND_FULL = 2 };

// Open addressing with linear probing over 32-byte slots.  A free slot is
// claimed with atomicCAS on its key; the winner of the race owns it and every
// other writer of the same key sees the key on its retry.
__device__ __forceinline__ int find_or_insert(Slot *tab, uint64_t mask, uint64_t key,
                                              uint32_t max_probe, uint32_t *slot_out) {
    uint64_t h = mix64(key) & mask;
    for (uint32_t i = 0; i < max_probe; ++i) {
        unsigned long long k = ldcg_u64(&tab[h].key);
        if (k == key) {
            *slot_out = (uint32_t)h;
            return FIND_FOUND;
        }
        if (k == kEmptyKey) {
            unsigned long long old = atomicCAS(&tab[h].key, kEmptyKey, (unsigned long long)key);
            if (old == kEmptyKey) {
                *slot_out = (uint32_t)h;
                return FIND_INSERTED;
            }
            if (old == key) {
                *slot_out = (uint32_t)h;
                return FIND_FOUND;
            }
        }
        h = (h + 1) & mask;
    }
    return FIND_FULL;
}

// ------------------------------------------------------- warp helpers ---
__device__ __forceinline__ uint64_t shfl64(uint64_t v, int src) {
    return __shfl_sync(kFull, (unsigned long long)v, src);
}
__device__ __forceinline__ uint64_t shfl_xor64(uint64_t v, int m) {
    return __shfl_xor_sync(kFull, (unsigned long long)v, m);
}
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ------------------------------------------------------------- barrier ---
// Grid-wide barrier for a cooperative launch.  The arrival counter only grows
// (one release add per CTA per barrier, no reset), so barrier number e is
// complete when the counter reaches e * nblocks (compared modulo 2^32).
// Thread 0 of each CTA waits with a time bound: when it expires, or when
// another CTA has flagged an error, it records ST_TIMEOUT (first error wins)
// and leaves; the caller checks the error word after every barrier, so all
// CTAs stop together at the next one.
__device__ __forceinline__ void grid_barrier(uint32_t *counter, uint32_t nblocks, uint32_t &epoch,
                                             uint32_t *err, uint64_t timeout_ns) {
    __syncthreads();
    if (threadIdx.x == 0) {
        epoch += 1;
        const uint32_t target = epoch * nblocks;
        // release at GPU scope: cumulative over the CTA's writes, which the
        // CTA barrier above ordered before this thread's arrival
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(counter) : "memory");
        const uint64_t t0 = globaltimer_ns();
        uint32_t spins = 0;
        while ((int32_t)(ld_acquire_u32(counter) - target) < 0) {
            if ((++spins & 63u) == 0) {
                if (ldcg_u32(err) != 0) break;
                if (globaltimer_ns() - t0 > timeout_ns) {
                    set_error(err, ST_TIMEOUT);
                    break;
                }
            }
        }
        // the acquire load that saw the last arrival orders this thread after
        // every CTA's release; the CTA barrier below carries that to the rest
    }
    __syncthreads();
}

}  // namespace uastar

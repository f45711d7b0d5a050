// The GA* round loop, generic over the problem (grid / puzzle) and the team
// that runs it (the whole cooperative grid for one large instance, or one
// CTA per instance in the batched and serving engines).
//
// Each team thread owns one binary min-heap for popping.  A round is:
//
//   phase 1  every thread pops the minimum of its own heap; the team's
//            minimum popped f is reduced (warp shuffles, one CAS per warp);
//            stale entries (f no longer matching the node's g) are dropped;
//            a goal pop lowers goal_best; every other pop is expanded.
//            The warp then spreads all successors of its 32 pops evenly over
//            its lanes; each lane finds-or-inserts its successor in the
//            open-addressed dedup table (atomicCAS on the key) and lowers the
//            slot's g with a CAS loop.  Only a strict improvement makes the
//            successor a candidate, so among equal-g writers of one slot in a
//            round exactly one candidate carries the final g.
//   barrier  then a uniform decision: stop when goal_best <= the round's
//            minimum popped f (the GA* optimality test of the reference,
//            src/pathway/GPU-solver.cu:219-243), fail when nothing was popped.
//   phase 2  candidates are pushed round-robin over all heaps; a candidate is
//            the slot's winner iff the slot's g still equals its g, and only
//            the winner writes prev/aux and pushes.
//   barrier
//
// This replaces the reference's per-round kExtractExpand -> host copy ->
// MergesortPairs -> kAssign -> host copy -> kDeduplicate -> kHeapInsert
// chain (src/pathway/GPU-solver.cu:180-328) with one persistent kernel and
// no host round trip: the per-round sort + unique of the successor list is
// replaced by the table's atomic minimum (same result: the minimum g per
// state among this round's successors and the stored node).
#pragma once
#include <cstdint>

#include "ga_device.cuh"

namespace uastar {

template <class E> struct SearchMem {
    Slot *tab;
    uint64_t mask;          // slots - 1 (power of two)
    uint64_t max_inserted;  // load limit
    uint32_t max_probe;
    E *heaps;               // team.size() heaps of `stride` entries; index 0 unused
    uint32_t stride;
    uint32_t *heap_size;
    Cand *cand;             // >= team.size() * kMoves records
    uint64_t max_rounds;    // absolute round limit (ITER_LIMIT)
};

// ------------------------------------------------------------------ teams ---
struct GridTeam {
    TeamState *st;  // global memory
    uint32_t epoch;
    uint64_t timeout_ns;
    __device__ uint32_t rank() const { return blockIdx.x * blockDim.x + threadIdx.x; }
    __device__ uint32_t size() const { return gridDim.x * blockDim.x; }
    __device__ void sync() { grid_barrier(&st->barrier, gridDim.x, epoch, &st->error, timeout_ns); }
    __device__ uint64_t rd64(const unsigned long long *p) const { return ldcg_u64(p); }
    __device__ uint32_t rd32(const uint32_t *p) const { return ldcg_u32(p); }
};

struct BlockTeam {
    TeamState *st;  // shared memory
    __device__ uint32_t rank() const { return threadIdx.x; }
    __device__ uint32_t size() const { return blockDim.x; }
    __device__ void sync() { __syncthreads(); }
    __device__ uint64_t rd64(const unsigned long long *p) const {
        return *reinterpret_cast<const volatile unsigned long long *>(p);
    }
    __device__ uint32_t rd32(const uint32_t *p) const {
        return *reinterpret_cast<const volatile uint32_t *>(p);
    }
};

// ------------------------------------------------------------------ heaps ---
// 1-indexed binary heap in global memory; the two children 2i, 2i+1 of a
// node are adjacent (one 32-byte sector for 16-byte entries).
template <class P>
__device__ __forceinline__ bool heap_pop(typename P::Entry *hp, uint32_t &size,
                                         typename P::Entry &out) {
    using E = typename P::Entry;
    if (size == 0) return false;
    out = P::load(hp + 1);
    const E last = P::load(hp + size);
    size -= 1;
    if (size == 0) return true;
    uint32_t now = 1;
    for (;;) {
        uint32_t c = now << 1;
        if (c > size) break;
        E a = P::load(hp + c);
        if (c < size) {
            const E b = P::load(hp + c + 1);
            if (P::less(b, a)) {
                a = b;
                ++c;
            }
        }
        if (!P::less(a, last)) break;
        P::store(hp + now, a);
        now = c;
    }
    P::store(hp + now, last);
    return true;
}

template <class P>
__device__ __forceinline__ void heap_push(typename P::Entry *hp, uint32_t &size,
                                          const typename P::Entry &v) {
    using E = typename P::Entry;
    uint32_t now = ++size;
    while (now > 1) {
        const uint32_t par = now >> 1;
        const E pv = P::load(hp + par);
        if (!P::less(v, pv)) break;
        P::store(hp + now, pv);
        now = par;
    }
    P::store(hp + now, v);
}

// ---------------------------------------------------------- cost minima ---
template <class P> __device__ __forceinline__ uint64_t warp_min_cost(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t w = shfl_xor64(v, o);
        if (P::cost_cmp(w, v) < 0) v = w;
    }
    return v;
}

// Lower *addr to v (in P's cost order).  Starts from the guess "unset" so that
// the first CAS either installs v or returns the current value.  Returns true
// iff this call strictly lowered the word.
template <class P>
__device__ __forceinline__ bool atomic_min_cost(unsigned long long *addr, uint64_t v) {
    unsigned long long cur = kInfCost;
    while (P::cost_cmp(v, cur) < 0) {
        const unsigned long long old = atomicCAS(addr, cur, (unsigned long long)v);
        if (old == cur) return true;
        cur = old;
    }
    return false;
}

__device__ __forceinline__ Cand load_cand(const Cand *p) {
    const uint4 a = __ldcg(reinterpret_cast<const uint4 *>(p));
    const uint4 b = __ldcg(reinterpret_cast<const uint4 *>(p) + 1);
    Cand c;
    c.slot = a.x;
    c.parent = a.y;
    c.g = ((unsigned long long)a.w << 32) | a.z;
    c.f = ((unsigned long long)b.y << 32) | b.x;
    c.aux = b.z;
    c.pad = b.w;
    return c;
}

// ------------------------------------------------------------ the search ---
// Runs up to `budget` rounds (resumable: state lives in TeamState, the heaps
// and the table).  Returns ST_RUNNING if the budget ran out first, else the
// final status.  Every team thread must call it.
template <class P, class Team>
__device__ uint32_t ga_search(const P &prob, Team &team, const SearchMem<typename P::Entry> &m,
                              uint64_t budget) {
    using E = typename P::Entry;
    TeamState *st = team.st;
    const uint32_t k = team.size(), rank = team.rank();
    const uint32_t lane = threadIdx.x & 31u;
    uint64_t nE = 0, nS = 0, nP = 0;

    if (team.rd32(&st->started) == 0) {
        if (rank == 0) {
            const uint64_t key0 = prob.start_key();
            uint32_t s0;
            if (find_or_insert(m.tab, m.mask, key0, m.max_probe, &s0) == FIND_FULL) {
                set_error(&st->error, ST_HASH_FULL);
            } else {
                const uint32_t aux0 = prob.start_aux();
                m.tab[s0].g = 0;
                m.tab[s0].aux = aux0;
                m.tab[s0].prev = kNone;
                uint32_t sz = 0;
                heap_push<P>(m.heaps, sz, prob.make_entry(prob.f_of(key0, 0, aux0), 0, s0));
                m.heap_size[0] = sz;
                st->inserted = 1;
            }
            st->started = 1;
        }
        team.sync();
    }

    uint32_t base = team.rd32(&st->base);
    uint64_t round = team.rd64(&st->round);
    uint32_t status = ST_RUNNING;
    E *const myheap = m.heaps + (size_t)rank * m.stride;

    for (uint64_t it = 0;; ++it) {
        const uint32_t par = (uint32_t)(round & 1);

        // ---------------------------------------------------- phase 1 ---
        E e;
        uint32_t hs = ldcg_u32(&m.heap_size[rank]);
        bool have = false;
        if (hs) {
            have = heap_pop<P>(myheap, hs, e);
            m.heap_size[rank] = hs;
        }
        const uint64_t ecost = have ? P::entry_cost(e) : kInfCost;
        const uint64_t wmin = warp_min_cost<P>(ecost);
        if (lane == 0 && wmin != kInfCost) atomic_min_cost<P>(&st->round_min[par], wmin);

        uint64_t key = 0, g = 0;
        uint32_t aux = 0, pslot = 0, mv = 0;
        if (have) {
            pslot = e.slot;
            P::load_node(m.tab + pslot, key, g, aux);
            const uint64_t fcur = prob.f_of(key, g, aux);
            if (fcur != ecost) {
                // stale: the node was improved after this entry was pushed
            } else if (prob.is_goal(key)) {
                atomic_min_cost<P>(&st->goal_best, fcur);
                st->goal_slot = pslot;  // every goal pop names the same slot
            } else {
                ++nE;
                mv = prob.moves(key, aux);
            }
        }

        // Spread the warp's successors over its lanes.
        const uint32_t cnt = __popc(mv);
        uint32_t incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(kFull, incl, o);
            if (lane >= (uint32_t)o) incl += t;
        }
        const uint32_t total = __shfl_sync(kFull, incl, 31);
        const uint32_t excl = incl - cnt;
        for (uint32_t b0 = 0; b0 < total; b0 += 32) {
            const uint32_t j = b0 + lane;
            // owner = largest lane whose exclusive prefix is <= j (it has cnt > 0)
            uint32_t owner = 0;
#pragma unroll
            for (int s = 16; s > 0; s >>= 1) {
                const uint32_t ex = __shfl_sync(kFull, excl, owner + s);
                if (ex <= j) owner += s;
            }
            const uint32_t kth = j - __shfl_sync(kFull, excl, owner);
            const uint32_t omask = __shfl_sync(kFull, mv, owner);
            const uint64_t okey = shfl64(key, owner), og = shfl64(g, owner);
            const uint32_t oaux = __shfl_sync(kFull, aux, owner);
            const uint32_t oslot = __shfl_sync(kFull, pslot, owner);
            bool improved = false, inserted = false;
            uint32_t nslot = 0, naux = 0;
            uint64_t ng = 0, nf = 0;
            if (j < total) {
                const int move = (int)__fns(omask, 0, (int)kth + 1);
                uint64_t nkey;
                prob.apply(okey, og, oaux, move, nkey, ng, naux, nf);
                ++nS;
                const int r = find_or_insert(m.tab, m.mask, nkey, m.max_probe, &nslot);
                if (r == FIND_FULL) {
                    set_error(&st->error, ST_HASH_FULL);
                } else {
                    inserted = (r == FIND_INSERTED);
                    improved = atomic_min_cost<P>(&m.tab[nslot].g, ng);
                }
            }
            const uint32_t ib = __ballot_sync(kFull, inserted);
            if (ib && lane == (uint32_t)(__ffs(ib) - 1)) {
                const unsigned long long before = atomicAdd(&st->inserted, (unsigned long long)__popc(ib));
                if (before + __popc(ib) > m.max_inserted) set_error(&st->error, ST_HASH_FULL);
            }
            const uint32_t bal = __ballot_sync(kFull, improved);
            if (bal) {
                const uint32_t leader = (uint32_t)(__ffs(bal) - 1);
                uint32_t cbase = 0;
                if (lane == leader) cbase = atomicAdd(&st->cand_count[par], (uint32_t)__popc(bal));
                cbase = __shfl_sync(kFull, cbase, leader);
                if (improved) {
                    Cand c;
                    c.slot = nslot;
                    c.parent = oslot;
                    c.g = ng;
                    c.f = nf;
                    c.aux = naux;
                    c.pad = 0;
                    m.cand[cbase + __popc(bal & lanemask_lt())] = c;
                }
            }
        }

        team.sync();

        // -------------------------------------------------- decision ---
        // Every value read here is written only before the barrier above or
        // after the next one, so all threads decide alike.
        const uint64_t rmin = team.rd64(&st->round_min[par]);
        const uint64_t gbest = team.rd64(&st->goal_best);
        // Phase-2 errors of round r are written to error2[r & 1] and read at
        // the decision of round r + 1, so no thread can see one that another
        // thread of the same decision missed.
        uint32_t err = team.rd32(&st->error);
        if (!err) err = team.rd32(&st->error2[par ^ 1]);
        const uint32_t ncand = team.rd32(&st->cand_count[par]);
        round += 1;
        if (err) {
            status = err;
            break;
        }
        if (gbest != kInfCost && P::cost_cmp(gbest, rmin) <= 0) {
            status = ST_OK;
            break;
        }
        if (rmin == kInfCost) {
            status = ST_NO_SOLUTION;
            break;
        }
        if (round >= m.max_rounds) {
            status = ST_ITER_LIMIT;
            break;
        }

        // ---------------------------------------------------- phase 2 ---
        if (rank == 0) {
            st->round_min[par ^ 1] = kInfCost;
            st->cand_count[par ^ 1] = 0;
        }
        const uint32_t target = (rank + base) % k;
        base = (uint32_t)(((uint64_t)base + ncand) % k);
        if (rank < ncand) {
            E *th = m.heaps + (size_t)target * m.stride;
            uint32_t ths = ldcg_u32(&m.heap_size[target]);
            for (uint32_t i = rank; i < ncand; i += k) {
                const Cand c = load_cand(m.cand + i);
                if (ldcg_u64(&m.tab[c.slot].g) != c.g) continue;  // lost to a better writer
                m.tab[c.slot].prev = c.parent;
                m.tab[c.slot].aux = c.aux;
                if (ths + 1 >= m.stride) {
                    set_error(&st->error2[par], ST_HEAP_OVERFLOW);
                    break;
                }
                heap_push<P>(th, ths, prob.make_entry(c.f, c.g, c.slot));
                ++nP;
            }
            m.heap_size[target] = ths;
        }
        team.sync();
        if (it + 1 >= budget) break;
    }

    // Persist the resumable state (uniform values; rank 0 writes).
    if (rank == 0) {
        st->round = round;
        st->base = base;
        if (status != ST_RUNNING) st->status = status;
    }
    // Flush statistics: one atomic per warp.
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        nE += __shfl_xor_sync(kFull, (unsigned long long)nE, o);
        nS += __shfl_xor_sync(kFull, (unsigned long long)nS, o);
        nP += __shfl_xor_sync(kFull, (unsigned long long)nP, o);
    }
    if (lane == 0) {
        atomicAdd(&st->expanded, (unsigned long long)nE);
        atomicAdd(&st->generated, (unsigned long long)nS);
        atomicAdd(&st->pushed, (unsigned long long)nP);
    }
    return status;
}

}  // namespace uastar

// The GA* round loop, generic over the problem (grid / puzzle) and the team
// that runs it (the whole cooperative grid for one large instance, or one
// CTA per instance in the batched and serving engines).
//
// A team is C CTAs of T threads; each CTA owns H binary min-heaps (the first
// H threads are their owners, T / H threads per heap), so the team has
// k = C * H heaps.  A round is:
//
//   phase 1  each heap owner pops its heap's minimum; the round's minimum
//            popped f is reduced (warp shuffles, one CAS per warp); stale
//            entries (f no longer matching the node's g) are dropped; a goal
//            pop lowers goal_best; every other pop is expanded.  The CTA then
//            spreads the successors of its H pops over all T threads; each
//            thread relaxes its successor in the open-addressed dedup table
//            with one 16-byte CAS on (key, g): it either claims an empty slot
//            with its g, or learns the slot's g and lowers it with a CAS loop.
//            Only a strict improvement makes the successor a candidate, so
//            among equal-g writers of one slot in a round exactly one
//            candidate carries the final g.
//   barrier  then a uniform decision: stop when the best goal f popped so
//            far <= the round's minimum popped f (the GA* optimality test of
//            the reference, src/pathway/GPU-solver.cu:219-243), fail when
//            nothing was popped.
//   phase 2  CTA c takes the candidates of CTA (c + round) mod C's region
//            (the successors of that CTA's pops); its threads check them in
//            parallel (a candidate is the slot's winner iff the slot's g
//            still equals its g; only the winner writes prev/aux) and its
//            heap owners push the winners, dealt round-robin over the CTA's
//            heaps.
//
// There is no barrier after phase 2: a CTA that finishes its pushes starts
// the next round at once.  Its own heaps are all it pops; a relax of round
// r + 1 that lowers a slot's g while round r's check of that slot is still
// running only turns round r's candidate into a loser (round r + 1's own
// candidate for the slot carries the better g), and round r + 1's prev/aux
// writes come after its barrier, so after every write of round r.  The
// round-indexed team fields and the candidate buffers are multi-buffered
// for this (TeamState).
//
// Heaps are CTA-private, so the top levels of every heap live in shared
// memory (a pop touches global memory only below them).
//
// This replaces the reference's per-round kExtractExpand -> host copy ->
// MergesortPairs -> kAssign -> host copy -> kDeduplicate -> kHeapInsert
// chain (src/pathway/GPU-solver.cu:180-328) with one persistent kernel and
// no host round trip: by default the per-round sort + unique of the
// successor list is replaced by the table's atomic minimum (same result: the
// minimum g per state among this round's successors and the stored node);
// the kSort variant keeps the reference's order with a team radix sort
// (ga_sort.cuh) between the decision and the push phase.
#pragma once
#include <cstdint>

#include "ga_device.cuh"
#include "ga_sort.cuh"

namespace uastar {

template <class E> struct SearchMem {
    Slot *tab;
    uint64_t mask;          // slots - 1 (power of two)
    uint64_t max_inserted;  // load limit
    uint32_t max_probe;
    E *heaps;               // k heaps of `stride` entries, CTA c owns heaps [c*H, (c+1)*H)
    uint32_t stride;        // entries per heap: saved shared top, then the bricks
    uint32_t hcap;          // maximum heap size
    uint32_t L;             // heap levels kept in shared memory (>= 1)
    uint32_t *heap_size;    // k sizes
    Cand *cand;             // cand_records<P>(C, H) records
    uint64_t max_rounds;    // absolute round limit (ITER_LIMIT)
    // A resumable search pauses (returns ST_RUNNING) at the end of the round
    // in which `inserted` passes grow_at, with the round's candidates pushed
    // and no work in flight, so that the host can move the table to a larger
    // one and resume; ~0 = never.
    uint64_t grow_at = ~0ull;
    // A time slice: the search also pauses at the end of the first round
    // that team rank 0 finishes at or after this globaltimer value (ns);
    // 0 = none.  The serving loop's quanta end on it, so that every resident
    // search runs for the same time rather than the same number of rounds.
    uint64_t deadline_ns = 0;
    // Split rounds (CTA and cluster teams, table-minimum dedup, separate
    // owner warps): the heap owners arrive at the team barrier as soon as
    // their pops are published and refill their heaps while the relaxers
    // finish, pass the barrier, decide and stage the pushes; the owners then
    // wait for the staging only.  Needs SearchSmem<P>::bytes_split shared
    // memory.  0 = one barrier for all threads.
    uint32_t split = 0;
    // Sort-based dedup (ga_search<.., true>): every round's successors are
    // radix-sorted by key and each key's minimum-g record is relaxed once.
    unsigned long long *sort_buf = nullptr;  // 2 x C * H * kMoves pairs
    uint32_t *sort_hist = nullptr;           // 256 x (C + 1) digit counts
    uint32_t sort_bits = 0;                  // key bits to sort on
};

// Named CTA barriers (0 is __syncthreads): barrier.sync waits for `n`
// threads (a multiple of 32) to have arrived; barrier.arrive counts this
// thread without waiting.  Both order this thread's earlier memory accesses
// before the barrier's completion for the threads that wait on it.  The
// non-.aligned forms: a warp may reach them diverged (owner lanes leave
// their chores at different times).
__device__ __forceinline__ void named_sync(uint32_t id, uint32_t n) {
    asm volatile("barrier.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
__device__ __forceinline__ void named_arrive(uint32_t id, uint32_t n) {
    asm volatile("barrier.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// ------------------------------------------------------------------ teams ---
// Split rounds (SearchMem::split) need the team barrier in two halves:
// early_arrive() by the owner warps (no wait), relaxers_sync() by the
// relaxer warps (arrive and wait), late_wait() by the owner warps after
// their chores.  The grid team has no split form.
struct GridTeam {
    static constexpr bool kSplit = false;
    __device__ void early_arrive() {}  // (no split form: never called)
    __device__ void relaxers_sync(uint32_t) {}
    __device__ void late_wait() {}
    TeamState *st;  // global memory
    uint32_t epoch;
    uint64_t timeout_ns;
    __device__ uint32_t cta() const { return blockIdx.x; }
    __device__ uint32_t ctas() const { return gridDim.x; }
    __device__ void sync() { grid_barrier(&st->barrier, gridDim.x, epoch, &st->error, timeout_ns); }
    __device__ uint64_t rd64(const unsigned long long *p) const { return ldcg_u64(p); }
    __device__ uint32_t rd32(const uint32_t *p) const { return ldcg_u32(p); }
};

// A thread-block cluster as one team: CTA rank within the cluster, hardware
// cluster barrier (barrier.cluster arrive.release / wait.acquire; all CTAs of
// a cluster are co-scheduled, so the barrier needs no time bound), team
// state in global memory read through L2.  The barrier's release/acquire at
// cluster scope orders every memory access of the cluster's threads, global
// ones included, so no separate fence is needed.
struct ClusterTeam {
    static constexpr bool kSplit = true;
    TeamState *st;  // global memory
    __device__ uint32_t cta() const {
        uint32_t r;
        asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
        return r;
    }
    __device__ uint32_t ctas() const {
        uint32_t r;
        asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
        return r;
    }
    __device__ void sync() {
        asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
    }
    // split halves: the cluster barrier's own arrive and wait, in the forms
    // that a diverged warp may execute
    __device__ void early_arrive() { asm volatile("barrier.cluster.arrive.release;" ::: "memory"); }
    __device__ void relaxers_sync(uint32_t) {
        asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
    }
    __device__ void late_wait() { asm volatile("barrier.cluster.wait.acquire;" ::: "memory"); }
    __device__ uint64_t rd64(const unsigned long long *p) const { return ldcg_u64(p); }
    __device__ uint32_t rd32(const uint32_t *p) const { return ldcg_u32(p); }
};

struct BlockTeam {
    static constexpr bool kSplit = true;
    TeamState *st;  // shared memory
    __device__ uint32_t cta() const { return 0; }
    __device__ uint32_t ctas() const { return 1; }
    __device__ void sync() { __syncthreads(); }
    // split halves: named barrier 1 over the whole CTA, owners arriving early
    __device__ void early_arrive() { named_arrive(1, blockDim.x); }
    __device__ void relaxers_sync(uint32_t n) { named_sync(1, n); }
    __device__ void late_wait() {}
    __device__ uint64_t rd64(const unsigned long long *p) const {
        return *reinterpret_cast<const volatile unsigned long long *>(p);
    }
    __device__ uint32_t rd32(const uint32_t *p) const {
        return *reinterpret_cast<const volatile uint32_t *>(p);
    }
};

// ------------------------------------------------------------------ heaps ---
// A 1-indexed binary min-heap.  Entries 1..2^L-1 (the top L levels) live in
// shared memory.  Below them the tree is cut into bricks: complete subtrees
// of D levels whose 2^D - 1 entries fill one 128-byte line in global memory
// (D = 3 for 16-byte entries, 4 for 8-byte entries; slot 0 of a brick is
// unused).  A sift-down reads both child bricks of a node in one burst of
// independent loads, so it waits on global memory once per D levels instead
// of once per level.  Bricks are stored level by level: the 2^(L + b*D)
// bricks of brick level b follow the 2^L (2^(b*D) - 1) / (2^D - 1) bricks of
// the levels above it, in the order of their root indices.
template <class P> struct BrickHeap {
    using E = typename P::Entry;
    static constexpr uint32_t D = sizeof(E) == 16 ? 3 : 4;
    static constexpr uint32_t BE = 1u << D;  // entries per brick line
    static_assert(BE * sizeof(E) == 128, "one brick per 128-byte line");
    E *g;       // this heap's bricks
    E *s;       // shared top, index 0 unused
    E *scr;     // shared scratch: three bricks (0, 1: the sift-down; 2: the buffer drain)
    uint32_t L; // levels in shared memory

    __device__ __forceinline__ uint32_t topn() const { return (1u << L) - 1; }
    // global entry offset of heap index i (i > topn)
    __device__ __forceinline__ uint64_t off(uint32_t i) const {
        const uint32_t l = 31u - (uint32_t)__clz(i);
        const uint32_t r = l - L;
        const uint32_t bl = r / D;
        const uint32_t d = r - bl * D;
        const uint32_t root = i >> d;
        const uint32_t local = (1u << d) | (i & ((1u << d) - 1u));
        const uint64_t first = (((1ull << (bl * D)) - 1ull) << L) / (BE - 1u);
        const uint64_t id = first + (root - (1ull << (L + bl * D)));
        return id * BE + local;
    }
    __device__ __forceinline__ E ld(uint32_t i) const { return i <= topn() ? s[i] : P::load(g + off(i)); }
    __device__ __forceinline__ void st(uint32_t i, const E &v) const {
        if (i <= topn())
            s[i] = v;
        else
            P::store(g + off(i), v);
    }
    // Root of the brick holding heap index i (i > topn), and i's depth in it.
    __device__ __forceinline__ uint32_t brick_root(uint32_t i, uint32_t *depth = nullptr) const {
        const uint32_t r = 31u - (uint32_t)__clz(i) - L;
        const uint32_t d = r - (r / D) * D;
        if (depth) *depth = d;
        return i >> d;
    }
    // Start copying the brick rooted at `root` into scratch brick `h` with
    // asynchronous global -> shared copies (no registers held); complete
    // with cp_async_wait_all() before reading it.
    __device__ __forceinline__ void fetch_async(uint32_t root, uint32_t h) const {
        const char *src = reinterpret_cast<const char *>(g + off(root) - 1);
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(scr + h * BE);
#pragma unroll
        for (int q = 0; q < 8; ++q)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + 16u * q), "l"(src + 16 * q)
                         : "memory");
    }
    // Copy the brick rooted at heap index `root` into scratch half `h`.
    __device__ __forceinline__ void fetch(uint32_t root, uint32_t h) const {
        const uint4 *src = reinterpret_cast<const uint4 *>(g + off(root) - 1);
        uint4 *dst = reinterpret_cast<uint4 *>(scr + h * BE);
        uint4 v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = __ldcg(src + q);
#pragma unroll
        for (int q = 0; q < 8; ++q) dst[q] = v[q];
    }
};

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Fill the root hole: `last` (the old heap[size]) is sifted down from the
// root.  `size` is the size after removal.  Returns the position where
// `last` came to rest (every position written lies on the path to it).
template <class P>
__device__ __forceinline__ uint32_t heap_sift_down(const BrickHeap<P> &h, uint32_t size, typename P::Entry last) {
    using E = typename P::Entry;
    constexpr uint32_t D = BrickHeap<P>::D, BE = BrickHeap<P>::BE;
    const uint32_t topn = h.topn();
    uint32_t now = 1;
    // shared-memory levels
    for (;;) {
        uint32_t c = now << 1;
        if (c > size || c > topn) break;
        E a = h.s[c];
        if (c < size) {
            const E b = h.s[c + 1];
            if (P::less(b, a)) {
                a = b;
                ++c;
            }
        }
        if (!P::less(a, last)) {
            h.s[now] = last;
            return now;
        }
        h.s[now] = a;
        now = c;
    }
    if ((now << 1) > size) {
        h.st(now, last);
        return now;
    }
    // global bricks: `half` is the scratch half holding the brick of `now`
    // (none while `now` is in shared memory), `depth` its level in that brick
    int half = -1;
    uint32_t depth = 0;
    for (;;) {
        uint32_t c = now << 1;
        if (c > size) break;
        E a, b;
        const bool two = c < size;
        int ch = half;
        if (half >= 0 && depth + 1 < D) {
            const uint32_t la = (1u << (depth + 1)) | (c & ((1u << (depth + 1)) - 1u));
            a = h.scr[half * BE + la];
            if (two) b = h.scr[half * BE + la + 1];
        } else {
            // the children are the roots of two bricks
            h.fetch(c, 0);
            if (two) h.fetch(c + 1, 1);
            a = h.scr[1];
            if (two) b = h.scr[BE + 1];
            ch = 0;
        }
        bool right = two && P::less(b, a);
        if (right) a = b;
        if (!P::less(a, last)) break;
        h.st(now, a);
        if (half >= 0 && depth + 1 < D) {
            depth += 1;
        } else {
            half = right ? 1 : 0;
            depth = 0;
            (void)ch;
        }
        now = c + (right ? 1u : 0u);
    }
    h.st(now, last);
    return now;
}

// Entry at heap index `par` (the parent of a brick's root), from the shared
// top or else by reading its whole brick into scratch half `half`: the brick
// a climb that passes `par` continues in, so that it is read only once.
template <class P>
__device__ __forceinline__ typename P::Entry heap_parent(const BrickHeap<P> &h, uint32_t par, uint32_t half) {
    constexpr uint32_t BE = BrickHeap<P>::BE;
    if (par <= h.topn()) return h.s[par];
    uint32_t d;
    const uint32_t root = h.brick_root(par, &d);
    h.fetch(root, half);
    return h.scr[half * BE + ((1u << d) | (par & ((1u << d) - 1u)))];
}

// Fill the vacant heap position `now` with v, moving v up as far as it goes.
// Below the shared top the climb works brick by brick: the brick holding the
// current position is read once (one burst of independent loads) into a
// scratch half, the climb inside it runs in shared memory and the brick is
// written back; at a brick's root the parent's whole brick is read into the
// other half, which the climb continues in if it goes on, so a climb waits
// on global memory once per brick it passes through (most pass none or one)
// instead of once per level.  `bottom`: `now` is the heap's new last
// position, so a brick rooted there holds nothing else yet (all its other
// positions are below it) and is not read.  `have` >= 0: the brick of `now`
// is already in that scratch half.
template <class P>
__device__ __forceinline__ void heap_climb(const BrickHeap<P> &h, uint32_t now, const typename P::Entry &v,
                                           bool bottom = false, int have = -1) {
    using E = typename P::Entry;
    constexpr uint32_t BE = BrickHeap<P>::BE;
    const uint32_t topn = h.topn();
    int cur = have;
    while (now > topn) {
        uint32_t d;
        const uint32_t root = h.brick_root(now, &d);  // d = depth of `now` in its brick
        if (cur < 0) {
            if (!(bottom && d == 0)) h.fetch(root, 0);
            cur = 0;
        }
        bottom = false;
        E *const b = h.scr + cur * BE;
        uint4 *const gl = reinterpret_cast<uint4 *>(h.g + h.off(root) - 1);
        uint32_t loc = (1u << d) | (now & ((1u << d) - 1u));
        while (loc > 1) {
            const E pv = b[loc >> 1];
            if (!P::less(v, pv)) break;
            b[loc] = pv;
            loc >>= 1;
            now >>= 1;
        }
        bool done = loc > 1;
        if (!done) {
            // at the brick's root: its parent is in the brick above (read
            // into the other half) or in the shared top
            const E pv = heap_parent<P>(h, now >> 1, (uint32_t)(cur ^ 1));
            if (!P::less(v, pv)) {
                done = true;
            } else {
                b[1] = pv;
                now >>= 1;
            }
        }
        if (done) b[loc] = v;
        const uint4 *src = reinterpret_cast<const uint4 *>(b);
#pragma unroll
        for (int q = 0; q < 8; ++q) gl[q] = src[q];
        if (done) return;
        cur ^= 1;  // the parent's brick, if `now` is still below the top
    }
    while (now > 1) {
        const uint32_t par = now >> 1;
        const E pv = h.s[par];
        if (!P::less(v, pv)) break;
        h.s[now] = pv;
        now = par;
    }
    h.s[now] = v;
}

// Insert v.
template <class P>
__device__ __forceinline__ void heap_push(const BrickHeap<P> &h, uint32_t &size, const typename P::Entry &v) {
    heap_climb<P>(h, ++size, v, true);
}

// Insert the n entries at v (an insertion buffer's drain).  They take the
// positions size+1 .. size+n, consecutive leaves at the bottom of the tree
// that share one brick (two at a brick or level boundary): that brick is
// read once into scratch brick 2 (`have`: already there, read ahead by the
// caller), every entry's climb inside it runs there,
// and it is written back when the bottom moves to another brick, before a
// climb that leaves it (finished by heap_climb from the brick above), and at
// the end.  A drain of n entries so waits on global memory about once
// instead of n times.  (A bottom position that roots its own brick needs no
// read: nothing else in that brick is in use.)
template <class P>
__device__ __forceinline__ void heap_push_run(const BrickHeap<P> &h, uint32_t &size, const typename P::Entry *v,
                                              uint32_t n, uint32_t have = 0) {
    using E = typename P::Entry;
    constexpr uint32_t D = BrickHeap<P>::D, BE = BrickHeap<P>::BE;
    const uint32_t topn = h.topn();
    E *const b = h.scr + 2 * BE;  // scratch brick 2
    uint32_t cached = have;       // root of the brick held in b (0: none)
    const auto flush = [&]() {
        if (!cached) return;
        uint4 *const gl = reinterpret_cast<uint4 *>(h.g + h.off(cached) - 1);
        const uint4 *src = reinterpret_cast<const uint4 *>(b);
#pragma unroll
        for (int q = 0; q < 8; ++q) gl[q] = src[q];
        cached = 0;
    };
    for (uint32_t i = 0; i < n; ++i) {
        const E x = v[i];
        uint32_t now = size + 1;
        if (now <= topn) {  // shared top only: no brick involved
            heap_push<P>(h, size, x);
            continue;
        }
        size = now;
        const uint32_t l = 31u - (uint32_t)__clz(now);
        const uint32_t r = l - h.L;
        const uint32_t d = r - (r / D) * D;
        const uint32_t root = now >> d;
        if (root != cached) {
            flush();
            if (d > 0) h.fetch(root, 2);
            cached = root;
        }
        uint32_t loc = (1u << d) | (now & ((1u << d) - 1u));
        while (loc > 1) {
            const E pv = b[loc >> 1];
            if (!P::less(x, pv)) break;
            b[loc] = pv;
            loc >>= 1;
            now >>= 1;
        }
        if (loc > 1) {
            b[loc] = x;
            continue;
        }
        // at the brick's root: its parent is in the brick above (read whole
        // into scratch half 0, where the climb continues) or the shared top
        const E pv = heap_parent<P>(h, now >> 1, 0);
        if (!P::less(x, pv)) {
            b[1] = x;
            continue;
        }
        b[1] = pv;
        flush();
        heap_climb<P>(h, now >> 1, x, false, 0);
    }
    flush();
}

// Global entries per heap and the largest heap size for L shared levels and
// a requested capacity (host side).
template <class P> struct HeapGeometry {
    uint32_t stride;  // entries of global memory per heap (saved top + bricks)
    uint32_t hcap;    // maximum heap size
};
// Offset of the bricks within a heap's global block: the first entries hold
// the shared top while a resumable search is parked.
template <class P> __host__ __device__ constexpr uint32_t top_reserve(uint32_t L) {
    return ((1u << L) + BrickHeap<P>::BE - 1u) / BrickHeap<P>::BE * BrickHeap<P>::BE;
}
template <class P> __host__ HeapGeometry<P> heap_geometry(uint32_t L, uint64_t want) {
    constexpr uint32_t D = BrickHeap<P>::D, BE = BrickHeap<P>::BE;
    uint32_t levels = 0;
    while (levels < 30 && ((1ull << levels) - 1) < want) ++levels;
    uint32_t nbl = levels > L ? (levels - L + D - 1) / D : 1;
    if (nbl < 1) nbl = 1;
    while (L + nbl * D > 31) --nbl;
    const uint64_t bricks = (((1ull << (nbl * D)) - 1ull) << L) / (BE - 1u);
    HeapGeometry<P> geo;
    geo.stride = (uint32_t)(bricks * BE) + top_reserve<P>(L);
    geo.hcap = (uint32_t)((1ull << (L + nbl * D)) - 1ull);
    return geo;
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

// (key, g) half of a slot, updated as one 16-byte word.
struct __align__(16) KeyG {
    unsigned long long key, g;
};
__device__ __forceinline__ KeyG cas128(Slot *s, KeyG cmp, KeyG val) {
    return atomicCAS(reinterpret_cast<KeyG *>(s), cmp, val);
}

// Bit 0: g strictly lowered; bit 1: a new slot was claimed; RELAX_FULL: the
// probe limit was reached.
enum : int { RELAX_NONE = 0, RELAX_IMPROVED = 1, RELAX_CLAIMED = 2, RELAX_INSERTED = 3, RELAX_FULL = 4 };

// Find-or-insert `key` and lower its g to `g` in one pass.  The home slot is
// tried with a single 16-byte CAS that either claims it empty with (key, g)
// or returns what it holds; later probe steps read first and only CAS a slot
// that is empty or holds the key.  Returns RELAX_INSERTED (new slot, g set),
// RELAX_IMPROVED (existing slot, g strictly lowered), RELAX_NONE (existing
// slot, g not better) or RELAX_FULL (probe limit).
//
// Where the problem keeps the parent link in the key word (P::kPrevInKey:
// grid cells are 32 bits), the word is cell | prev << 32 and the CAS sets g
// and prev together, so the slot's link always belongs to its g: the push
// phase then needs no winner check.  Keys compare on the cell half.  Where it
// keeps the link in the g word (P::kLink == LINK_IN_G), the CAS installs
// P::g_word(g, prev, move) and costs compare on P::word_g of it.
template <class P> __device__ __forceinline__ bool key_match(uint64_t word, uint64_t key) {
    if constexpr (P::kPrevInKey)
        return (word & 0xffffffffull) == key && word != kEmptyKey;
    else
        return word == key;
}

template <class P>
__device__ __forceinline__ int relax_at(Slot *tab, uint64_t h, KeyG cur, uint64_t word, uint64_t g,
                                        uint64_t gw, uint32_t *slot_out) {
    // the slot holds the key: lower g (and, with the link in the key or g
    // word, set the link with it)
    *slot_out = (uint32_t)h;
    while (P::cost_cmp(g, P::word_g(cur.g)) < 0) {
        const KeyG old = cas128(tab + h, cur, KeyG{P::kPrevInKey ? word : cur.key, gw});
        if (old.key == cur.key && old.g == cur.g) return RELAX_IMPROVED;
        cur = old;
    }
    return RELAX_NONE;
}

template <class P>
__device__ __forceinline__ int relax(Slot *tab, uint64_t mask, uint32_t max_probe, uint64_t key, uint64_t g,
                                     uint32_t prev, uint32_t *slot_out, int mv = -1) {
    // Linear probing.  The home slot is tried with one 16-byte CAS; past it
    // the probe reads the rest of the home slot's 128-byte line (4 slots) and
    // then whole lines, one dependent load per line.
    const uint64_t word = P::kPrevInKey ? (key | (uint64_t)prev << 32) : key;
    const uint64_t gw = P::g_word(g, prev, mv);
    uint64_t h = mix64(key) & mask;
    const KeyG empty{kEmptyKey, kInfCost};
    KeyG cur = cas128(tab + h, empty, KeyG{word, gw});
    if (cur.key == kEmptyKey) {
        *slot_out = (uint32_t)h;
        return RELAX_INSERTED;
    }
    if (key_match<P>(cur.key, key)) return relax_at<P>(tab, h, cur, word, g, gw, slot_out);
    uint32_t probed = 1;
    h = (h + 1) & mask;
    while (probed < max_probe) {
        // slots h .. end of h's line (the table is line-aligned, mask >= 3)
        const uint32_t n = 4u - (uint32_t)(h & 3u);
        ulonglong2 v[4];
#pragma unroll
        for (uint32_t q = 0; q < 4; ++q)
            if (q < n) v[q] = __ldcg(reinterpret_cast<const ulonglong2 *>(tab + h + q));
        for (uint32_t q = 0; q < n; ++q) {
            const uint64_t hq = h + q;
            if (key_match<P>(v[q].x, key)) return relax_at<P>(tab, hq, KeyG{v[q].x, v[q].y}, word, g, gw, slot_out);
            if (v[q].x == kEmptyKey) {
                cur = cas128(tab + hq, empty, KeyG{word, gw});
                if (cur.key == kEmptyKey) {
                    *slot_out = (uint32_t)hq;
                    return RELAX_INSERTED;
                }
                if (key_match<P>(cur.key, key)) return relax_at<P>(tab, hq, cur, word, g, gw, slot_out);
                // another key took it: keep probing
            }
        }
        probed += n;
        h = (h + n) & mask;
    }
    return RELAX_FULL;
}

// Wide keys: find-or-claim the 16-byte key with one 16-byte CAS per probed
// slot, then lower the slot's g with an 8-byte CAS loop.  A claimer whose g
// another writer of the same key has already undercut reports RELAX_CLAIMED.
template <class P>
__device__ __forceinline__ int relax_wide(Slot *tab, uint64_t mask, uint32_t max_probe, const Key128 &key,
                                          uint64_t g, uint32_t *slot_out) {
    uint64_t h = key_hash(key) & mask;
    const KeyG empty{kEmptyKey, kEmptyKey};
    for (uint32_t probe = 0; probe < max_probe; ++probe) {
        const KeyG cur = cas128(tab + h, empty, KeyG{key.lo, key.hi});
        const bool claimed = cur.key == kEmptyKey && cur.g == kEmptyKey;
        if (claimed || (cur.key == key.lo && cur.g == key.hi)) {
            *slot_out = (uint32_t)h;
            unsigned long long *gp = &WideSlots::w(tab + h)->g;
            unsigned long long old = claimed ? kInfCost : __ldcg(gp);
            while (P::cost_cmp(g, old) < 0) {
                const unsigned long long seen = atomicCAS(gp, old, (unsigned long long)g);
                if (seen == old) return claimed ? RELAX_INSERTED : RELAX_IMPROVED;
                old = seen;
            }
            return claimed ? RELAX_CLAIMED : RELAX_NONE;
        }
        h = (h + 1) & mask;
    }
    return RELAX_FULL;
}

template <class P>
__device__ __forceinline__ int relax_key(Slot *tab, uint64_t mask, uint32_t max_probe, const typename P::Key &key,
                                         uint64_t g, uint32_t prev, uint32_t *slot_out, int mv = -1) {
    if constexpr (P::kWide)
        return relax_wide<P>(tab, mask, max_probe, key, g, slot_out);
    else
        return relax<P>(tab, mask, max_probe, key, g, prev, slot_out, mv);
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

// Shared-memory layout of one CTA of a search team.
template <class Key> struct PopInfo {
    Key key;
    unsigned long long g;
    uint32_t aux, slot, mask, excl;  // excl: exclusive prefix of successor counts
};

// Candidate records of a team of C CTAs with H heaps each: two buffers (by
// round parity) of C regions, one per CTA, each a header record (its count
// in .slot) and room for the successors of the CTA's H pops.
template <class P> __host__ __device__ constexpr uint64_t cand_region_records(uint32_t H) {
    return (uint64_t)H * P::kMoves + 1;
}
template <class P> __host__ __device__ constexpr uint64_t cand_records(uint32_t C, uint32_t H) {
    return 2ull * C * cand_region_records<P>(H);
}

template <class P> struct SearchSmem {
    using E = typename P::Entry;
    // entries of a heap's insertion buffer: two rounds of pushes
    static constexpr uint32_t kBuf = 2 * P::kMoves;
    // Per-heap strides (entries) of the heap tops, brick scratch and
    // insertion buffers.  Heap h's owner is lane h % 32 of an owner warp, and
    // the owners walk their heaps in step: unpadded, every stride is a
    // multiple of 128 bytes, so all lanes of a warp would hit the same banks
    // (a 16- or 32-way conflict on every access).  One extra entry (16 bytes
    // for the scratch, whose bricks are copied with 16-byte cp.async) moves
    // consecutive heaps two or four banks apart: an 8-byte access of a half
    // warp and a 16-byte access of a quarter warp touch distinct banks.
    static __host__ __device__ constexpr uint32_t top_stride(uint32_t L) { return (1u << L) + 1u; }
    static constexpr uint32_t kScrStride = 3 * BrickHeap<P>::BE + 16 / sizeof(E);
    static constexpr uint32_t kBufStride = kBuf + 1;
    // pops, heap tops, brick scratch, insertion buffers, then warp totals
    static __host__ __device__ size_t tops_offset(uint32_t H) {
        return ((size_t)H * sizeof(PopInfo<typename P::Key>) + 15) & ~(size_t)15;
    }
    static __host__ __device__ size_t scr_offset(uint32_t H, uint32_t L) {
        return (tops_offset(H) + (size_t)H * top_stride(L) * sizeof(E) + 127) & ~(size_t)127;
    }
    static __host__ __device__ size_t buf_offset(uint32_t H, uint32_t L) {
        return scr_offset(H, L) + (size_t)H * kScrStride * sizeof(E);
    }
    static __host__ __device__ size_t scratch_offset(uint32_t H, uint32_t L) {
        return (buf_offset(H, L) + (size_t)H * kBufStride * sizeof(E) + 15) & ~(size_t)15;
    }
    // warp totals of the block scans, this CTA's round counters, then the
    // owner warps' minimum popped f (16 x 8 bytes)
    static constexpr uint32_t kScratchWords = 72;
    static __host__ __device__ size_t bytes(uint32_t H, uint32_t L) {
        return scratch_offset(H, L) + 4 * kScratchWords;
    }
    // the sort-based dedup's shared memory follows (T threads per CTA); or,
    // with split rounds, the push staging (the sift scratch is busy then)
    static __host__ __device__ size_t sort_offset(uint32_t H, uint32_t L) { return (bytes(H, L) + 15) & ~(size_t)15; }
    static __host__ __device__ size_t bytes_split(uint32_t H, uint32_t L) {
        return sort_offset(H, L) + (size_t)H * P::kMoves * sizeof(E);
    }
    static __host__ __device__ size_t bytes_sorted(uint32_t H, uint32_t L, uint32_t T) {
        return sort_offset(H, L) + sort_smem_bytes(T);
    }
};

// Exclusive prefix sum over the CTA of one value per thread (blockDim.x a
// multiple of 32, at most 1024); *total gets the sum.  Uses scratch[0] and
// scratch[2 .. 2 + warps).
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *scratch, uint32_t *total) {
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, o);
        if (lane >= (uint32_t)o) incl += t;
    }
    if (lane == 31) scratch[2 + w] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t acc = 0;
        for (uint32_t q = 0; q < nw; ++q) {
            const uint32_t t = scratch[2 + q];
            scratch[2 + q] = acc;
            acc += t;
        }
        scratch[0] = acc;
    }
    __syncthreads();
    const uint32_t off = scratch[2 + w] + incl - v;
    *total = scratch[0];
    __syncthreads();
    return off;
}

// ------------------------------------------------------------ the search ---
// Runs up to `budget` rounds (resumable: state lives in TeamState, the heaps
// and the table).  Returns ST_RUNNING if the budget ran out first or the
// table passed m.grow_at, else the final status.  Every thread of every CTA of the team must call it with the
// same H (heaps per CTA, 1 <= H <= blockDim.x); `smem` points at
// SearchSmem<P>::bytes(H, m.L) bytes of shared memory (128-byte aligned),
// bytes_sorted(H, m.L, blockDim.x) with kSort.
//
// kSort (keys of at most 32 bits) runs the reference's dedup order instead
// of the in-table minimum: the relax phase only writes every successor's
// record; after the decision the team radix-sorts the round's records by key
// (team_radix_sort), and the first record of each key's run with the least g
// (the sort is stable: the earliest of equal g) is relaxed into the table,
// once per key, and pushed if it strictly improved the slot.  Same result,
// three team barriers per sort pass more per round.
template <class P, class Team, bool kSort = false>
__device__ uint32_t ga_search(const P &prob, Team &team, const SearchMem<typename P::Entry> &m, uint32_t H,
                              unsigned char *smem, uint64_t budget) {
    static_assert(!kSort || (!P::kWide && P::kPrevInKey), "sorted dedup: 32-bit keys with the link in the key word");
    using E = typename P::Entry;
    TeamState *st = team.st;
    const uint32_t T = blockDim.x, tid = threadIdx.x, lane = tid & 31u;
    const uint32_t C = team.ctas(), cta = team.cta();
    const bool owner = tid < H;
    const uint32_t myh = cta * H + tid;  // global heap index (valid when owner)
    const uint32_t L = m.L, topn = (1u << L) - 1;
    const uint32_t owner_warps = (H + 31u) / 32u;
    // Warps past the owners relax successors while the owners refill their
    // heaps' root holes; with no such warps, everyone relaxes first.
    const uint32_t rfirst = T > owner_warps * 32u ? owner_warps * 32u : 0u;
    const uint32_t rthreads = T - rfirst;
    const bool relaxer = tid >= rfirst;
    // split rounds (SearchMem::split), uniform over the team
    bool split = false;
    if constexpr (Team::kSplit && !kSort) split = m.split != 0 && rfirst > 0;

    using Key = typename P::Key;
    PopInfo<Key> *pop = reinterpret_cast<PopInfo<Key> *>(smem);
    E *tops = reinterpret_cast<E *>(smem + SearchSmem<P>::tops_offset(H));
    E *scr = reinterpret_cast<E *>(smem + SearchSmem<P>::scr_offset(H, L));
    uint32_t *scratch = reinterpret_cast<uint32_t *>(smem + SearchSmem<P>::scratch_offset(H, L));

    E *const gblock = m.heaps + (size_t)(owner ? myh : 0) * m.stride;  // saved top, then bricks
    BrickHeap<P> myheap{gblock + top_reserve<P>(L), tops + (size_t)(owner ? tid : 0) * SearchSmem<P>::top_stride(L),
                        scr + (size_t)(owner ? tid : 0) * SearchSmem<P>::kScrStride, L};
    // The heap's insertion buffer: an unordered list of up to kBuf entries in
    // shared memory in front of the heap.  The push phase only appends to it;
    // a pop takes the smaller of the heap's root and the buffer's minimum;
    // the owner moves entries from the buffer into the heap in the relax
    // phase (drain), off the round's critical path, keeping room for the next
    // push phase.  The heap and the buffer together are the priority queue.
    constexpr uint32_t kBuf = SearchSmem<P>::kBuf;
    E *const ibuf =
        reinterpret_cast<E *>(smem + SearchSmem<P>::buf_offset(H, L)) + (size_t)(owner ? tid : 0) * SearchSmem<P>::kBufStride;
    uint32_t bn = 0;  // entries in ibuf (owner; empty whenever the search is parked)
    uint64_t nE = 0, nS = 0, nP = 0;

    // Every thread reads `started` before the team's rank 0 may set it below,
    // so that all take the same branch (and the same number of barriers).
    const bool fresh = team.rd32(&st->started) == 0;
    team.sync();
    if (fresh) {
        if (cta == 0 && tid == 0) {
            const Key key0 = prob.start_key();
            const uint32_t aux0 = prob.start_aux();
            uint32_t s0;
            if (relax_key<P>(m.tab, m.mask, m.max_probe, key0, 0, kNone, &s0) == RELAX_FULL) {
                set_error(&st->error, ST_HASH_FULL);
            } else {
                P::set_link(m.tab + s0, kNone, aux0);
                uint32_t sz = 0;
                heap_push<P>(myheap, sz, prob.make_entry(prob.f_of(key0, 0, aux0), 0, s0, aux0));
                m.heap_size[myh] = sz;
                st->inserted = 1;
            }
            st->started = 1;
        }
        team.sync();
    } else if (owner) {
        // resuming: bring the shared top of this heap back from global memory
        const uint32_t sz = ldcg_u32(&m.heap_size[myh]);
        for (uint32_t i = 1; i <= topn && i <= sz; ++i) myheap.s[i] = P::load(gblock + i);
    }
    __syncthreads();

    uint32_t base = team.rd32(&st->base);
    uint64_t round = team.rd64(&st->round);
    uint64_t gbest = team.rd64(&st->goal_best);     // best goal f over the decided rounds
    uint64_t ins_total = team.rd64(&st->inserted);  // slots in use after the decided rounds
    uint32_t status = ST_RUNNING;
    uint32_t hs = owner ? ldcg_u32(&m.heap_size[myh]) : 0;  // this owner's heap size (private)
    // Candidates: two buffers by round parity (a CTA may append round r + 1's
    // while another still reads round r's), each one region per CTA (its
    // header record holds the count), so a relaxing warp claims room with a
    // shared-memory atomic and the CTA publishes one count per round.
    const uint64_t RR = cand_region_records<P>(H);
    uint32_t *const s_cnt = scratch + 36;  // this CTA's candidates this round
    uint32_t *const s_ins = scratch + 37;  // dedup slots it claimed this round
    uint32_t *const s_ins2 = scratch + 38;  // (kSort) slots claimed after the sort
    uint32_t *const ssm = reinterpret_cast<uint32_t *>(smem + SearchSmem<P>::sort_offset(H, L));
    unsigned long long *const wmins = reinterpret_cast<unsigned long long *>(scratch + 40);  // per owner warp
    // Push-phase staging: one entry per candidate of this CTA's share (at most
    // H * kMoves), then the C + 1 region offsets of the round's candidates
    // (the host keeps C < 32 H); it reuses the sift-down scratch, idle then.
    static_assert(2 * BrickHeap<P>::BE >= P::kMoves, "staging fits the sift scratch");
    // With split rounds the owners may still be sifting while the relaxers
    // stage, so the staging has its own room after the CTA's other shared
    // memory (bytes_split).
    E *const stage =
        split ? reinterpret_cast<E *>(smem + SearchSmem<P>::sort_offset(H, L)) : scr;
    uint32_t *const roff = reinterpret_cast<uint32_t *>(scr + (size_t)H * P::kMoves);

    for (uint64_t it = 0;; ++it) {
        const uint32_t r3 = (uint32_t)(round % 3);
        Cand *const half = m.cand + (size_t)(round & 1) * C * RR;
        Cand *const myreg = half + (size_t)cta * RR + 1;
        if (tid == 0) {
            *s_cnt = 0;
            *s_ins = 0;
            *s_ins2 = 0;
        }

        // ------------------------------------------------ phase 1: pop ---
        // The owner takes the root now and refills the hole later in the
        // round (pending_sift), off the path to the successors.
        bool pending_sift = false, have_last = false;
        E last;
        if (tid < owner_warps * 32u) {
            E e;
            uint32_t mv = 0;
            const bool have = owner && (hs > 0 || bn > 0);
            if (have) {
                uint32_t bi = 0;
                for (uint32_t j = 1; j < bn; ++j)
                    if (P::less(ibuf[j], ibuf[bi])) bi = j;
                if (hs > 0 && (bn == 0 || !P::less(ibuf[bi], myheap.s[1]))) {
                    e = myheap.s[1];
                    // the heap's last entry refills the root unless the
                    // buffer has a run to drain (below), whose least entry
                    // refills it instead
                    if (bn <= kBuf - P::kMoves) {
                        last = myheap.ld(hs);
                        have_last = true;
                    }
                    hs -= 1;
                    pending_sift = hs > 0;
                } else {
                    e = ibuf[bi];
                    ibuf[bi] = ibuf[bn - 1];
                    bn -= 1;
                }
            }
            const uint64_t ecost = have ? P::entry_cost(e) : kInfCost;
            const uint64_t wmin = warp_min_cost<P>(ecost);
            if (lane == 0) wmins[tid >> 5] = wmin;  // the CTA's minimum goes out once, below
            if (have) {
                Key key;
                uint64_t g;
                uint32_t aux;
                P::load_node(m.tab + e.slot, key, g, aux);
                // where the entry names its node (grids), the neighbourhood
                // reads go out beside the node record's, in one round trip
                uint32_t mv_pre = 0;
                if constexpr (P::kEntryKey) mv_pre = prob.entry_moves(e);
                const uint64_t fcur = prob.f_of(key, g, aux);
                if (fcur != ecost) {
                    // stale: the node was improved after this entry was pushed
                } else if (prob.is_goal(key)) {
                    atomic_min_cost<P>(&st->goal_min[r3], fcur);
                    st->goal_slot = e.slot;  // every goal pop names the same slot
                } else {
                    ++nE;
                    if constexpr (P::kEntryKey)
                        mv = mv_pre;
                    else
                        mv = prob.moves(key, aux);
                    pop[tid].key = key;
                    pop[tid].g = g;
                    pop[tid].aux = aux;
                    pop[tid].slot = e.slot;
                }
            }
            // exclusive prefix of successor counts: within the warp here,
            // warp offsets added after the barrier
            const uint32_t cnt = __popc(mv);
            uint32_t incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(kFull, incl, o);
                if (lane >= (uint32_t)o) incl += t;
            }
            if (owner) {
                pop[tid].mask = mv;
                pop[tid].excl = incl - cnt;
            }
            if (lane == 31) scratch[2 + (tid >> 5)] = incl;
        }
        __syncthreads();
        uint64_t cmin = kInfCost;  // the CTA's minimum popped f (thread 0)
        if (tid == 0) {
            uint32_t acc = 0;
            for (uint32_t w = 0; w < owner_warps; ++w) {
                const uint32_t t = scratch[2 + w];
                scratch[2 + w] = acc;
                acc += t;
                if (P::cost_cmp(wmins[w], cmin) < 0) cmin = wmins[w];
            }
            scratch[0] = acc;
        }
        __syncthreads();
        if (owner) pop[tid].excl += scratch[2 + (tid >> 5)];
        const uint32_t total = scratch[0];
        __syncthreads();
        // into the team's round minimum, off the pop's path (before the barrier)
        if (tid == 0 && cmin != kInfCost) atomic_min_cost<P>(&st->round_min[r3], cmin);

        // ------------------ phase 1: relax successors / refill heap roots ---
        // Owner chores of the round, while the other warps relax: refill the
        // root hole, then drain the insertion buffer down to kBuf - kMoves
        // entries (room for this round's pushes).
        // The buffer's run to drain (its largest entries: the small ones are
        // popped soon), down to room for this round's pushes.  An overflow
        // stops the search at this round's decision, so it is reported before
        // the owner arrives at the team barrier.
        uint32_t run = 0;
        if (owner) {
            run = bn > kBuf - P::kMoves ? bn - (kBuf - P::kMoves) : 0u;
            if (hs + run > m.hcap) {
                set_error(&st->err[r3], ST_HEAP_OVERFLOW);
                run = m.hcap > hs ? m.hcap - hs : 0u;
            }
        }
        const auto chores = [&]() {
            // the run to the buffer's end, its largest entry last
            for (uint32_t q = 0; q < run; ++q) {
                const uint32_t end = bn - 1 - q;
                uint32_t bx = 0;
                for (uint32_t j = 1; j <= end; ++j)
                    if (P::less(ibuf[bx], ibuf[j])) bx = j;
                const E e = ibuf[bx];
                ibuf[bx] = ibuf[end];
                ibuf[end] = e;
            }
            // A root taken from the heap is refilled by the run's least entry
            // (heapreplace): one sift-down serves the pop and one push, and
            // the heap's last entry stays where it is.  Without a run the
            // last entry refills it.
            const bool replace = pending_sift && run > 0;
            E top = last;
            if (replace) {
                top = ibuf[bn - run];
                hs += 1;
            } else if (pending_sift && !have_last) {
                top = myheap.ld(hs + 1);  // (a run cut short by an overflow)
            }
            const uint32_t rest = run - (replace ? 1u : 0u);
            // the rest's bottom brick is read while the sift-down runs (a
            // fresh bottom brick, at depth 0, needs no read)
            uint32_t pre = 0;
            if (rest && hs + 1 > topn) {
                uint32_t d;
                const uint32_t root = myheap.brick_root(hs + 1, &d);
                if (d > 0) {
                    myheap.fetch_async(root, 2);
                    pre = root;
                }
            }
            if (pending_sift) {
                const uint32_t fin = heap_sift_down<P>(myheap, hs, top);
                // the sift wrote into that brick: its copy is stale
                if (pre && fin > topn && myheap.brick_root(fin) == pre) {
                    cp_async_wait_all();
                    pre = 0;
                }
            }
            if (pre) cp_async_wait_all();
            if (rest) heap_push_run<P>(myheap, hs, ibuf + (bn - rest), rest, pre);
            bn -= run;
        };
        if (split) {
            // owner warps: arrive at the team barrier now, refill the heaps,
            // then wait for the staging (below)
            if (!relaxer) {
                team.early_arrive();
                if (owner) chores();
            }
        } else if (rfirst > 0 && owner) {
            chores();
        }
        if constexpr (kSort) {
            // every successor's record, at its number in the CTA's list
            if (relaxer) {
                for (uint32_t j = tid - rfirst; j < total; j += rthreads) {
                    uint32_t lo = 0, hi = H - 1;
                    while (lo < hi) {
                        const uint32_t mid = (lo + hi + 1) >> 1;
                        if (pop[mid].excl <= j)
                            lo = mid;
                        else
                            hi = mid - 1;
                    }
                    const PopInfo<Key> &pi = pop[lo];
                    const int move = (int)__fns(pi.mask, 0, (int)(j - pi.excl) + 1);
                    typename P::Succ sc;
                    prob.succ_begin(pi.key, pi.g, pi.aux, move, sc);
                    uint32_t naux;
                    uint64_t nf;
                    prob.succ_end(sc, pi.aux, move, naux, nf);
                    ++nS;
                    Cand c;
                    c.slot = (uint32_t)sc.key;
                    c.parent = pi.slot;
                    c.g = sc.g;
                    c.f = nf;
                    c.aux = naux;
                    c.pad = 0;
                    myreg[j] = c;
                }
            }
        } else if (relaxer) {  // (not kSort)
            const uint32_t rt = tid - rfirst;
            for (uint32_t b0 = 0; b0 < total; b0 += rthreads) {
                const uint32_t j = b0 + rt;
                bool improved = false, inserted = false;
                uint32_t nslot = 0, naux = 0, oslot = 0;
                uint64_t ng = 0, nf = 0;
                if (j < total) {
                    // source pop = largest h with excl[h] <= j (it has a successor)
                    uint32_t lo = 0, hi = H - 1;
                    while (lo < hi) {
                        const uint32_t mid = (lo + hi + 1) >> 1;
                        if (pop[mid].excl <= j)
                            lo = mid;
                        else
                            hi = mid - 1;
                    }
                    const PopInfo<Key> &pi = pop[lo];
                    const int move = (int)__fns(pi.mask, 0, (int)(j - pi.excl) + 1);
                    oslot = pi.slot;
                    typename P::Succ sc;
                    prob.succ_begin(pi.key, pi.g, pi.aux, move, sc);
                    ng = sc.g;
                    ++nS;
                    const int r = relax_key<P>(m.tab, m.mask, m.max_probe, sc.key, sc.g, oslot, &nslot, move);
                    prob.succ_end(sc, pi.aux, move, naux, nf);
                    if (r == RELAX_FULL) {
                        set_error(&st->err[r3], ST_HASH_FULL);
                    } else {
                        inserted = (r & RELAX_CLAIMED) != 0;
                        improved = (r & RELAX_IMPROVED) != 0;
                        // (link in the g word: the claimer stores the node's
                        // pattern parts, the same for every writer of the key)
                        if constexpr (P::kLink == LINK_IN_G)
                            if (inserted) P::set_link(m.tab + nslot, oslot, naux);
                    }
                }
                const uint32_t ib = __ballot_sync(kFull, inserted);
                if (ib && lane == (uint32_t)(__ffs(ib) - 1)) atomicAdd(s_ins, (uint32_t)__popc(ib));
                const uint32_t bal = __ballot_sync(kFull, improved);
                if (bal) {
                    const uint32_t leader = (uint32_t)(__ffs(bal) - 1);
                    uint32_t cbase = 0;
                    if (lane == leader) cbase = atomicAdd(s_cnt, (uint32_t)__popc(bal));
                    cbase = __shfl_sync(kFull, cbase, leader);
                    if (improved) {
                        Cand c;
                        c.slot = nslot;
                        c.parent = oslot;
                        c.g = ng;
                        c.f = nf;
                        c.aux = naux;
                        c.pad = 0;
                        myreg[cbase + __popc(bal & lanemask_lt())] = c;
                    }
                }
            }
        }
        if (rfirst == 0 && owner) chores();

        // publish this CTA's round: its candidate count and claimed slots
        const auto publish = [&]() {
            half[(size_t)cta * RR].slot = kSort ? total : *s_cnt;
            if (*s_ins) atomicAdd(&st->ins[r3], (unsigned long long)*s_ins);
            // the time slice is read by one thread of the team, so that all
            // threads take the same decision
            if (cta == 0 && m.deadline_ns) st->quit[r3] = globaltimer_ns() >= m.deadline_ns ? 1u : 0u;
        };
        if (!split) {
            __syncthreads();
            if (tid == 0) publish();
            team.sync();
        } else if (relaxer) {
            named_sync(2, rthreads);  // every relaxer's counts are in
            if (tid == rfirst) publish();
            team.relaxers_sync(T);
        } else {
            // Owner warps, chores done: the relaxers arrive at barrier 3 once
            // they have decided and staged the pushes (or stopped); then the
            // team barrier has completed too.
            named_sync(3, T);
            team.late_wait();
        }

        // -------------------------------------------------- decision ---
        // Every value read here was written before the barrier above and is
        // not written again before every CTA has read it (see TeamState), so
        // all threads decide alike.
        // the push phase's region counts, read beside the decision's words:
        // the one region this CTA takes, or (kSort) every region
        const uint32_t src = (uint32_t)((cta + round) % C);
        const uint32_t per = (C + T - 1) / T, rb = tid * per, re = min(rb + per, C);
        const uint32_t pre0 = kSort ? (rb < re ? ldcg_u32(&half[(size_t)rb * RR].slot) : 0u)
                                    : ldcg_u32(&half[(size_t)src * RR].slot);
        const uint32_t pre1 = kSort && rb + 1 < re ? ldcg_u32(&half[(size_t)(rb + 1) * RR].slot) : 0u;
        const uint64_t rmin = team.rd64(&st->round_min[r3]);
        const uint64_t gmin = team.rd64(&st->goal_min[r3]);
        if (P::cost_cmp(gmin, gbest) < 0) gbest = gmin;
        uint32_t err = team.rd32(&st->err[r3]);
        if (!err) err = team.rd32(&st->error);
        ins_total += team.rd64(&st->ins[r3]);
        if (!err && ins_total > m.max_inserted) err = ST_HASH_FULL;
        const bool pause = ins_total > m.grow_at || (m.deadline_ns && team.rd32(&st->quit[r3]));
        round += 1;
        if (err)
            status = err;
        else if (gbest != kInfCost && P::cost_cmp(gbest, rmin) <= 0)
            status = ST_OK;
        else if (rmin == kInfCost)
            status = ST_NO_SOLUTION;
        else if (round >= m.max_rounds)
            status = ST_ITER_LIMIT;
        if (status != ST_RUNNING) {
            if (split && relaxer) named_arrive(3, T);  // the owner warps wait there
            break;
        }

        // ---------------------------------------------------- phase 2 ---
        if (cta == 0 && tid == 0) {
            const uint32_t a = (r3 + 2) % 3;  // the round after next
            st->round_min[a] = kInfCost;
            st->goal_min[a] = kInfCost;
            st->ins[a] = 0;
            st->err[a] = 0;
            st->quit[a] = 0;
        }
        // This CTA's share of the round's candidates is the whole region of
        // CTA (c + round) mod C: the successors of that CTA's H pops, a
        // sample of the whole search (each CTA pops its own heaps' best), read
        // contiguously; the pairing rotates every round.  All threads check a
        // part of the share: a candidate is the slot's winner iff the slot's
        // g still equals its g; winners write prev/aux and are staged for
        // their heap's owner.
        uint32_t nshare = pre0;
        if constexpr (kSort) {
            // The round's candidates are numbered region by region: offsets of
            // the C regions (each thread sums `per` consecutive regions' counts).
            uint32_t mine = 0;
            for (uint32_t r = rb; r < re; ++r) {
                const uint32_t n = r == rb ? pre0 : r == rb + 1 ? pre1 : ldcg_u32(&half[(size_t)r * RR].slot);
                roff[r] = n;
                mine += n;
            }
            uint32_t ncand;
            uint32_t off = block_excl_scan(mine, scratch, &ncand);
            for (uint32_t r = rb; r < re; ++r) {
                const uint32_t n = roff[r];
                roff[r] = off;
                off += n;
            }
            __syncthreads();
            nshare = ncand > cta ? (ncand - cta + C - 1) / C : 0u;
            // the region record of the round's candidate number i
            const auto rec = [&](uint32_t i) -> const Cand * {
                uint32_t lo = 0, hi = C - 1;  // the last region starting at or before i
                while (lo < hi) {
                    const uint32_t mid = (lo + hi + 1) >> 1;
                    if (roff[mid] <= i)
                        lo = mid;
                    else
                        hi = mid - 1;
                }
                return half + (size_t)lo * RR + 1 + (i - roff[lo]);
            };
            // Sort the round's successors by key, then CTA c takes the sorted
            // positions c, c + C, ...; a position that starts a key's run
            // relaxes the run's least-g record (the first of equal g).
            const uint64_t nmax = (uint64_t)C * H * P::kMoves;
            const unsigned long long *sorted = team_radix_sort<P::kMoves>(
                team, ncand, m.sort_bits, [&](uint32_t i) { return ldcg_u32(&rec(i)->slot); }, m.sort_buf,
                m.sort_buf + nmax, m.sort_hist, ssm, &st->error);
            const uint32_t nxt = (r3 + 1) % 3;  // claims count toward the next round's decision
            uint32_t claimed = 0;
            for (uint32_t q = tid; q < nshare; q += T) {
                const uint32_t p = cta + C * q;
                const unsigned long long v = __ldcg(sorted + p);
                const uint32_t key = (uint32_t)(v >> 32);
                E e;
                e.slot = kNone;
                if (p == 0 || (uint32_t)(__ldcg(sorted + p - 1) >> 32) != key) {
                    uint32_t bi = (uint32_t)v;
                    Cand best = load_cand(rec(bi < ncand ? bi : 0));
                    for (uint32_t p2 = p + 1; p2 < ncand; ++p2) {
                        const unsigned long long v2 = __ldcg(sorted + p2);
                        if ((uint32_t)(v2 >> 32) != key) break;
                        const uint32_t i2 = (uint32_t)v2;
                        const Cand c2 = load_cand(rec(i2 < ncand ? i2 : 0));
                        if (P::cost_cmp(c2.g, best.g) < 0) best = c2;
                    }
                    uint32_t nslot = 0;
                    const int r = relax<P>(m.tab, m.mask, m.max_probe, key, best.g, best.parent, &nslot);
                    if (r == RELAX_FULL) {
                        set_error(&st->err[nxt], ST_HASH_FULL);
                    } else {
                        claimed += (r & RELAX_CLAIMED) ? 1u : 0u;
                        if (r & RELAX_IMPROVED) e = prob.make_entry(best.f, best.g, nslot, best.aux);
                    }
                }
                stage[q] = e;
            }
            if (claimed) atomicAdd(s_ins2, claimed);
            __syncthreads();
            if (tid == 0 && *s_ins2) atomicAdd(&st->ins[nxt], (unsigned long long)*s_ins2);
        }
        const Cand *const sreg = half + (size_t)src * RR + 1;
        // (split rounds: the relaxers stage, the owner warps are waiting)
        const uint32_t q0 = split ? tid - rfirst : tid, qstep = split ? rthreads : T;
        const uint32_t nstage = kSort || (split && !relaxer) ? 0u : nshare;
        for (uint32_t q = q0; q < nstage; q += qstep) {
            const Cand c = load_cand(sreg + q);
            E e = prob.make_entry(c.f, c.g, c.slot, c.aux);
            if constexpr (P::kLink == LINK_FIELD) {
                if (P::slot_g(m.tab + c.slot) == c.g)
                    P::set_link(m.tab + c.slot, c.parent, c.aux);
                else
                    e.slot = kNone;  // lost to a better writer
            }
            // (link in the key or g word: every candidate is pushed; one that
            // lost to a better writer of the round is a stale entry, dropped
            // when popped, and at most one candidate per slot carries its
            // final g)
            stage[q] = e;
        }
        if (!split)
            __syncthreads();
        else if (relaxer)
            named_arrive(3, T);
        // The share is dealt round-robin over the CTA's heaps (at most
        // kMoves per heap: the share is at most H * kMoves) into their
        // insertion buffers, which the relax phase left with room for kMoves.
        if (owner) {
            for (uint32_t q = (tid + base) % H; q < nshare; q += H) {
                const E e = stage[q];
                if (e.slot == kNone) continue;
                ibuf[bn++] = e;
                ++nP;
            }
        }
        base = (uint32_t)(((uint64_t)base + nshare) % H);
        if (pause || it + 1 >= budget) break;
    }

    // Persist the resumable state: the buffers go into the heaps, then the
    // sizes and the shared tops.  (The pushes use the sift scratch, which
    // the last push phase's staging shares: wait for every owner first.)
    __syncthreads();
    if (owner && status == ST_RUNNING) {
        while (bn > 0) {
            if (hs + 1 > m.hcap) {
                set_error(&st->error, ST_HEAP_OVERFLOW);  // reported by the next decision
                break;
            }
            heap_push<P>(myheap, hs, ibuf[--bn]);
        }
    }
    if (owner) {
        m.heap_size[myh] = hs;
        for (uint32_t i = 1; i <= topn && i <= hs; ++i) P::store(gblock + i, myheap.s[i]);
    }
    if (cta == 0 && tid == 0) {
        st->round = round;
        st->base = base;
        st->goal_best = gbest;
        st->inserted = ins_total;
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

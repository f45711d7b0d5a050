// Moving a paused search to a larger dedup table (plain engine and serving
// loop).  A search paused by ga_search (it returned ST_RUNNING at a round
// boundary, its insertion buffers drained into its heaps) names slots in
// three places: the slots' prev links, the heap entries and the team's goal
// slot.  Growth re-inserts every occupied slot into the empty larger table,
// recording old -> new in `map`, then rewrites all three.  The kernels have
// internal linkage: each translation unit that launches them has its own.
#pragma once
#include <cstdint>

#include "ga_device.cuh"
#include "ga_search.cuh"

namespace uastar {
namespace {

// Re-insert the occupied slots of `src` (n slots) into `dst` (mask + 1
// empty slots).  Keys are unique, so an insert only races other keys for an
// empty slot; prev is copied as is and rewritten by k_grow_links.  Wide:
// 16-byte keys (WideSlot layout), claimed with one 16-byte CAS.  PrevInKey:
// the key word is cell | prev << 32 (grids), hashed on the cell.
template <bool Wide, bool PrevInKey>
__global__ void k_grow_move(const Slot *src, uint64_t n, Slot *dst, uint64_t mask, uint32_t *map) {
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < n; s += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 a = __ldcg(reinterpret_cast<const uint4 *>(src + s));
        const unsigned long long key = ((unsigned long long)a.y << 32) | a.x;
        if (key == kEmptyKey) continue;
        const uint4 b = __ldcg(reinterpret_cast<const uint4 *>(src + s) + 1);
        uint64_t h;
        if constexpr (Wide) {
            const Key128 k{key, ((unsigned long long)a.w << 32) | a.z};
            h = key_hash(k) & mask;
            for (uint64_t probe = 0; probe <= mask; ++probe) {
                const KeyG old = cas128(dst + h, KeyG{kEmptyKey, kEmptyKey}, KeyG{k.lo, k.hi});
                if (old.key == kEmptyKey && old.g == kEmptyKey) break;
                h = (h + 1) & mask;
            }
        } else {
            h = mix64(PrevInKey ? key & 0xffffffffull : key) & mask;
            for (uint64_t probe = 0; probe <= mask; ++probe) {
                if (atomicCAS(&dst[h].key, kEmptyKey, key) == kEmptyKey) break;
                h = (h + 1) & mask;
            }
        }
        uint4 *d = reinterpret_cast<uint4 *>(dst + h);
        d[0] = make_uint4(a.x, a.y, a.z, a.w);  // key and g (narrow), key (wide)
        d[1] = b;                               // aux, prev (old index) and pad (narrow); g, aux, prev (wide)
        map[s] = (uint32_t)h;
    }
}

// Link: where the slots keep their parent link (SlotLink).
template <bool Wide, int Link>
__global__ void k_grow_links(const Slot *src, uint64_t n, Slot *dst, const uint32_t *map) {
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < n; s += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t w = __ldcg(&src[s].key);
        if (w == kEmptyKey) continue;
        if constexpr (Link == LINK_IN_KEY) {
            const uint32_t p = (uint32_t)(w >> 32);
            dst[map[s]].key = (w & 0xffffffffull) | (uint64_t)(p == kNone ? kNone : map[p]) << 32;
        } else if constexpr (Link == LINK_IN_G) {
            const uint64_t gw = __ldcg(&src[s].g);
            const uint32_t p = (uint32_t)gw;
            dst[map[s]].g = (gw & ~0xffffffffull) | (p == kNone ? kNone : map[p]);
        } else if constexpr (Wide) {
            const uint32_t p = __ldcg(&WideSlots::w(src + s)->prev);
            WideSlots::w(dst + map[s])->prev = p == kNone ? kNone : map[p];
        } else {
            const uint32_t p = __ldcg(&src[s].prev);
            dst[map[s]].prev = p == kNone ? kNone : map[p];
        }
    }
}

// One warp per heap: entries 1..size, the saved shared top first (heap
// indices <= 2^L - 1 at the head of the heap's block), then the bricks.
template <class P>
__global__ void k_grow_heaps(typename P::Entry *heaps, uint32_t stride, uint32_t L, const uint32_t *heap_size,
                             uint32_t k, const uint32_t *map, TeamState *st) {
    using E = typename P::Entry;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t topn = (1u << L) - 1u;
    for (uint32_t h = warp; h < k; h += nwarps) {
        E *gblock = heaps + (size_t)h * stride;
        const BrickHeap<P> bh{gblock + top_reserve<P>(L), nullptr, nullptr, L};
        const uint32_t sz = heap_size[h];
        for (uint32_t i = 1 + lane; i <= sz; i += 32) {
            E *q = i <= topn ? gblock + i : bh.g + bh.off(i);
            E e = P::load(q);
            e.slot = map[e.slot];
            P::store(q, e);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (st->goal_slot != kNone) st->goal_slot = map[st->goal_slot];
        st->barrier = 0;  // a grid team's next launch counts barriers from zero
    }
}

}  // namespace
}  // namespace uastar

// Plain engine: one instance per persistent cooperative launch, the whole GPU
// as one GA* team (k heaps = k threads), plus the C-ABI glue shared by all
// engines.  The search kernel is ga_search<> (ga_search.cuh) on a GridTeam.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "engine_internal.h"
#include "ga_device.cuh"
#include "ga_problems.cuh"
#include "ga_search.cuh"
#include "ga_grow.cuh"
#include "ga_ida.cuh"

using namespace uastar;

// ------------------------------------------------------------------ kernels ---
namespace uastar {

__global__ void k_fill_ff(uint4 *p, size_t n16) {
    const uint4 v = make_uint4(~0u, ~0u, ~0u, ~0u);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16;
         i += (size_t)gridDim.x * blockDim.x)
        p[i] = v;
}

template <class P, bool kSort = false>
__global__ void __launch_bounds__(512, 1) k_plain_search(P prob, SearchMem<typename P::Entry> m,
                                                      TeamState *st, uint64_t timeout_ns, uint32_t H) {
    extern __shared__ __align__(128) unsigned char smem[];
    GridTeam team{st, 0u, timeout_ns};
    ga_search<P, GridTeam, kSort>(prob, team, m, H, smem, ~0ull);
}

// The search kernel of a plain solve: the sorted-dedup variant exists for
// grids only.
template <class P> const void *plain_kernel(bool sorted) {
    if constexpr (std::is_same<P, GridProblem>::value)
        if (sorted) return (const void *)k_plain_search<P, true>;
    return (const void *)k_plain_search<P, false>;
}

// Stand-alone run of the search's team sort (uastar_sort_keys): the whole
// grid as one team sorts n keys (n <= gridDim.x * blockDim.x * 8) and writes
// the stable permutation.
__global__ void __launch_bounds__(256, 1) k_team_sort(const uint32_t *keys, uint32_t n, uint32_t bits,
                                                      unsigned long long *buf, uint32_t *hist, uint32_t *perm,
                                                      TeamState *st, uint64_t timeout_ns) {
    extern __shared__ __align__(128) unsigned char smem[];
    GridTeam team{st, 0u, timeout_ns};
    const unsigned long long *out = team_radix_sort<8>(
        team, n, bits, [&](uint32_t i) { return __ldg(keys + i); }, buf, buf + n, hist,
        reinterpret_cast<uint32_t *>(smem), &st->error);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        perm[i] = (uint32_t)__ldcg(out + i);
}

// The best open node of a paused puzzle search: the minimum entry (least f,
// then deepest) among the entries of the heaps' saved shared tops that are
// current (their f still matches the node's g), as key << 32 | slot into
// *best by atomicMin.  The heap roots are the per-heap minima, so this is the
// open list's minimum unless every root near it is stale.
template <int N>
__global__ void k_best_open(PuzzleProblem<N> prob, SearchMem<PuzzleEntry> m, uint32_t k,
                            unsigned long long *best) {
    const uint32_t topn = (1u << m.L) - 1u;
    const uint64_t total = (uint64_t)k * topn;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t h = (uint32_t)(t / topn), i = (uint32_t)(t % topn) + 1;
        if (i > __ldcg(&m.heap_size[h])) continue;
        const PuzzleEntry e = PuzzleProblem<N>::load(m.heaps + (size_t)h * m.stride + i);
        typename PuzzleProblem<N>::Key key;
        uint64_t g;
        uint32_t aux;
        PuzzleProblem<N>::load_node(m.tab + e.slot, key, g, aux);
        if (prob.f_of(key, g, aux) != PuzzleProblem<N>::entry_cost(e)) continue;  // stale
        atomicMin(best, ((unsigned long long)e.key << 32) | e.slot);
    }
}

// Round-latency floor of the plain engine's launch geometry: `rounds` rounds
// of one team barrier each.  With `tab` set, every thread first does one
// 16-byte atomicCAS on a pseudo-random slot of the dedup table and the next
// round's slot depends on what it returned (a dependent chain, like a relax
// that waits for its CAS); compare and swap values are the same word, so
// the table is never changed.
__global__ void __launch_bounds__(512, 1) k_round_floor(TeamState *st, uint64_t timeout_ns, Slot *tab,
                                                        uint64_t mask, uint32_t rounds) {
    GridTeam team{st, 0u, timeout_ns};
    uint64_t x = mix64((uint64_t)blockIdx.x * blockDim.x + threadIdx.x + 1);
    const KeyG probe{0x5A5A5A5A5A5A5A5Aull, 0x5A5A5A5A5A5A5A5Aull};
    for (uint32_t r = 0; r < rounds; ++r) {
        if (tab) {
            const KeyG seen = cas128(tab + (x & mask), probe, probe);
            x = mix64(x ^ seen.key ^ r);
        }
        team.sync();
        if (ldcg_u32(&st->error)) break;
    }
    if (x == 0) st->pad0_ = 1;  // keeps the chain live (x is never 0 in practice)
}

// Walk the prev chain from the goal slot (one thread: a pointer chase).
// Writes keys goal -> start; *len = count, or cap + 1 when truncated.
__global__ void k_walk(const Slot *tab, uint32_t goal_slot, unsigned long long *keys,
                       uint64_t cap, unsigned long long *len, int link) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    uint32_t s = goal_slot;
    uint64_t n = 0;
    while (s != kNone && n < cap) {
        uint64_t key;
        uint32_t prev;
        slot_key_prev(tab + s, link, key, prev);
        keys[n++] = key;
        s = prev;
    }
    *len = (s != kNone) ? cap + 1 : n;
}

// The same walk for 16-byte keys: two words (lo, hi) per board.
__global__ void k_walk_wide(const Slot *tab, uint32_t goal_slot, unsigned long long *keys, uint64_t cap,
                            unsigned long long *len) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    uint32_t s = goal_slot;
    uint64_t n = 0;
    while (s != kNone && n < cap) {
        const WideSlot *w = WideSlots::w(tab + s);
        keys[2 * n] = __ldcg(&w->lo);
        keys[2 * n + 1] = __ldcg(&w->hi);
        ++n;
        s = __ldcg(&w->prev);
    }
    *len = (s != kNone) ? cap + 1 : n;
}

int32_t fill_ff_async(uastar_engine *eng, void *p, size_t bytes, cudaStream_t stream) {
    const size_t n16 = bytes / 16;
    const int blocks = (int)std::min<size_t>((n16 + 255) / 256, (size_t)std::max(1, eng->sms * 8));
    k_fill_ff<<<std::max(1, blocks), 256, 0, stream>>>(static_cast<uint4 *>(p), n16);
    eng->launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? UASTAR_OK : fail_cuda(eng, e, "fill");
}

int32_t fail_cuda(uastar_engine *eng, cudaError_t e, const char *what) {
    eng->set_err(std::string(what) + ": " + cudaGetErrorString(e));
    return UASTAR_CUDA_ERROR;
}

}  // namespace uastar

namespace {

inline uint32_t next_pow2_u32(uint32_t v) {
    uint32_t p = 1;
    while (p < v) p <<= 1;
    return p;
}
inline int ceil_log2_u64(uint64_t v) {
    int l = 0;
    while ((1ull << l) < v) ++l;
    return l;
}
inline double now_ms() {
    return std::chrono::duration<double, std::milli>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

TeamState fresh_team_state() {
    TeamState s;
    team_state_init(&s);
    return s;
}

int32_t fill_ff(uastar_engine *eng, void *p, size_t bytes) {
    const size_t n16 = bytes / 16;
    const int blocks = std::max(1, eng->sms * 8);
    k_fill_ff<<<blocks, 256, 0, eng->stream>>>(static_cast<uint4 *>(p), n16);
    eng->launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? UASTAR_OK : fail_cuda(eng, e, "fill");
}

struct PlainOut {
    TeamState st;
    double kernel_ms;  // all search launches of the solve
    uint64_t slots;    // final table size
    int grows;         // in-place table growths
    SearchMem<PuzzleEntry> mem;  // the last attempt's memory (puzzle solves; used by the bounded mode)
    uint32_t k;        // heaps
};

// Run one instance with the whole GPU as the team.  Grows the dedup table /
// heaps and retries when they overflow and were auto-sized.
// Shared-memory heap levels: the largest L (at least 1) whose tops, pop
// records and brick scratch fit `budget` bytes, or exactly `levels` if > 0.
template <class P> uint32_t fit_levels(uint32_t H, int levels, size_t budget) {
    if (levels > 0) return (uint32_t)std::min(levels, 12);
    uint32_t best = 1;
    if (levels < 0) return best;
    for (uint32_t L = 1; L <= 12; ++L) {
        if (SearchSmem<P>::bytes(H, L) > budget) break;
        best = L;
    }
    return best;
}

// Heaps of the plain engine when the configuration leaves them to the
// engine: grids need few (their rounds are bounded by the path length, not
// by the work per round), puzzles gain throughput from more.
template <class P> uint32_t plain_heaps(const uastar_config &c) {
    return c.heaps > 0 ? (uint32_t)c.heaps : (P::kMoves >= 8 ? 8192u : 16384u);
}

// Moves a paused search's table to one 4x larger (k_grow_*), swapping it in
// as eng->tab.  Returns false (and changes nothing) if the memory is not there.
template <class P>
bool grow_table(uastar_engine *eng, SearchMem<typename P::Entry> &m, uint32_t k, TeamState *st) {
    const uint64_t old_n = m.mask + 1, new_n = old_n * 4;
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const size_t need = (new_n * sizeof(Slot) > eng->tab_next.bytes ? new_n * sizeof(Slot) : 0) +
                        (old_n * 4 > eng->grow_map.bytes ? old_n * 4 : 0);
    // at most 2^31 slots: every slot index stays below the no-parent mark kNone
    if (new_n > (1ull << 31)) return false;
    if (need + (256ull << 20) > free_b) {  // the batched engine's cached buffers give way
        release_batch_buffers(eng);
        cudaMemGetInfo(&free_b, &total_b);
        if (need + (256ull << 20) > free_b) return false;
    }
    if (eng->tab_next.ensure(new_n * sizeof(Slot)) != cudaSuccess) return false;
    if (eng->grow_map.ensure(old_n * 4) != cudaSuccess) return false;
    if (fill_ff(eng, eng->tab_next.p, new_n * sizeof(Slot)) != UASTAR_OK) return false;
    const int blocks = std::max(1, eng->sms * 8);
    Slot *src = m.tab, *dst = eng->tab_next.as<Slot>();
    uint32_t *map = eng->grow_map.as<uint32_t>();
    k_grow_move<P::kWide, P::kPrevInKey><<<blocks, 256, 0, eng->stream>>>(src, old_n, dst, new_n - 1, map);
    k_grow_links<P::kWide, P::kLink><<<blocks, 256, 0, eng->stream>>>(src, old_n, dst, map);
    k_grow_heaps<P><<<blocks, 256, 0, eng->stream>>>(m.heaps, m.stride, m.L, m.heap_size, k, map, st);
    eng->launches += 3;
    if (cudaGetLastError() != cudaSuccess) return false;
    std::swap(eng->tab, eng->tab_next);
    m.tab = eng->tab.as<Slot>();
    m.mask = new_n - 1;
    m.max_inserted = (uint64_t)((double)new_n * eng->cfg.max_load);
    return true;
}

// max_log2 > 0 caps the dedup table at 2^max_log2 slots (the memory-bounded
// mode): a search that fills it pauses near its load limit at a round
// boundary and returns with status ST_RUNNING, its heaps and table intact.
template <class P>
int32_t run_plain(uastar_engine *eng, const P &prob, int log2_auto, uint32_t stride_auto,
                  PlainOut *out, int max_log2 = 0) {
    using E = typename P::Entry;
    const uastar_config &c = eng->cfg;
    const uint32_t block = (uint32_t)c.block_threads;
    const uint32_t tph = c.threads_per_heap > 0 ? (uint32_t)c.threads_per_heap : 4u;
    const uint32_t H = std::max(1u, block / std::min(tph, block));
    const uint32_t nblocks = (plain_heaps<P>(c) + H - 1) / H;
    const uint32_t k = nblocks * H;
    int log2 = c.hash_log2_slots > 0 ? c.hash_log2_slots : log2_auto;
    if (log2 > 31) {
        eng->set_err("hash_log2_slots must be at most 31");
        return UASTAR_BAD_INPUT;
    }
    if (max_log2 > 0) log2 = std::min(log2, max_log2);
    uint32_t stride = c.heap_capacity > 0 ? next_pow2_u32((uint32_t)c.heap_capacity + 1) : stride_auto;
    if (c.dedup != 0 && c.dedup != 1) {
        eng->set_err("dedup must be 0 (table minimum) or 1 (sorted)");
        return UASTAR_BAD_INPUT;
    }
    bool sorted = false;
    uint32_t sort_bits = 0;
    if constexpr (std::is_same<P, GridProblem>::value) {
        sorted = c.dedup == 1;
        sort_bits = (uint32_t)std::max(1, ceil_log2_u64((uint64_t)prob.H * (uint64_t)prob.W));
    }
    const void *kfn = plain_kernel<P>(sorted);
    const size_t sort_extra = sorted ? sort_smem_bytes(block) + 16 : 0;

    // shared heap tops: as many levels as fit while the whole team stays
    // co-resident (ceil(nblocks / SMs) CTAs per SM)
    int smem_optin = 0, smem_sm = 0;
    cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, eng->device);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, eng->device);
    const int per_sm = (int)((nblocks + eng->sms - 1) / eng->sms);
    const size_t smem_budget = (size_t)std::max(8 * 1024, std::min(smem_optin, smem_sm / std::max(1, per_sm) - 2048));
    const uint32_t L = fit_levels<P>(H, c.heap_top_levels, smem_budget - sort_extra);
    const size_t smem = sorted ? SearchSmem<P>::bytes_sorted(H, L, block) : SearchSmem<P>::bytes(H, L);
    cudaError_t e = cudaSuccess;
    if (eng->smem_limit[kfn] < smem) {
        e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return fail_cuda(eng, e, "smem attribute");
        eng->smem_limit[kfn] = smem;
    }
    int max_active = 0;
    const auto occ_key = std::make_tuple(kfn, block, smem);
    const auto occ = eng->occupancy.find(occ_key);
    if (occ != eng->occupancy.end()) {
        max_active = occ->second;
    } else {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_active, kfn, (int)block, smem);
        if (e != cudaSuccess) return fail_cuda(eng, e, "occupancy");
        eng->occupancy[occ_key] = max_active;
    }
    if (nblocks + 1 > 32 * H) {  // the push phase keeps nblocks + 1 region offsets in shared memory
        eng->set_err("too many CTAs for the heaps per CTA (need CTAs < 32 * block_threads / threads_per_heap)");
        return UASTAR_BAD_INPUT;
    }
    if ((uint64_t)max_active * eng->sms < nblocks) {
        eng->set_err("heaps / (block_threads / threads_per_heap) exceed one co-resident wave of the GPU");
        return UASTAR_BAD_INPUT;
    }
    HeapGeometry<P> hg = heap_geometry<P>(L, stride);
    out->kernel_ms = 0;
    out->grows = 0;

    for (int attempt = 0; attempt < 6; ++attempt) {
        const uint64_t slots = 1ull << log2;
        const size_t tab_b = slots * sizeof(Slot);
        const size_t heap_b = (size_t)k * hg.stride * sizeof(E);
        const size_t cand_b = cand_records<P>(nblocks, H) * sizeof(Cand);
        // the batched engine's cached buffers give way to a table that does not fit
        if ((e = eng->tab.ensure(tab_b)) != cudaSuccess) {
            release_batch_buffers(eng);
            e = eng->tab.ensure(tab_b);
        }
        if (e != cudaSuccess) return fail_cuda(eng, e, "alloc table");
        if ((e = eng->heaps.ensure(heap_b)) != cudaSuccess) {
            release_batch_buffers(eng);
            e = eng->heaps.ensure(heap_b);
        }
        if (e != cudaSuccess) return fail_cuda(eng, e, "alloc heaps");
        if ((e = eng->heap_size.ensure((size_t)k * 4)) != cudaSuccess) return fail_cuda(eng, e, "alloc heap sizes");
        if ((e = eng->cand.ensure(cand_b)) != cudaSuccess) return fail_cuda(eng, e, "alloc candidates");
        if ((e = eng->team.ensure(sizeof(TeamState))) != cudaSuccess) return fail_cuda(eng, e, "alloc state");
        const uint64_t sort_n = (uint64_t)k * P::kMoves;  // a round's successors at most
        if (sorted && (e = eng->sortb.ensure(2 * sort_n * 8 + 256ull * (nblocks + 1) * 4)) != cudaSuccess)
            return fail_cuda(eng, e, "alloc sort buffers");

        int32_t rc = fill_ff(eng, eng->tab.p, tab_b);
        if (rc) return rc;
        if ((e = cudaMemsetAsync(eng->heap_size.p, 0, (size_t)k * 4, eng->stream)) != cudaSuccess)
            return fail_cuda(eng, e, "memset");
        TeamState init = fresh_team_state();
        if ((e = cudaMemcpyAsync(eng->team.p, &init, sizeof init, cudaMemcpyHostToDevice, eng->stream)) !=
            cudaSuccess)
            return fail_cuda(eng, e, "state upload");

        SearchMem<E> m;
        m.tab = eng->tab.as<Slot>();
        m.mask = slots - 1;
        m.max_inserted = (uint64_t)((double)slots * c.max_load);
        m.max_probe = 4096;
        m.heaps = eng->heaps.as<E>();
        m.stride = hg.stride;
        m.hcap = hg.hcap;
        m.L = L;
        m.heap_size = eng->heap_size.as<uint32_t>();
        m.cand = eng->cand.as<Cand>();
        m.max_rounds = (uint64_t)c.max_rounds;
        if (sorted) {
            m.sort_buf = eng->sortb.as<unsigned long long>();
            m.sort_hist = reinterpret_cast<uint32_t *>(m.sort_buf + 2 * sort_n);
            m.sort_bits = sort_bits;
        }
        // an auto-sized table grows in place (x4) when half full; at the cap
        // the search pauses instead, two rounds' worth of inserts short of
        // the load limit
        const bool auto_table = c.hash_log2_slots <= 0 || max_log2 > 0;
        const uint64_t full_at = m.max_inserted > 4ull * k * P::kMoves ? m.max_inserted - 4ull * k * P::kMoves : 0;
        auto pause_point = [&](uint64_t n) { return max_log2 > 0 && n >= (1ull << max_log2) ? full_at : n / 2; };
        m.grow_at = auto_table ? pause_point(slots) : ~0ull;
        TeamState *st = eng->team.as<TeamState>();
        uint64_t timeout_ns = (uint64_t)(c.wait_timeout_s * 1e9);
        P pr = prob;
        uint32_t h_arg = H;
        for (;;) {
            void *args[] = {&pr, &m, &st, &timeout_ns, &h_arg};
            cudaEventRecord(eng->ev0, eng->stream);
            e = cudaLaunchCooperativeKernel(kfn, dim3(nblocks), dim3(block), args, smem, eng->stream);
            if (e != cudaSuccess) return fail_cuda(eng, e, "cooperative launch");
            eng->launches++;
            cudaEventRecord(eng->ev1, eng->stream);
            if ((e = cudaMemcpyAsync(&out->st, st, sizeof(TeamState), cudaMemcpyDeviceToHost, eng->stream)) !=
                cudaSuccess)
                return fail_cuda(eng, e, "state download");
            if ((e = cudaStreamSynchronize(eng->stream)) != cudaSuccess) return fail_cuda(eng, e, "search");
            float ms = 0;
            cudaEventElapsedTime(&ms, eng->ev0, eng->ev1);
            out->kernel_ms += ms;
            if (out->st.status != ST_RUNNING) break;
            // paused: at the cap the caller takes over; otherwise grow
            if (max_log2 > 0 && m.mask + 1 >= (1ull << max_log2)) break;
            if (grow_table<P>(eng, m, k, st)) {
                out->grows += 1;
                const uint64_t n = m.mask + 1;
                const uint64_t fa = m.max_inserted > 4ull * k * P::kMoves ? m.max_inserted - 4ull * k * P::kMoves : 0;
                m.grow_at = max_log2 > 0 && n >= (1ull << max_log2) ? fa : n / 2;
            } else {
                m.grow_at = ~0ull;  // no room: carry on up to the load limit
                if ((e = cudaMemsetAsync(&st->barrier, 0, sizeof(uint32_t), eng->stream)) != cudaSuccess)
                    return fail_cuda(eng, e, "state reset");
            }
        }
        out->slots = m.mask + 1;
        if constexpr (std::is_same<E, PuzzleEntry>::value) out->mem = m;
        out->k = k;
        log2 = ceil_log2_u64(out->slots);
        if (out->st.status == ST_RUNNING) break;  // paused at the cap

        const uint32_t s = out->st.status;
        if (s != ST_HASH_FULL && s != ST_HEAP_OVERFLOW) break;
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        if (s == ST_HASH_FULL && auto_table && log2 + 2 <= 31 && (max_log2 <= 0 || log2 + 2 <= max_log2) &&
            (out->slots * 4 * sizeof(Slot)) < free_b + eng->tab.bytes) {
            log2 += 2;
            continue;
        }
        if (s == ST_HEAP_OVERFLOW && c.heap_capacity <= 0 && hg.hcap < (1u << 22) &&
            (size_t)k * hg.stride * 8 * sizeof(E) < free_b + eng->heaps.bytes) {
            hg = heap_geometry<P>(L, (uint64_t)hg.hcap * 8);
            continue;
        }
        break;
    }
    return UASTAR_OK;
}

int32_t walk_keys(uastar_engine *eng, uint32_t goal_slot, uint64_t cap, std::vector<uint64_t> *keys, int link) {
    cudaError_t e;
    const size_t need = (size_t)cap * 8 + 64;
    if ((e = eng->walk.ensure(need)) != cudaSuccess) return fail_cuda(eng, e, "alloc walk");
    unsigned long long *d_keys = eng->walk.as<unsigned long long>();
    unsigned long long *d_len = d_keys + cap;
    k_walk<<<1, 32, 0, eng->stream>>>(eng->tab.as<Slot>(), goal_slot, d_keys, cap, d_len, link);
    eng->launches++;
    if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda(eng, e, "walk launch");
    unsigned long long len = 0;
    if (cap <= 8192) {
        // short walks (puzzles): the whole buffer and its length in one copy
        std::vector<uint64_t> all(cap + 1);
        if ((e = cudaMemcpyAsync(all.data(), d_keys, (cap + 1) * 8, cudaMemcpyDeviceToHost, eng->stream)) !=
                cudaSuccess ||
            (e = cudaStreamSynchronize(eng->stream)) != cudaSuccess)
            return fail_cuda(eng, e, "walk");
        len = all[cap];
        if (len > cap) {
            eng->set_err("solution path longer than the walk buffer");
            return UASTAR_ARENA_FULL;
        }
        keys->assign(all.begin(), all.begin() + (ptrdiff_t)len);
        std::reverse(keys->begin(), keys->end());
        return UASTAR_OK;
    }
    if ((e = cudaMemcpyAsync(&len, d_len, 8, cudaMemcpyDeviceToHost, eng->stream)) != cudaSuccess)
        return fail_cuda(eng, e, "walk length");
    if ((e = cudaStreamSynchronize(eng->stream)) != cudaSuccess) return fail_cuda(eng, e, "walk");
    if (len > cap) {
        eng->set_err("solution path longer than the walk buffer");
        return UASTAR_ARENA_FULL;
    }
    keys->resize(len);
    if (len && (e = cudaMemcpyAsync(keys->data(), d_keys, len * 8, cudaMemcpyDeviceToHost, eng->stream)) !=
                   cudaSuccess)
        return fail_cuda(eng, e, "walk keys");
    if ((e = cudaStreamSynchronize(eng->stream)) != cudaSuccess) return fail_cuda(eng, e, "walk copy");
    std::reverse(keys->begin(), keys->end());
    return UASTAR_OK;
}

// Boards goal -> start of a 16-byte-key search, reversed to start -> goal.
int32_t walk_keys_wide(uastar_engine *eng, uint32_t goal_slot, uint64_t cap, std::vector<Key128> *keys) {
    cudaError_t e;
    if ((e = eng->walk.ensure((size_t)cap * 16 + 64)) != cudaSuccess) return fail_cuda(eng, e, "alloc walk");
    unsigned long long *d_keys = eng->walk.as<unsigned long long>();
    unsigned long long *d_len = d_keys + 2 * cap;
    k_walk_wide<<<1, 32, 0, eng->stream>>>(eng->tab.as<Slot>(), goal_slot, d_keys, cap, d_len);
    eng->launches++;
    if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda(eng, e, "walk launch");
    unsigned long long len = 0;
    if ((e = cudaMemcpyAsync(&len, d_len, 8, cudaMemcpyDeviceToHost, eng->stream)) != cudaSuccess)
        return fail_cuda(eng, e, "walk length");
    if ((e = cudaStreamSynchronize(eng->stream)) != cudaSuccess) return fail_cuda(eng, e, "walk");
    if (len > cap) {
        eng->set_err("solution path longer than the walk buffer");
        return UASTAR_ARENA_FULL;
    }
    keys->resize(len);
    if (len && (e = cudaMemcpyAsync(keys->data(), d_keys, len * 16, cudaMemcpyDeviceToHost, eng->stream)) !=
                   cudaSuccess)
        return fail_cuda(eng, e, "walk keys");
    if ((e = cudaStreamSynchronize(eng->stream)) != cudaSuccess) return fail_cuda(eng, e, "walk copy");
    std::reverse(keys->begin(), keys->end());
    return UASTAR_OK;
}

int32_t grid_load_impl(uastar_engine *eng, const uint64_t *words, int32_t H, int32_t W) {
    if (!eng) return UASTAR_BAD_INPUT;
    if (!words || H <= 0 || W <= 0 || (uint64_t)H * (uint64_t)W >= (1ull << 31)) {
        eng->set_err("grid must be non-empty with H*W < 2^31 cells (path cell ids are int32, as in the reference)");
        return UASTAR_BAD_INPUT;
    }
    const uint64_t cells = (uint64_t)H * W;
    const size_t bytes = ((cells + 63) / 64) * 8;
    cudaError_t e;
    if ((e = eng->bitmap.ensure(bytes + 16)) != cudaSuccess) return fail_cuda(eng, e, "alloc bitmap");
    if ((e = cudaMemcpyAsync(eng->bitmap.p, words, bytes, cudaMemcpyHostToDevice, eng->stream)) != cudaSuccess)
        return fail_cuda(eng, e, "bitmap upload");
    eng->gH = H;
    eng->gW = W;
    eng->grid_loaded = true;
    return UASTAR_OK;
}

int32_t grid_solve_impl(uastar_engine *eng, const uint64_t *host_words, int32_t sx, int32_t sy,
                        int32_t ex, int32_t ey, uastar_grid_result *out) {
    const double t0 = now_ms();
    std::memset(out, 0, sizeof(*out));
    eng->last_ok = false;
    eng->path_cached = false;
    eng->last_kind = UASTAR_KIND_GRID;
    if (!eng->grid_loaded) {
        eng->set_err("no grid loaded");
        return out->status = UASTAR_BAD_INPUT;
    }
    const int32_t H = eng->gH, W = eng->gW;
    if (sx < 0 || sx >= H || sy < 0 || sy >= W || ex < 0 || ex >= H || ey < 0 || ey >= W) {
        eng->set_err("start/goal out of range");
        return out->status = UASTAR_BAD_INPUT;
    }
    GridProblem prob;
    prob.bm = eng->bitmap.as<uint32_t>();
    prob.H = H;
    prob.W = W;
    prob.sx = sx;
    prob.sy = sy;
    prob.ex = ex;
    prob.ey = ey;
    const uint64_t cells = (uint64_t)H * W;
    const int log2_auto = std::min(28, std::max(20, ceil_log2_u64(cells) - 1));
    const uint32_t per_heap =
        (uint32_t)std::min<uint64_t>(8192, std::max<uint64_t>(64, 4 * cells / plain_heaps<GridProblem>(eng->cfg)));
    PlainOut po;
    int32_t rc = run_plain(eng, prob, log2_auto, next_pow2_u32(per_heap), &po);
    if (rc) return out->status = rc;
    const TeamState &st = po.st;
    out->status = (int32_t)st.status;
    out->expanded = (int64_t)st.expanded;
    out->generated = (int64_t)st.generated;
    out->pushed = (int64_t)st.pushed;
    out->rounds = (int64_t)st.round;
    out->table_used = (int64_t)st.inserted;
    out->kernel_ms = po.kernel_ms;
    out->table_grows = po.grows;
    if (st.status == ST_OK) {
        out->straight = (int64_t)(st.goal_best >> 32);
        out->diagonal = (int64_t)(st.goal_best & 0xffffffffu);
        out->cost_exact = (double)out->straight + (double)out->diagonal * std::sqrt(2.0);
        out->cost = (float)out->cost_exact;
        eng->last_ok = true;
        eng->last_goal_slot = st.goal_slot;
        eng->lsx = sx;
        eng->lsy = sy;
        eng->lex = ex;
        eng->ley = ey;
        // Path: walk prev pointers on the device, re-validate on the host.
        std::vector<uint64_t> keys;
        const uint64_t cap = std::min<uint64_t>(cells + 1, 1ull << 26);
        rc = walk_keys(eng, st.goal_slot, cap, &keys, GridProblem::kLink);
        if (rc) return out->status = rc;
        eng->path.assign(keys.size(), 0);
        for (size_t i = 0; i < keys.size(); ++i) eng->path[i] = (int32_t)keys[i];
        eng->path_cached = true;
        out->path_len = (int64_t)keys.size();
        // float32 g accumulated along the path in order, as the reference's
        // CPU solver computes it (CPU-solver.cpp:105)
        {
            const float sqrt2f = 1.4142135623731f;
            float fc = 0.0f;
            for (size_t i = 1; i < eng->path.size(); ++i) {
                const int64_t u = eng->path[i - 1], v = eng->path[i];
                const bool diag = (u / W != v / W) && (u % W != v % W);
                fc = fc + (diag ? sqrt2f : 1.0f);
            }
            out->cost = fc;
        }
        if (host_words) {
            int64_t a = 0, b = 0;
            float fc = 0;
            if (uastar_validate_grid_path(host_words, H, W, sx, sy, ex, ey, eng->path.data(),
                                          (int64_t)eng->path.size(), &a, &b, &fc) != UASTAR_OK ||
                a != out->straight || b != out->diagonal) {
                eng->set_err("engine returned a path that fails host validation");
                eng->last_ok = false;
                return out->status = UASTAR_CUDA_ERROR;
            }
            out->cost = fc;
        }
    } else if (st.status == ST_RUNNING) {
        eng->set_err("search kernel ended without a status");
        out->status = UASTAR_CUDA_ERROR;
    }
    out->solve_ms = now_ms() - t0;
    return out->status;
}

bool board_ok(int n, const uint8_t *tiles) {
    int seen = 0;
    for (int i = 0; i < n * n; ++i) {
        if (tiles[i] >= n * n || (seen >> tiles[i] & 1)) return false;
        seen |= 1 << tiles[i];
    }
    return true;
}

template <int N>
int32_t puzzle_solve_n(uastar_engine *eng, const uint8_t *tiles, PlainOut *po) {
    PuzzleProblem<N> prob;
    prob.pdb = eng->pdb[N].as<uint8_t>();
    prob.start = pack_board(N, tiles);
    prob.goal = PuzzleProblem<N>::goal_key();
    const int log2_start = eng->puzzle_log2_start > 0 ? eng->puzzle_log2_start : (N == 3 ? 20 : 22);
    return run_plain(eng, prob, log2_start, N == 3 ? 1024 : 16383, po);
}

// 5x5: 16-byte keys (PuzzleProblem<5>)
template <>
int32_t puzzle_solve_n<5>(uastar_engine *eng, const uint8_t *tiles, PlainOut *po) {
    PuzzleProblem<5> prob;
    prob.pdb = eng->pdb[5].as<uint8_t>();
    prob.start = PuzzleProblem<5>::pack(tiles);
    prob.goal = PuzzleProblem<5>::goal_key();
    return run_plain(eng, prob, 22, 16383, po);
}

// Boards (tiles per cell) along the prev chain ending at `slot`, start first.
template <int N>
int32_t walk_boards(uastar_engine *eng, uint32_t slot, std::vector<std::vector<uint8_t>> *boards) {
    boards->clear();
    if constexpr (N == 5) {
        std::vector<Key128> keys;
        if (int32_t rc = walk_keys_wide(eng, slot, 4096, &keys)) return rc;
        for (const Key128 &k : keys) {
            std::vector<uint8_t> b(25);
            for (int c = 0; c < 25; ++c) b[c] = (uint8_t)PuzzleProblem<5>::field(k, c);
            boards->push_back(b);
        }
    } else {
        std::vector<uint64_t> keys;
        if (int32_t rc = walk_keys(eng, slot, 4096, &keys, PuzzleProblem<4>::kLink)) return rc;
        for (uint64_t k : keys) {
            std::vector<uint8_t> b(N * N);
            for (int c = 0; c < N * N; ++c) b[c] = (uint8_t)((k >> (4 * c)) & 15);
            boards->push_back(b);
        }
    }
    return UASTAR_OK;
}

// Moves (0..3, the reference's DX/DY order) between consecutive boards.
void boards_to_moves(int n, const std::vector<std::vector<uint8_t>> &boards, std::vector<int32_t> *moves) {
    auto blank = [n](const std::vector<uint8_t> &b) {
        for (int c = 0; c < n * n; ++c)
            if (b[c] == 0) return c;
        return -1;
    };
    for (size_t i = 1; i < boards.size(); ++i) {
        const int d = blank(boards[i]) - blank(boards[i - 1]);
        moves->push_back(d == n ? 0 : d == -n ? 1 : d == 1 ? 2 : 3);
    }
}

// ---- exact phase of the memory-bounded mode: IDA* passes (ga_ida.cuh) ----
// A board on the host: tiles, blank cell, the move that reached it (+1) and
// the moves from the start (2 bits each, first lowest).
struct HostBoard {
    uint8_t b[25];
    int8_t blank;
    uint8_t last;
    uint64_t prefix;
};

// Blank move mv (0..3 = (+1,0), (-1,0), (0,+1), (0,-1) in (row, column), the
// reference's DX/DY) on an n x n board; false if it leaves the board.
template <int N> bool host_blank_move(HostBoard &h, int mv) {
    const int bx = h.blank / N, by = h.blank % N;
    const int nx = bx + (mv == 0) - (mv == 1), ny = by + (mv == 2) - (mv == 3);
    if (nx < 0 || nx >= N || ny < 0 || ny >= N) return false;
    const int q = nx * N + ny;
    h.b[h.blank] = h.b[q];
    h.b[q] = 0;
    h.blank = (int8_t)q;
    return true;
}

template <int N> bool host_is_goal(const uint8_t *b) {
    for (int i = 0; i < N * N; ++i)
        if (b[i] != (i + 1) % (N * N)) return false;
    return true;
}

// The start's search tree cut at the first depth with at least `want` nodes
// (at most max_depth <= 32), without moves that undo the previous one (the
// search prunes those too).  A goal met on the way ends the cut: every
// shorter move sequence was enumerated before it, so its depth is optimal.
template <int N>
void ida_roots(const uint8_t *tiles, size_t want, int max_depth, std::vector<IdaRoot> *roots,
               std::vector<int32_t> *goal_moves, bool *goal) {
    std::vector<HostBoard> cur(1), next;
    HostBoard &s0 = cur[0];
    std::memset(&s0, 0, sizeof s0);
    std::memcpy(s0.b, tiles, N * N);
    for (int i = 0; i < N * N; ++i)
        if (!tiles[i]) s0.blank = (int8_t)i;
    *goal = host_is_goal<N>(tiles);
    if (*goal) return;
    for (int d = 0; d < max_depth && cur.size() < want; ++d) {
        next.clear();
        next.reserve(cur.size() * 3);
        for (const HostBoard &h : cur)
            for (int mv = 0; mv < 4; ++mv) {
                if (h.last && mv == ((h.last - 1) ^ 1)) continue;
                HostBoard m = h;
                if (!host_blank_move<N>(m, mv)) continue;
                m.last = (uint8_t)(mv + 1);
                m.prefix = h.prefix | ((uint64_t)mv << (2 * d));
                if (host_is_goal<N>(m.b)) {
                    *goal = true;
                    goal_moves->clear();
                    for (int j = 0; j <= d; ++j) goal_moves->push_back((int32_t)((m.prefix >> (2 * j)) & 3));
                    return;
                }
                next.push_back(m);
            }
        cur.swap(next);
        if (cur.size() >= want || d + 1 >= max_depth) {
            roots->resize(cur.size());
            for (size_t i = 0; i < cur.size(); ++i) {
                IdaRoot &r = (*roots)[i];
                if constexpr (N == 5) {
                    const Key128 k = PuzzleProblem<5>::pack(cur[i].b);
                    r.lo = k.lo;
                    r.hi = k.hi;
                } else {
                    r.lo = pack_board(N, cur[i].b);
                    r.hi = 0;
                }
                r.g = (uint32_t)(d + 1);
                r.last = cur[i].last;
                r.prefix = cur[i].prefix;
            }
            return;
        }
    }
}

// IDA* passes from the lower bound lb up to the length ub of the solution
// in hand, for at most budget_ms.  A pass that finds a goal writes the
// optimal moves; one that completes without a goal raises out->lower_bound
// to its next threshold; reaching ub proves the solution in hand optimal.
template <int N>
int32_t ida_exact(uastar_engine *eng, const uint8_t *tiles, int32_t lb, int32_t ub, double budget_ms,
                  std::vector<int32_t> *moves, uastar_bounded_result *out) {
    constexpr int kMaxDepth = N == 3 ? 48 : N == 4 ? 100 : 200;
    const double t0 = now_ms();
    std::vector<IdaRoot> roots;
    std::vector<int32_t> goal_moves;
    bool goal = false;
    ida_roots<N>(tiles, 1u << 18, 24, &roots, &goal_moves, &goal);
    if (goal) {  // the cut met the goal first: that is the optimum
        *moves = goal_moves;
        out->lower_bound = (int32_t)goal_moves.size();
        out->exact_optimal = 1;
        out->exact_ms = now_ms() - t0;
        return UASTAR_OK;
    }
    const size_t head = (sizeof(IdaPass) + 255) & ~(size_t)255;
    cudaError_t e;
    if ((e = eng->ida.ensure(head + roots.size() * sizeof(IdaRoot))) != cudaSuccess) return fail_cuda(eng, e, "alloc ida");
    IdaPass *d_pass = eng->ida.as<IdaPass>();
    IdaRoot *d_roots = reinterpret_cast<IdaRoot *>(eng->ida.as<unsigned char>() + head);
    if ((e = cudaMemcpyAsync(d_roots, roots.data(), roots.size() * sizeof(IdaRoot), cudaMemcpyHostToDevice,
                             eng->stream)) != cudaSuccess)
        return fail_cuda(eng, e, "ida roots");
    PuzzleProblem<N> prob;
    prob.pdb = eng->pdb[N].as<uint8_t>();
    prob.goal = PuzzleProblem<N>::goal_key();
    prob.start = prob.goal;
    uint32_t t = (uint32_t)std::max(lb, 0);
    bool optimal = false;
    while (t < (uint32_t)ub) {
        const double left_ms = budget_ms - (now_ms() - t0);
        if (left_ms <= 0) break;
        IdaPass init;
        std::memset(&init, 0, sizeof init);
        init.min_exceed = ~0u;
        if ((e = cudaMemcpyAsync(d_pass, &init, sizeof init, cudaMemcpyHostToDevice, eng->stream)) != cudaSuccess)
            return fail_cuda(eng, e, "ida state");
        // threads read the device clock at their start: the pass ends
        // `left_ms` after it began
        k_ida_pass<PuzzleProblem<N>, kMaxDepth><<<std::max(1, eng->sms * 8), 128, 0, eng->stream>>>(
            prob, d_roots, (uint32_t)roots.size(), t, d_pass, (unsigned long long)(left_ms * 1e6));
        eng->launches++;
        if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda(eng, e, "ida launch");
        IdaPass res;
        if ((e = cudaMemcpyAsync(&res, d_pass, sizeof res, cudaMemcpyDeviceToHost, eng->stream)) != cudaSuccess ||
            (e = cudaStreamSynchronize(eng->stream)) != cudaSuccess)
            return fail_cuda(eng, e, "ida pass");
        out->exact_passes += 1;
        out->exact_nodes += (int64_t)res.nodes;
        if (res.found) {
            const IdaRoot &r = roots[res.found_root];
            moves->clear();
            for (uint32_t j = 0; j < r.g; ++j) moves->push_back((int32_t)((r.prefix >> (2 * j)) & 3));
            for (uint32_t j = 0; j < res.found_len; ++j) moves->push_back((int32_t)res.moves[j]);
            out->lower_bound = (int32_t)moves->size();
            optimal = true;
            break;
        }
        if (res.stopped) break;  // out of time (or a subtree deeper than the stack): t stays the bound
        if (res.min_exceed == ~0u) break;  // nothing cut off and no goal: cannot happen on a solvable board
        t = res.min_exceed;
        out->lower_bound = std::max(out->lower_bound, (int32_t)std::min<uint32_t>(t, (uint32_t)ub));
    }
    if (!optimal && t >= (uint32_t)ub) {
        out->lower_bound = ub;  // every shorter solution was ruled out
        optimal = true;
    }
    out->exact_optimal = optimal ? 1 : 0;
    out->exact_ms = now_ms() - t0;
    return UASTAR_OK;
}

// Memory-bounded solve: segments of exact GA*, each with the table capped.
// A segment that fills the table pauses; the open list's minimum f then is
// a lower bound on the remaining optimum (admissible h: every optimal path
// crosses the open list), the search commits to the open node holding it
// (least f, deepest) and the next segment starts there.  The first segment's
// bound is a lower bound on the whole puzzle's optimum.
template <int N>
int32_t puzzle_bounded_n(uastar_engine *eng, const uint8_t *tiles, int max_log2, uastar_bounded_result *out,
                         std::vector<int32_t> *moves) {
    uint8_t cur[25];
    std::memcpy(cur, tiles, N * N);
    cudaError_t e;
    // Where the segments cannot go on (their limit, or no open node to
    // commit to), the exact phase still runs from the first bound, with no
    // solution in hand; failing it too, the segments' status stands.
    const auto fallback = [&](int32_t status, const char *why) -> int32_t {
        if (eng->cfg.exact_ms >= 0) {
            moves->clear();
            const int32_t rc2 = ida_exact<N>(eng, tiles, out->lower_bound, 1 << 30,
                                             eng->cfg.exact_ms > 0 ? (double)eng->cfg.exact_ms : 3000.0, moves, out);
            if (rc2 != UASTAR_OK) return rc2;
            if (out->exact_optimal) return UASTAR_OK;
        }
        eng->set_err(why);
        return status;
    };
    for (int seg = 0; seg < 256; ++seg) {
        PuzzleProblem<N> prob;
        prob.pdb = eng->pdb[N].as<uint8_t>();
        if constexpr (N == 5)
            prob.start = PuzzleProblem<5>::pack(cur);
        else
            prob.start = pack_board(N, cur);
        prob.goal = PuzzleProblem<N>::goal_key();
        PlainOut po;
        int32_t rc = run_plain(eng, prob, std::min(N == 3 ? 20 : 22, max_log2), N == 3 ? 1024 : 16383, &po, max_log2);
        if (rc) return rc;
        out->segments = seg + 1;
        out->expanded += (int64_t)po.st.expanded;
        out->generated += (int64_t)po.st.generated;
        out->kernel_ms += po.kernel_ms;
        std::vector<std::vector<uint8_t>> boards;
        if (po.st.status == ST_OK) {
            if (seg == 0) out->lower_bound = (int32_t)po.st.goal_best;
            if ((rc = walk_boards<N>(eng, po.st.goal_slot, &boards))) return rc;
            boards_to_moves(N, boards, moves);
            // more than one segment: the exact phase, from the first
            // segment's bound up to this solution's length
            if (seg > 0 && eng->cfg.exact_ms >= 0)
                return ida_exact<N>(eng, tiles, out->lower_bound, (int32_t)moves->size(),
                                    eng->cfg.exact_ms > 0 ? (double)eng->cfg.exact_ms : 3000.0, moves, out);
            return UASTAR_OK;
        }
        if (po.st.status != ST_RUNNING) return (int32_t)po.st.status;
        // paused with the table full: commit to the best open node
        if ((e = eng->walk.ensure(4096 * 8 + 64)) != cudaSuccess) return fail_cuda(eng, e, "alloc walk");
        unsigned long long *d_best = eng->walk.as<unsigned long long>();
        const unsigned long long none = ~0ull;
        cudaMemcpyAsync(d_best, &none, 8, cudaMemcpyHostToDevice, eng->stream);
        k_best_open<N><<<std::max(1, eng->sms * 4), 256, 0, eng->stream>>>(prob, po.mem, po.k, d_best);
        eng->launches++;
        unsigned long long best = ~0ull;
        cudaMemcpyAsync(&best, d_best, 8, cudaMemcpyDeviceToHost, eng->stream);
        if ((e = cudaStreamSynchronize(eng->stream)) != cudaSuccess) return fail_cuda(eng, e, "best open node");
        if (best == ~0ull) {
            return fallback(UASTAR_HASH_FULL, "bounded search: no current open node at the memory bound");
        }
        const uint32_t f = (uint32_t)(best >> 48);  // entry key = f << 16 | (0xffff - g)
        if (seg == 0) out->lower_bound = (int32_t)f;
        if ((rc = walk_boards<N>(eng, (uint32_t)best, &boards))) return rc;
        if (boards.size() < 2) {
            return fallback(UASTAR_HASH_FULL, "bounded search: the best open node is the start");
        }
        boards_to_moves(N, boards, moves);
        std::memcpy(cur, boards.back().data(), N * N);
    }
    return fallback(UASTAR_ITER_LIMIT, "bounded search: segment limit reached");
}

}  // namespace

// ------------------------------------------------------------------ C ABI ---
extern "C" {

const char *uastar_build_info(void) {
    return "uastar_gb300 GA* engine, built for sm_103a";
}

uastar_engine *uastar_create(int32_t ordinal, const uastar_config *cfg) {
    auto *eng = new uastar_engine();
    eng->device = ordinal;
    if (cfg) eng->cfg = *cfg;
    uastar_config &c = eng->cfg;
    if (c.heaps < 0) c.heaps = 0;  // 0: chosen per problem kind (plain_heaps)
    if (c.block_threads <= 0) c.block_threads = 256;
    c.block_threads = std::max(32, std::min(512, (c.block_threads + 31) / 32 * 32));
    if (!(c.max_load > 0.0 && c.max_load < 1.0)) c.max_load = 0.8;
    if (c.max_rounds <= 0) c.max_rounds = 1ll << 31;
    if (!(c.wait_timeout_s > 0.0)) c.wait_timeout_s = 10.0;
    cudaError_t e = cudaSetDevice(ordinal);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&eng->sms, cudaDevAttrMultiProcessorCount, ordinal);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&eng->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&eng->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&eng->ev1);
    if (e != cudaSuccess) {
        delete eng;
        return nullptr;
    }
    eng->stream = eng->own_stream;
    return eng;
}

void uastar_destroy(uastar_engine *eng) {
    if (!eng) return;
    if (eng->serve) uastar_serve_stop(eng, 0.0, nullptr);
    cudaSetDevice(eng->device);
    cudaStreamSynchronize(eng->stream);
    for (DevBuf *b : {&eng->tab, &eng->heaps, &eng->heap_size, &eng->cand, &eng->team, &eng->walk,
                      &eng->tab_next, &eng->grow_map, &eng->sortb,
                      &eng->bitmap, &eng->b_desc, &eng->b_out, &eng->b_queue, &eng->b_bitmaps,
                      &eng->b_tab, &eng->b_heaps, &eng->b_hsize, &eng->b_cand, &eng->b_walk,
                      &eng->b_walklen, &eng->b_cstate, &eng->b_cnext})
        b->release();
    for (auto &b : eng->pdb) b.release();
    for (auto &kv : eng->b_graphs) cudaGraphExecDestroy(kv.second);
    if (eng->ev0) cudaEventDestroy(eng->ev0);
    if (eng->ev1) cudaEventDestroy(eng->ev1);
    if (eng->own_stream) cudaStreamDestroy(eng->own_stream);
    delete eng;
}

const char *uastar_last_error(const uastar_engine *eng) { return eng ? eng->err.c_str() : "null engine"; }

int32_t uastar_sort_keys(uastar_engine *eng, const uint32_t *keys, int64_t n, int32_t key_bits, uint32_t *perm) {
    if (!eng) return UASTAR_BAD_INPUT;
    constexpr uint32_t T = 256, kPer = 8;
    const uint64_t C = (uint64_t)std::max(1, eng->sms);
    if (n < 0 || (n > 0 && (!keys || !perm)) || key_bits < 0 || key_bits > 32) {
        eng->set_err("sort: bad arguments");
        return UASTAR_BAD_INPUT;
    }
    if ((uint64_t)n > C * T * kPer) {
        eng->set_err("sort: more than 2048 keys per SM");
        return UASTAR_BAD_INPUT;
    }
    const uint32_t bits = key_bits == 0 ? 32u : (uint32_t)key_bits;
    if (bits < 32)
        for (int64_t i = 0; i < n; ++i)
            if (keys[i] >> bits) {
                eng->set_err("sort: a key has bits above key_bits");
                return UASTAR_BAD_INPUT;
            }
    if (n == 0) return UASTAR_OK;
    cudaSetDevice(eng->device);
    const size_t nn = (size_t)n;
    const size_t bytes = nn * 4 + nn * 4 + 2 * nn * 8 + 256 * (C + 1) * 4 + 64;
    cudaError_t e;
    if ((e = eng->sortb.ensure(bytes)) != cudaSuccess) return fail_cuda(eng, e, "alloc sort");
    if ((e = eng->team.ensure(sizeof(TeamState))) != cudaSuccess) return fail_cuda(eng, e, "alloc state");
    unsigned long long *buf = eng->sortb.as<unsigned long long>();
    uint32_t *d_keys = reinterpret_cast<uint32_t *>(buf + 2 * nn);
    uint32_t *d_perm = d_keys + nn;
    uint32_t *hist = d_perm + nn;
    TeamState *st = eng->team.as<TeamState>();
    TeamState init = fresh_team_state();
    if ((e = cudaMemcpyAsync(st, &init, sizeof init, cudaMemcpyHostToDevice, eng->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_keys, keys, nn * 4, cudaMemcpyHostToDevice, eng->stream)) != cudaSuccess)
        return fail_cuda(eng, e, "sort upload");
    uint32_t n32 = (uint32_t)n, bits_arg = bits;
    uint64_t timeout_ns = (uint64_t)(eng->cfg.wait_timeout_s * 1e9);
    void *args[] = {&d_keys, &n32, &bits_arg, &buf, &hist, &d_perm, &st, &timeout_ns};
    e = cudaLaunchCooperativeKernel((const void *)k_team_sort, dim3((unsigned)C), dim3(T), args,
                                    sort_smem_bytes(T), eng->stream);
    if (e != cudaSuccess) return fail_cuda(eng, e, "sort launch");
    eng->launches++;
    uint32_t err = 0;
    if ((e = cudaMemcpyAsync(perm, d_perm, nn * 4, cudaMemcpyDeviceToHost, eng->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(&err, &st->error, 4, cudaMemcpyDeviceToHost, eng->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(eng->stream)) != cudaSuccess)
        return fail_cuda(eng, e, "sort");
    if (err) {
        eng->set_err("sort: a team barrier gave up");
        return UASTAR_TIMEOUT;
    }
    return UASTAR_OK;
}

int32_t uastar_round_floor(uastar_engine *eng, int32_t rounds, double *us_barrier, double *us_cas_barrier) {
    if (!eng || rounds <= 0 || rounds > (1 << 20)) return UASTAR_BAD_INPUT;
    cudaSetDevice(eng->device);
    const uastar_config &c = eng->cfg;
    const uint32_t block = (uint32_t)c.block_threads;
    const uint32_t tph = c.threads_per_heap > 0 ? (uint32_t)c.threads_per_heap : 4u;
    const uint32_t H = std::max(1u, block / std::min(tph, block));
    const uint32_t nblocks = (plain_heaps<GridProblem>(c) + H - 1) / H;
    int max_active = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_active, (const void *)k_round_floor,
                                                                  (int)block, 0);
    if (e != cudaSuccess) return fail_cuda(eng, e, "occupancy");
    if ((uint64_t)max_active * eng->sms < nblocks) {
        eng->set_err("round floor: the launch geometry exceeds one co-resident wave");
        return UASTAR_BAD_INPUT;
    }
    // a table larger than L2, so that the CAS is a memory round trip
    const uint64_t slots = std::max<uint64_t>(1ull << 26, eng->tab.bytes / sizeof(Slot));
    if ((e = eng->tab.ensure(slots * sizeof(Slot))) != cudaSuccess) return fail_cuda(eng, e, "alloc table");
    if ((e = eng->team.ensure(sizeof(TeamState))) != cudaSuccess) return fail_cuda(eng, e, "alloc state");
    uint64_t n = 1;
    while (n * 2 <= eng->tab.bytes / sizeof(Slot)) n *= 2;
    TeamState *st = eng->team.as<TeamState>();
    uint64_t timeout_ns = (uint64_t)(c.wait_timeout_s * 1e9);
    double out[2] = {0, 0};
    for (int mode = 0; mode < 2; ++mode) {
        TeamState init = fresh_team_state();
        if ((e = cudaMemcpyAsync(st, &init, sizeof init, cudaMemcpyHostToDevice, eng->stream)) != cudaSuccess)
            return fail_cuda(eng, e, "state upload");
        Slot *tab = mode ? eng->tab.as<Slot>() : nullptr;
        uint64_t mask = n - 1;
        uint32_t r = (uint32_t)rounds;
        void *args[] = {&st, &timeout_ns, &tab, &mask, &r};
        cudaEventRecord(eng->ev0, eng->stream);
        e = cudaLaunchCooperativeKernel((const void *)k_round_floor, dim3(nblocks), dim3(block), args, 0,
                                        eng->stream);
        if (e != cudaSuccess) return fail_cuda(eng, e, "round floor launch");
        eng->launches++;
        cudaEventRecord(eng->ev1, eng->stream);
        uint32_t err = 0;
        if ((e = cudaMemcpyAsync(&err, &st->error, 4, cudaMemcpyDeviceToHost, eng->stream)) != cudaSuccess ||
            (e = cudaStreamSynchronize(eng->stream)) != cudaSuccess)
            return fail_cuda(eng, e, "round floor");
        if (err) {
            eng->set_err("round floor: a team barrier gave up");
            return UASTAR_TIMEOUT;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, eng->ev0, eng->ev1);
        out[mode] = 1e3 * ms / rounds;
    }
    if (us_barrier) *us_barrier = out[0];
    if (us_cas_barrier) *us_cas_barrier = out[1];
    return UASTAR_OK;
}

int32_t uastar_set_stream(uastar_engine *eng, void *cuda_stream) {
    if (!eng) return UASTAR_BAD_INPUT;
    eng->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : eng->own_stream;
    return UASTAR_OK;
}

int64_t uastar_kernel_launches(const uastar_engine *eng) { return eng ? eng->launches.load() : 0; }

int32_t uastar_grid_load(uastar_engine *eng, const uint64_t *words, int32_t H, int32_t W) {
    if (!eng) return UASTAR_BAD_INPUT;
    cudaSetDevice(eng->device);
    int32_t rc = grid_load_impl(eng, words, H, W);
    if (rc) return rc;
    cudaError_t e = cudaStreamSynchronize(eng->stream);
    return e == cudaSuccess ? UASTAR_OK : fail_cuda(eng, e, "bitmap upload");
}

int32_t uastar_grid_solve_loaded(uastar_engine *eng, int32_t sx, int32_t sy, int32_t ex, int32_t ey,
                                 uastar_grid_result *out) {
    if (!eng || !out) return UASTAR_BAD_INPUT;
    cudaSetDevice(eng->device);
    return grid_solve_impl(eng, nullptr, sx, sy, ex, ey, out);
}

int32_t uastar_grid_solve(uastar_engine *eng, const uint64_t *words, int32_t H, int32_t W, int32_t sx,
                          int32_t sy, int32_t ex, int32_t ey, uastar_grid_result *out) {
    if (!eng || !out) return UASTAR_BAD_INPUT;
    cudaSetDevice(eng->device);
    const double t0 = now_ms();
    int32_t rc = grid_load_impl(eng, words, H, W);
    if (rc) {
        std::memset(out, 0, sizeof(*out));
        return out->status = rc;
    }
    rc = grid_solve_impl(eng, words, sx, sy, ex, ey, out);
    out->solve_ms = now_ms() - t0;
    return rc;
}

int64_t uastar_grid_path(uastar_engine *eng, int32_t *ids, int64_t cap) {
    if (!eng) return -UASTAR_BAD_INPUT;
    if (eng->last_kind != UASTAR_KIND_GRID || !eng->last_ok || !eng->path_cached) return -UASTAR_NO_SOLUTION;
    const int64_t n = (int64_t)eng->path.size();
    if (ids)
        for (int64_t i = 0; i < n && i < cap; ++i) ids[i] = eng->path[i];
    return n;
}

int32_t uastar_puzzle_solve(uastar_engine *eng, int32_t n, const uint8_t *tiles, uastar_puzzle_result *out) {
    if (!eng || !out) return UASTAR_BAD_INPUT;
    const double t0 = now_ms();
    std::memset(out, 0, sizeof(*out));
    cudaSetDevice(eng->device);
    eng->last_ok = false;
    eng->path_cached = false;
    eng->last_kind = UASTAR_KIND_PUZZLE;
    if ((n < 3 || n > 5) || !tiles || !board_ok(n, tiles)) {
        eng->set_err("puzzle must be 3x3, 4x4 or 5x5 with tiles 0..n*n-1 once each");
        return out->status = UASTAR_BAD_INPUT;
    }
    if (!eng->pdb_ready[n]) {
        eng->set_err("pattern database not resident: call uastar_pdb_build or uastar_pdb_load");
        return out->status = UASTAR_BAD_INPUT;
    }
    if (!board_solvable(n, tiles)) {
        out->status = UASTAR_NO_SOLUTION;
        out->solve_ms = now_ms() - t0;
        return out->status;
    }
    PlainOut po;
    int32_t rc = n == 3   ? puzzle_solve_n<3>(eng, tiles, &po)
                 : n == 4 ? puzzle_solve_n<4>(eng, tiles, &po)
                          : puzzle_solve_n<5>(eng, tiles, &po);
    if (rc) return out->status = rc;
    const TeamState &st = po.st;
    out->status = (int32_t)st.status;
    out->expanded = (int64_t)st.expanded;
    out->generated = (int64_t)st.generated;
    out->pushed = (int64_t)st.pushed;
    out->rounds = (int64_t)st.round;
    out->table_used = (int64_t)st.inserted;
    out->kernel_ms = po.kernel_ms;
    out->table_grows = po.grows;
    if (st.status == ST_OK) {
        out->steps = (int32_t)st.goal_best;
        eng->path.clear();
        std::vector<int> blanks;  // blank cell of each board, start -> goal
        if (n == 5) {
            std::vector<Key128> keys;
            rc = walk_keys_wide(eng, st.goal_slot, 4096, &keys);
            if (rc) return out->status = rc;
            for (const Key128 &k : keys) {
                int b = 24;
                for (int c = 0; c < 24; ++c)
                    if (PuzzleProblem<5>::field(k, c) == 0) b = c;
                blanks.push_back(b);
            }
        } else {
            std::vector<uint64_t> keys;
            rc = walk_keys(eng, st.goal_slot, 4096, &keys, PuzzleProblem<4>::kLink);
            if (rc) return out->status = rc;
            for (uint64_t k : keys) {
                int b = -1;
                for (int c = 0; c < n * n; ++c)
                    if (((k >> (4 * c)) & 15) == 0) b = c;
                blanks.push_back(b);
            }
        }
        for (size_t i = 1; i < blanks.size(); ++i) {
            const int d = blanks[i] - blanks[i - 1];
            eng->path.push_back(d == n ? 0 : d == -n ? 1 : d == 1 ? 2 : 3);
        }
        if ((int64_t)eng->path.size() != out->steps ||
            uastar_validate_puzzle_moves(n, tiles, eng->path.data(), (int64_t)eng->path.size()) != UASTAR_OK) {
            eng->set_err("engine returned moves that fail host validation");
            return out->status = UASTAR_CUDA_ERROR;
        }
        eng->last_ok = true;
        eng->path_cached = true;
        eng->last_n = n;
        std::memcpy(eng->last_tiles, tiles, (size_t)n * n);
    } else if (st.status == ST_RUNNING) {
        eng->set_err("search kernel ended without a status");
        out->status = UASTAR_CUDA_ERROR;
    }
    out->solve_ms = now_ms() - t0;
    return out->status;
}

int32_t uastar_puzzle_solve_bounded(uastar_engine *eng, int32_t n, const uint8_t *tiles, int32_t max_log2_slots,
                                    uastar_bounded_result *out) {
    if (!eng || !out) return UASTAR_BAD_INPUT;
    const double t0 = now_ms();
    std::memset(out, 0, sizeof(*out));
    cudaSetDevice(eng->device);
    eng->last_ok = false;
    eng->path_cached = false;
    eng->last_kind = UASTAR_KIND_PUZZLE;
    if (n < 3 || n > 5 || !tiles || !board_ok(n, tiles) || max_log2_slots < 16 || max_log2_slots > 31) {
        eng->set_err("bounded solve: 3x3, 4x4 or 5x5 board with tiles 0..n*n-1 once each, 16 <= max_log2_slots <= 31");
        return out->status = UASTAR_BAD_INPUT;
    }
    if (!eng->pdb_ready[n]) {
        eng->set_err("pattern database not resident: call uastar_pdb_build or uastar_pdb_load");
        return out->status = UASTAR_BAD_INPUT;
    }
    if (!board_solvable(n, tiles)) {
        out->status = UASTAR_NO_SOLUTION;
        out->solve_ms = now_ms() - t0;
        return out->status;
    }
    std::vector<int32_t> moves;
    int32_t rc = n == 3   ? puzzle_bounded_n<3>(eng, tiles, max_log2_slots, out, &moves)
                 : n == 4 ? puzzle_bounded_n<4>(eng, tiles, max_log2_slots, out, &moves)
                          : puzzle_bounded_n<5>(eng, tiles, max_log2_slots, out, &moves);
    out->status = rc;
    if (rc == UASTAR_OK) {
        out->steps = (int32_t)moves.size();
        if (uastar_validate_puzzle_moves(n, tiles, moves.data(), (int64_t)moves.size()) != UASTAR_OK) {
            eng->set_err("bounded solve returned moves that fail host validation");
            out->status = UASTAR_CUDA_ERROR;
        } else {
            eng->path = moves;
            eng->last_ok = true;
            eng->path_cached = true;
            eng->last_n = n;
            std::memcpy(eng->last_tiles, tiles, (size_t)n * n);
        }
    }
    out->solve_ms = now_ms() - t0;
    return out->status;
}

int64_t uastar_puzzle_moves(uastar_engine *eng, int32_t *moves, int64_t cap) {
    if (!eng) return -UASTAR_BAD_INPUT;
    if (eng->last_kind != UASTAR_KIND_PUZZLE || !eng->last_ok || !eng->path_cached) return -UASTAR_NO_SOLUTION;
    const int64_t n = (int64_t)eng->path.size();
    if (moves)
        for (int64_t i = 0; i < n && i < cap; ++i) moves[i] = eng->path[i];
    return n;
}

}  // extern "C"

// Team-wide stable LSD radix sort of (32-bit key, 32-bit position) pairs.
//
// The reference sorts every round's successor list by (cell, g) with
// moderngpu's MergesortPairs and keeps the first record of each cell
// (src/pathway/GPU-solver.cu:218-235, kAssign in src/pathway/GPU-kernel.cuh:338-398)
// so that its dedup kernel sees each cell once.  This is the same step for a
// search team: every thread of every CTA of the team calls team_radix_sort
// with the same arguments, between two of the team's barriers.
//
// A pass sorts on 8 bits of the key.  CTA c owns the tile of positions
// [c * tile, (c + 1) * tile) (tile = ceil(n / C)) and holds its elements in
// registers for the whole pass:
//   1. rank: chunk by chunk (T elements in tile order), each element's rank
//      among the tile's elements of its digit that precede it — warp peers by
//      __match_any_sync, warps by a per-digit scan in shared memory; the
//      tile's 256 digit counts go to hist[digit * C + c].          barrier
//   2. column scan: CTA c scans the rows of digits c, c + C, ...: each entry
//      becomes the count of that digit in the tiles before it, the row total
//      goes to hist[256 * C + digit].                              barrier
//   3. scatter: an element of digit d lands at (elements of smaller digits)
//      + (digit d in earlier tiles) + its rank, which keeps equal keys in
//      position order (stable).                                    barrier
// Key bits [0, bits) are sorted, in ceil(bits / 8) passes.  Every index
// computed from the count matrix is checked against n before it is used;
// a violation (only possible after a barrier gave up) sets *err.
#pragma once
#include <cstdint>

#include "ga_device.cuh"

namespace uastar {

// Shared memory of the sort for T threads per CTA (4-byte words): per-warp
// digit counts, running tile counts, scatter bases, scan scratch.
__host__ __device__ constexpr size_t sort_smem_bytes(uint32_t T) {
    return ((size_t)(T / 32 + 2) * 256 + 40) * 4;
}

// Exclusive prefix over the CTA of one value per thread; scratch holds
// 2 + warps words.  Returns the prefix; *total gets the sum.
__device__ __forceinline__ uint32_t sort_block_scan(uint32_t v, uint32_t *scratch, uint32_t *total) {
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

// Sorts the n pairs (key(i) << 32 | i), i < n, by key bits [0, bits), stably.
// `key(i)` gives the key of input position i (read in the first pass only).
// buf0 / buf1 hold n pairs each; hist holds 256 * (C + 1) words.  Returns the
// buffer holding the result.  n <= C * kPer * blockDim.x is the caller's
// guarantee (a tile fits the registers).
template <int kPer, class Team, class KeyFn>
__device__ const unsigned long long *team_radix_sort(Team &team, uint32_t n, uint32_t bits, KeyFn key,
                                                     unsigned long long *buf0, unsigned long long *buf1,
                                                     uint32_t *hist, uint32_t *sm, uint32_t *err) {
    const uint32_t T = blockDim.x, tid = threadIdx.x, w = tid >> 5, nw = T >> 5;
    const uint32_t C = team.ctas(), cta = team.cta();
    uint32_t *const whist = sm;                   // nw x 256
    uint32_t *const cnt = sm + (size_t)nw * 256;  // 256: running tile counts
    uint32_t *const base = cnt + 256;             // 256: scatter bases
    uint32_t *const scan = base + 256;            // 40: block scans
    const uint32_t tile = (n + C - 1) / C;
    const uint32_t K = (tile + T - 1) / T;  // chunks of the tile (<= kPer)
    const uint32_t first = cta * tile;
    const unsigned long long *in = nullptr;
    unsigned long long *out = buf0;
    const uint32_t passes = bits == 0 ? 0u : (bits + 7u) / 8u;
    for (uint32_t pass = 0; pass < passes; ++pass) {
        const uint32_t shift = pass * 8u;
        unsigned long long v[kPer];
        uint32_t rank[kPer];
        for (uint32_t d = tid; d < 256; d += T) cnt[d] = 0;
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            if ((uint32_t)k >= K) break;  // uniform over the CTA
            const uint32_t e = (uint32_t)k * T + tid;
            const uint32_t i = first + e;
            const bool valid = e < tile && i < n;
            v[k] = 0;
            if (valid) v[k] = pass == 0 ? ((unsigned long long)key(i) << 32 | i) : __ldcg(in + i);
            const uint32_t d = valid ? (uint32_t)(v[k] >> (32 + shift)) & 255u : 256u;
            __syncthreads();  // the previous chunk's ranks are read
            for (uint32_t q = tid; q < nw * 256; q += T) whist[q] = 0;
            __syncthreads();
            const uint32_t peers = __match_any_sync(kFull, d);
            const uint32_t wr = __popc(peers & lanemask_lt());
            if (valid && wr == 0) whist[w * 256 + d] = __popc(peers);
            __syncthreads();
            for (uint32_t dd = tid; dd < 256; dd += T) {
                uint32_t run = cnt[dd];
                for (uint32_t q = 0; q < nw; ++q) {
                    const uint32_t t = whist[q * 256 + dd];
                    whist[q * 256 + dd] = run;
                    run += t;
                }
                cnt[dd] = run;
            }
            __syncthreads();
            rank[k] = valid ? whist[w * 256 + d] + wr : 0u;
        }
        __syncthreads();
        for (uint32_t d = tid; d < 256; d += T) hist[(size_t)d * C + cta] = cnt[d];
        team.sync();

        // column scans: digit rows c, c + C, ...
        const uint32_t per = (C + T - 1) / T, cb = tid * per, ce = min(cb + per, C);
        for (uint32_t d = cta; d < 256; d += C) {
            uint32_t *row = hist + (size_t)d * C;
            uint32_t s = 0;
            for (uint32_t c = cb; c < ce; ++c) s += __ldcg(row + c);
            uint32_t tot;
            uint32_t off = sort_block_scan(s, scan, &tot);
            for (uint32_t c = cb; c < ce; ++c) {
                const uint32_t t = __ldcg(row + c);
                row[c] = off;
                off += t;
            }
            if (tid == 0) hist[(size_t)256 * C + d] = tot;
        }
        team.sync();

        // scatter: base[d] = elements of digits < d + digit d in earlier tiles
        const uint32_t dper = (256 + T - 1) / T, db = tid * dper, de = min(db + dper, 256u);
        uint32_t s = 0;
        for (uint32_t d = db; d < de; ++d) s += __ldcg(hist + (size_t)256 * C + d);
        uint32_t tot;
        uint32_t off = sort_block_scan(s, scan, &tot);
        for (uint32_t d = db; d < de; ++d) {
            base[d] = off + __ldcg(hist + (size_t)d * C + cta);
            off += __ldcg(hist + (size_t)256 * C + d);
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            if ((uint32_t)k >= K) break;
            const uint32_t e = (uint32_t)k * T + tid;
            if (e < tile && first + e < n) {
                const uint32_t d = (uint32_t)(v[k] >> (32 + shift)) & 255u;
                const uint32_t pos = base[d] + rank[k];
                if (pos < n)
                    out[pos] = v[k];
                else
                    set_error(err, ST_TIMEOUT);
            }
        }
        in = out;
        out = out == buf0 ? buf1 : buf0;
        team.sync();
    }
    if (passes == 0) {
        // nothing to sort on: the identity order
        for (uint32_t i = cta * T + tid; i < n; i += C * T) buf0[i] = ((unsigned long long)key(i) << 32) | i;
        team.sync();
        return buf0;
    }
    return in;
}

}  // namespace uastar

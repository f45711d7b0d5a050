// Host-side utilities of the engine: seeded instance generators, the
// reachability screen and the path validators declared in uastar_gpu.h.
// Plain C++ (no CUDA); compiled into libuastar_gb300.so next to the engine.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <unordered_set>
#include <vector>

#include "../../include/uastar_gpu.h"

namespace {

// splitmix64 (Steele, Lea & Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014): output #i of the stream seeded with s is
// mix(s + (i+1) * gamma).  Counter-based use lets grid rows be generated in
// parallel with bit-identical results on any host.
constexpr uint64_t kGamma = 0x9E3779B97F4A7C15ull;

inline uint64_t sm64_mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline uint64_t sm64_at(uint64_t seed, uint64_t i) { return sm64_mix(seed + (i + 1) * kGamma); }

// Blank moves 0..3 as (row, column) deltas: the reference's DX/DY[0..3]
// (src/utils.hpp:120-121).
constexpr int kPDX[4] = {1, -1, 0, 0};
constexpr int kPDY[4] = {0, 0, 1, -1};
// 8 grid moves: 4 straight then 4 diagonal (src/utils.hpp:120-122).
constexpr int kGDX[8] = {1, -1, 0, 0, 1, 1, -1, -1};
constexpr int kGDY[8] = {0, 0, 1, -1, 1, -1, 1, -1};
constexpr float kSqrt2f = 1.4142135623731f;  // src/utils.hpp:119

inline bool bit_open(const uint64_t *w, uint64_t id) { return (w[id >> 6] >> (id & 63)) & 1ull; }

}  // namespace

extern "C" {

int32_t uastar_gen_grid(uint64_t seed, int32_t H, int32_t W, double block_rate, int32_t sx,
                        int32_t sy, int32_t ex, int32_t ey, uint64_t *words) {
    if (H <= 0 || W <= 0 || !words || !(block_rate >= 0.0 && block_rate <= 1.0))
        return UASTAR_BAD_INPUT;
    if (sx < 0 || sx >= H || sy < 0 || sy >= W || ex < 0 || ex >= H || ey < 0 || ey >= W)
        return UASTAR_BAD_INPUT;
    const uint64_t cells = (uint64_t)H * (uint64_t)W;
    const uint64_t nwords = (cells + 63) / 64;
    // Cell id is blocked iff (splitmix64 output #id >> 32) < thr.
    const double t = std::floor(block_rate * 4294967296.0);
    const uint64_t thr = t >= 4294967296.0 ? (1ull << 32) : (uint64_t)t;
    auto fill = [&](uint64_t w0, uint64_t w1) {
        for (uint64_t w = w0; w < w1; ++w) {
            uint64_t v = 0;
            const uint64_t base = w * 64;
            const uint64_t lim = std::min<uint64_t>(64, cells - base);
            for (uint64_t b = 0; b < lim; ++b) {
                const uint64_t r = sm64_at(seed, base + b) >> 32;
                if (r >= thr) v |= 1ull << b;
            }
            words[w] = v;
        }
    };
    unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    if (nwords < (1u << 16)) nt = 1;
    std::vector<std::thread> th;
    for (unsigned i = 0; i < nt; ++i) {
        const uint64_t a = nwords * i / nt, b = nwords * (i + 1) / nt;
        th.emplace_back(fill, a, b);
    }
    for (auto &x : th) x.join();
    const uint64_t s = (uint64_t)sx * W + sy, e = (uint64_t)ex * W + ey;
    words[s >> 6] |= 1ull << (s & 63);
    words[e >> 6] |= 1ull << (e & 63);
    return UASTAR_OK;
}

int32_t uastar_gen_puzzle(uint64_t seed, int32_t n, int32_t walk_len, uint8_t *tiles) {
    if (n < 2 || n > 5 || walk_len < 0 || !tiles) return UASTAR_BAD_INPUT;
    const int nn = n * n;
    for (int i = 0; i < nn; ++i) tiles[i] = (uint8_t)((i + 1) % nn);
    int bx = n - 1, by = n - 1, last = -1;
    uint64_t ctr = 0;
    for (int step = 0; step < walk_len; ++step) {
        int cand[4], c = 0;
        for (int d = 0; d < 4; ++d) {
            if (last >= 0 && d == (last ^ 1)) continue;  // never undo the previous move
            int nx = bx + kPDX[d], ny = by + kPDY[d];
            if (nx >= 0 && nx < n && ny >= 0 && ny < n) cand[c++] = d;
        }
        const uint64_t r = sm64_at(seed, ctr++) >> 32;
        const int d = cand[(int)((r * (uint64_t)c) >> 32)];
        const int nx = bx + kPDX[d], ny = by + kPDY[d];
        std::swap(tiles[bx * n + by], tiles[nx * n + ny]);
        bx = nx;
        by = ny;
        last = d;
    }
    return UASTAR_OK;
}

int32_t uastar_gen_zigzag(int32_t H, int32_t W, int32_t height_gap, uint64_t *words,
                          int32_t *sx, int32_t *sy, int32_t *ex, int32_t *ey) {
    // Same maze as the reference's zigzag module (src/pathway/input/zigzag.cpp:14-40):
    // every height_gap-th row is a wall with one gap, alternating between the
    // last column and the first column; start/goal at the middle column of the
    // first/last row.
    if (H <= 0 || W <= 0 || height_gap <= 0 || !words) return UASTAR_BAD_INPUT;
    const uint64_t cells = (uint64_t)H * W;
    std::memset(words, 0, ((cells + 63) / 64) * 8);
    bool gap_first = false;
    for (int x = 0; x < H; ++x) {
        const bool wall = x > 0 && x % height_gap == 0;
        for (int y = 0; y < W; ++y) {
            bool open = true;
            if (wall) open = gap_first ? (y == 0) : (y == W - 1);
            if (open) {
                const uint64_t id = (uint64_t)x * W + y;
                words[id >> 6] |= 1ull << (id & 63);
            }
        }
        if (wall) gap_first = !gap_first;
    }
    if (sx) *sx = 0;
    if (sy) *sy = W / 2;
    if (ex) *ex = H - 1;
    if (ey) *ey = W / 2;
    return UASTAR_OK;
}

int32_t uastar_grid_reachable(const uint64_t *words, int32_t H, int32_t W, int32_t sx,
                              int32_t sy, int32_t ex, int32_t ey) {
    if (!words || H <= 0 || W <= 0) return 0;
    const uint64_t cells = (uint64_t)H * W;
    const uint64_t s = (uint64_t)sx * W + sy, e = (uint64_t)ex * W + ey;
    if (s == e) return 1;
    std::vector<uint64_t> seen((cells + 63) / 64, 0);
    std::vector<uint32_t> q;
    q.reserve(1 << 20);
    q.push_back((uint32_t)s);
    seen[s >> 6] |= 1ull << (s & 63);
    for (size_t head = 0; head < q.size(); ++head) {
        const uint64_t id = q[head];
        if (!bit_open(words, id)) continue;  // a blocked cell has no out-moves
        const int x = (int)(id / W), y = (int)(id % W);
        for (int d = 0; d < 8; ++d) {
            const int nx = x + kGDX[d], ny = y + kGDY[d];
            if (nx < 0 || nx >= H || ny < 0 || ny >= W) continue;
            const uint64_t nid = (uint64_t)nx * W + ny;
            if (nid == e) return 1;
            if (seen[nid >> 6] >> (nid & 63) & 1ull) continue;
            seen[nid >> 6] |= 1ull << (nid & 63);
            q.push_back((uint32_t)nid);
        }
    }
    return 0;
}

int32_t uastar_grid_screen(const uint64_t *words, int32_t H, int32_t W, int32_t sx, int32_t sy,
                           int32_t ex, int32_t ey, int64_t limit) {
    // Bounded forward search from the start and bounded backward search from
    // the goal (a cell u reaches v iff u is open and v is one of its 8
    // neighbours).  A search that exhausts its component without meeting the
    // other endpoint proves the goal unreachable; if both outgrow `limit`
    // cells the endpoints are presumed connected.
    if (!words || H <= 0 || W <= 0 || limit < 0) return 0;
    const uint64_t s = (uint64_t)sx * W + sy, e = (uint64_t)ex * W + ey;
    if (s == e) return 1;
    // Visited cells in a flat open-addressed set (linear probing, all-ones =
    // free) sized to 4x the bound, so it never fills.
    uint64_t cap = 64;
    while (cap < 4 * (uint64_t)limit + 64) cap <<= 1;
    std::vector<uint32_t> set(cap);
    for (int dir = 0; dir < 2; ++dir) {
        const uint64_t from = dir == 0 ? s : e, to = dir == 0 ? e : s;
        std::fill(set.begin(), set.end(), 0xFFFFFFFFu);
        int64_t nseen = 0;
        auto insert = [&](uint32_t id) {
            uint64_t h = ((uint64_t)id * 0x9E3779B97F4A7C15ull) >> 20;
            for (;; ++h) {
                uint32_t &slot = set[h & (cap - 1)];
                if (slot == id) return false;
                if (slot == 0xFFFFFFFFu) {
                    slot = id;
                    ++nseen;
                    return true;
                }
            }
        };
        std::vector<uint32_t> q;
        q.push_back((uint32_t)from);
        insert((uint32_t)from);
        bool overflow = false;
        for (size_t head = 0; head < q.size(); ++head) {
            if (nseen > limit) {
                overflow = true;
                break;
            }
            const uint64_t id = q[head];
            const int x = (int)(id / W), y = (int)(id % W);
            if (dir == 0 && !bit_open(words, id)) continue;
            for (int d = 0; d < 8; ++d) {
                const int nx = x + kGDX[d], ny = y + kGDY[d];
                if (nx < 0 || nx >= H || ny < 0 || ny >= W) continue;
                const uint64_t nid = (uint64_t)nx * W + ny;
                if (dir == 1 && !bit_open(words, nid)) continue;  // predecessors must be open
                if (nid == to) return 1;
                if (insert((uint32_t)nid)) q.push_back((uint32_t)nid);
            }
        }
        if (!overflow) return 0;
    }
    return 2;
}

int32_t uastar_validate_grid_path(const uint64_t *words, int32_t H, int32_t W, int32_t sx,
                                  int32_t sy, int32_t ex, int32_t ey, const int32_t *ids,
                                  int64_t len, int64_t *straight, int64_t *diagonal,
                                  float *cost) {
    if (!words || !ids || len < 1) return UASTAR_BAD_INPUT;
    const int64_t cells = (int64_t)H * W;
    if (ids[0] != (int64_t)sx * W + sy || ids[len - 1] != (int64_t)ex * W + ey)
        return UASTAR_BAD_INPUT;
    int64_t a = 0, b = 0;
    float c = 0.0f;
    for (int64_t i = 1; i < len; ++i) {
        const int64_t u = ids[i - 1], v = ids[i];
        if (u < 0 || u >= cells || v < 0 || v >= cells) return UASTAR_BAD_INPUT;
        if (!bit_open(words, (uint64_t)u)) return UASTAR_BAD_INPUT;
        const int64_t dx = std::llabs(u / W - v / W), dy = std::llabs(u % W - v % W);
        if (dx > 1 || dy > 1 || dx + dy == 0) return UASTAR_BAD_INPUT;
        if (dx + dy == 2) {
            ++b;
            c = c + kSqrt2f;
        } else {
            ++a;
            c = c + 1.0f;
        }
    }
    if (straight) *straight = a;
    if (diagonal) *diagonal = b;
    if (cost) *cost = c;
    return UASTAR_OK;
}

int32_t uastar_validate_puzzle_moves(int32_t n, const uint8_t *tiles, const int32_t *moves,
                                     int64_t len) {
    if (n < 2 || n > 5 || !tiles || (len > 0 && !moves)) return UASTAR_BAD_INPUT;
    const int nn = n * n;
    uint8_t b[25];
    int seen = 0, bx = -1, by = -1;
    for (int i = 0; i < nn; ++i) {
        b[i] = tiles[i];
        if (b[i] >= nn || (seen >> b[i] & 1)) return UASTAR_BAD_INPUT;
        seen |= 1 << b[i];
        if (!b[i]) {
            bx = i / n;
            by = i % n;
        }
    }
    for (int64_t i = 0; i < len; ++i) {
        const int d = moves[i];
        if (d < 0 || d > 3) return UASTAR_BAD_INPUT;
        const int nx = bx + kPDX[d], ny = by + kPDY[d];
        if (nx < 0 || nx >= n || ny < 0 || ny >= n) return UASTAR_BAD_INPUT;
        std::swap(b[bx * n + by], b[nx * n + ny]);
        bx = nx;
        by = ny;
    }
    for (int i = 0; i < nn; ++i)
        if (b[i] != (uint8_t)((i + 1) % nn)) return UASTAR_BAD_INPUT;
    return UASTAR_OK;
}

}  // extern "C"

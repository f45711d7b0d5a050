// The two search problems the engine instantiates GA* for.
//
// A problem supplies: the heap entry type and its order, the cost word
// (compared with cost_cmp), the start/goal keys, f = g + h, the valid-move
// mask of a popped node and the successor of one move.
//
// GridProblem   — 8-direction grid of uAstar's --pathway mode.  Costs are the
//                 exact pair (straight A, diagonal B) with value A + B*sqrt(2),
//                 packed A<<32 | B and compared with integer arithmetic only,
//                 so the search is exact where the reference accumulates float32.
// PuzzleProblem — n x n sliding tile of --puzzle with the additive disjoint
//                 pattern database; integer move counts.
#pragma once
#include <cstdint>

#include "ga_device.cuh"

namespace uastar {

// ----------------------------------------------------------------- grid ---
struct __align__(16) GridEntry {
    uint32_t fa, fb;  // f = fa + fb*sqrt(2)
    uint32_t slot;
    uint32_t cell;    // the node's cell: a pop reads its bitmap neighbourhood
                      // while the node record is still in flight
};

// sign((a1 + b1*sqrt2) - (a2 + b2*sqrt2)) for packed a<<32|b words; kInfCost
// is larger than every cost.  Exact for a, b < 2^31.
__host__ __device__ __forceinline__ int grid_cost_cmp(uint64_t p, uint64_t q) {
    if (p == q) return 0;
    if (p == kInfCost) return 1;
    if (q == kInfCost) return -1;
    const int64_t d = (int64_t)(p >> 32) - (int64_t)(q >> 32);            // straight diff
    const int64_t e = (int64_t)(q & 0xffffffffu) - (int64_t)(p & 0xffffffffu);  // value = d - e*sqrt2
    if (e == 0) return d > 0 ? 1 : (d < 0 ? -1 : 0);
    if (d >= 0 && e < 0) return 1;
    if (d <= 0 && e > 0) return -1;
    const uint64_t lhs = (uint64_t)(d * d), rhs = (uint64_t)(2 * e * e);
    const int s = lhs > rhs ? 1 : -1;  // never equal: sqrt(2) is irrational
    return d > 0 ? s : -s;
}

struct GridProblem : NarrowSlots {
    using Entry = GridEntry;
    static constexpr int kMoves = 8;
    // Slot key word = cell | prev << 32 (cells are < 2^32 - 1): the relax CAS
    // sets g and the parent link together, so no push-phase winner check.
    static constexpr bool kPrevInKey = true;
    static constexpr int kLink = LINK_IN_KEY;
    __device__ static uint32_t slot_prev(const Slot *s) { return (uint32_t)(__ldcg(&s->key) >> 32); }
    __device__ static void set_link(Slot *, uint32_t, uint32_t) {}  // the link lives in the key word

    const uint32_t *bm;  // bitmap as 32-bit words (same bytes as the uint64 words)
    int32_t H, W;
    int32_t sx, sy, ex, ey;

    __device__ static int cost_cmp(uint64_t a, uint64_t b) { return grid_cost_cmp(a, b); }

    __device__ __forceinline__ bool open(int64_t id) const {
        return (__ldg(bm + (id >> 5)) >> (id & 31)) & 1u;
    }
    __device__ uint64_t start_key() const { return (uint64_t)sx * W + sy; }
    // a grid node's aux is its own cell (carried into its heap entries)
    __device__ uint32_t start_aux() const { return (uint32_t)start_key(); }
    __device__ bool is_goal(uint64_t key) const { return key == (uint64_t)ex * W + ey; }
    // The entry names its node's key: moves() can start before load_node().
    // On grids of at most 2^29 cells it also carries the move that reached
    // the node (bits 29-31 of the cell word), and the expansion skips every
    // successor that is the parent p or one of p's neighbours: one step from
    // p costs at most sqrt2, two steps through the node at least 2, so the
    // relax could never succeed.  (By induction along the parent chain this
    // holds although the ancestors skipped successors too: a neighbour n of
    // the node that is skipped was relaxed by the nearest ancestor that did
    // not skip it, at that ancestor's g + one step, while the node's g is at
    // least that g + 1 and the step from the node at least 1.)  The start
    // node has no incoming move.  Entries that are stale are not expanded, so
    // the move is always that of the node's current g and parent.
    static constexpr bool kEntryKey = true;
    static constexpr uint32_t kCellBits = 29;
    __device__ __forceinline__ bool dirs() const { return (uint64_t)(uint32_t)H * (uint32_t)W <= (1ull << kCellBits); }
    __device__ __forceinline__ uint64_t entry_key(const GridEntry &e) const {
        return dirs() ? (e.cell & ((1u << kCellBits) - 1u)) : e.cell;
    }
    // successors of the move that reached a node that can never improve
    // (bit j = move j), indexed by that move
    __device__ __forceinline__ static uint32_t pruned(uint32_t in) {
        return (uint32_t)(0x1529468a57ab3dceull >> (8 * in)) & 0xffu;
    }
    __device__ __forceinline__ uint32_t entry_moves(const GridEntry &e) const {
        const uint64_t key = entry_key(e);
        uint32_t m = moves(key, 0);
        if (dirs() && key != start_key()) m &= ~pruned(e.cell >> kCellBits);
        return m;
    }

    // Octile heuristic (src/pathway/CPU-solver.cpp:139-146): with dx, dy the
    // distances to the goal, h = min(dx,dy)*sqrt2 + |dx-dy| — as a pair.
    __device__ __forceinline__ uint64_t h_of(uint64_t key) const {
        const uint32_t c = (uint32_t)key;  // H*W < 2^32 is checked on the host
        const int x = (int)(c / (uint32_t)W), y = (int)(c - (uint32_t)x * (uint32_t)W);
        const int dx = abs(x - ex), dy = abs(y - ey);
        const int mn = min(dx, dy), mx = max(dx, dy);
        return ((uint64_t)(mx - mn) << 32) | (uint64_t)mn;
    }
    __device__ __forceinline__ uint64_t f_of(uint64_t key, uint64_t g, uint32_t) const {
        return g + h_of(key);  // field-wise: both halves stay below 2^31
    }

    // Open bits of the cells (r, y-1), (r, y), (r, y+1) as bits 0..2 (0 for a
    // row or column outside the grid).  Two 32-bit words cover the three
    // cells, and their addresses depend on the cell alone, so the three rows
    // of a node are read in one round trip of independent loads.
    __device__ __forceinline__ uint32_t row3(int r, int y) const {
        if (r < 0 || r >= H) return 0;
        const int64_t c0 = (int64_t)r * W + y - 1;  // cell (r, y-1); -1 only for (0, 0)
        const uint64_t lo = c0 < 0 ? 0 : (uint64_t)c0;
        const uint64_t wlast = ((uint64_t)(uint32_t)H * (uint32_t)W + 63) / 64 * 2 - 1;  // last 32-bit word
        const uint64_t w0 = lo >> 5, w1 = w0 + 1 <= wlast ? w0 + 1 : wlast;
        const uint64_t v = (uint64_t)__ldg(bm + w0) | ((uint64_t)__ldg(bm + w1) << 32);
        uint32_t bits = (uint32_t)(v >> (lo & 31u)) & 7u;
        if (c0 < 0) bits = (bits << 1) & 7u;  // the window starts one cell before the grid
        if (y == 0) bits &= ~1u;              // (r, -1) is no cell
        if (y == W - 1) bits &= ~4u;          // (r, W) is no cell (the next row's first)
        return bits;
    }

    // Valid moves of a popped cell, bit i = direction i (4 straight, then 4
    // diagonal; src/utils.hpp:120-122).  Only an open cell moves
    // (CPU-solver.cpp:98-100).  A move into a blocked cell is legal in the
    // reference but such a cell has no out-moves, so it is generated only
    // when it is the goal: no path cost changes.
    __device__ uint32_t moves(uint64_t key, uint32_t) const {
        const uint32_t c = (uint32_t)key;
        const int x = (int)(c / (uint32_t)W), y = (int)(c - (uint32_t)x * (uint32_t)W);
        const uint32_t rows[3] = {row3(x - 1, y), row3(x, y), row3(x + 1, y)};
        if (!(rows[1] & 2u)) return 0;
        uint32_t m = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int dx = c_dx(i), dy = c_dy(i);
            const bool goal = x + dx == ex && y + dy == ey;
            if (((rows[dx + 1] >> (dy + 1)) & 1u) || goal) m |= 1u << i;
        }
        return m;
    }
    __device__ __forceinline__ static int c_dx(int i) {
        return i == 0 ? 1 : i == 1 ? -1 : i < 4 ? 0 : (i < 6 ? 1 : -1);
    }
    __device__ __forceinline__ static int c_dy(int i) {
        return i < 2 ? 0 : i == 2 ? 1 : i == 3 ? -1 : ((i & 1) ? -1 : 1);
    }
    __device__ void apply(uint64_t key, uint64_t g, uint32_t, int mv, uint64_t &nkey,
                          uint64_t &ng, uint32_t &naux, uint64_t &nf) const {
        const uint32_t c = (uint32_t)key;
        const int x = (int)(c / (uint32_t)W), y = (int)(c - (uint32_t)x * (uint32_t)W);
        nkey = (uint64_t)(x + c_dx(mv)) * W + (uint64_t)(y + c_dy(mv));
        ng = g + (mv < 4 ? (1ull << 32) : 1ull);
        naux = in_aux(nkey, mv);
        nf = ng + h_of(nkey);
    }
    // Successor in two steps (the puzzle's second step waits on a database
    // load that is issued in the first, so that it overlaps the table CAS);
    // for grids everything is register arithmetic in the first.
    struct Succ {
        uint64_t key, g, f;
    };
    __device__ __forceinline__ void succ_begin(uint64_t key, uint64_t g, uint32_t aux, int mv, Succ &s) const {
        uint32_t naux;
        apply(key, g, aux, mv, s.key, s.g, naux, s.f);
    }
    __device__ __forceinline__ void succ_end(const Succ &s, uint32_t, int mv, uint32_t &naux, uint64_t &nf) const {
        naux = in_aux(s.key, mv);
        nf = s.f;
    }
    // a successor's entry cell word: its cell and, where it fits, the move
    __device__ __forceinline__ uint32_t in_aux(uint64_t nkey, int mv) const {
        return (uint32_t)nkey | (dirs() ? (uint32_t)mv << kCellBits : 0u);
    }
    __device__ __forceinline__ Entry make_entry(uint64_t f, uint64_t, uint32_t slot, uint32_t aux) const {
        Entry e;
        e.fa = (uint32_t)(f >> 32);
        e.fb = (uint32_t)f;
        e.slot = slot;
        e.cell = aux;
        return e;
    }
    __device__ __forceinline__ static uint64_t entry_cost(const Entry &e) {
        return ((uint64_t)e.fa << 32) | e.fb;
    }
    // Equal f: no preference (a deeper-first tie-break measured no change in
    // expansions or time on the 1000^2 and 20000^2 grids).
    __device__ __forceinline__ static bool less(const Entry &a, const Entry &b) {
        return grid_cost_cmp(entry_cost(a), entry_cost(b)) < 0;
    }
    __device__ __forceinline__ static Entry load(const Entry *p) {
        const uint4 u = __ldcg(reinterpret_cast<const uint4 *>(p));
        Entry e;
        e.fa = u.x;
        e.fb = u.y;
        e.slot = u.z;
        e.cell = u.w;
        return e;
    }
    __device__ __forceinline__ static void store(Entry *p, const Entry &e) {
        *reinterpret_cast<uint4 *>(p) = make_uint4(e.fa, e.fb, e.slot, e.cell);
    }
    // Node record fields needed at pop time: key and g share the first 16 B.
    __device__ __forceinline__ static void load_node(const Slot *s, uint64_t &key, uint64_t &g,
                                                     uint32_t &aux) {
        const ulonglong2 v = __ldcg(reinterpret_cast<const ulonglong2 *>(s));
        key = v.x & 0xffffffffull;
        g = v.y;
        aux = (uint32_t)key;
    }
};

// --------------------------------------------------------------- puzzle ---
struct __align__(8) PuzzleEntry {
    uint32_t key;   // f << 16 | (0xFFFF - g): min f, then max g
    uint32_t slot;
};

// Disjoint pattern partitions of the reference (src/puzzle/CPU-solver.hpp:43-70)
// and the mixed-radix multipliers of its rank (src/puzzle/database.cpp:8-25):
// multiple[j] = prod_{i=j}^{k-1} (n*n - i), rank = sum_j v_j * multiple[j+1],
// v_j = cell of tracked tile j minus the number of earlier tracked tiles on
// lower cells (database.cpp:140-163).
template <int N> struct PuzzlePatterns;
template <> struct PuzzlePatterns<3> {
    static constexpr int kNum = 1;
    __host__ __device__ static constexpr int count(int) { return 8; }
    __host__ __device__ static constexpr int tile(int, int j) { return j + 1; }
    __host__ __device__ static constexpr uint64_t offset(int) { return 0; }
};
template <> struct PuzzlePatterns<4> {
    static constexpr int kNum = 2;
    __host__ __device__ static constexpr int count(int p) { return p == 0 ? 8 : 7; }
    __host__ __device__ static constexpr int tile(int p, int j) {
        return p == 0 ? (j < 6 ? j + 1 : (j == 6 ? 9 : 13))
                      : (j < 2 ? j + 7 : (j < 5 ? j + 8 : j + 9));
    }
    __host__ __device__ static constexpr uint64_t offset(int p) { return p == 0 ? 0ull : 518918400ull; }
};

// 5x5: the four 6-tile partitions, in the reference's tracked order (the
// order fixes the rank; src/puzzle/CPU-solver.hpp:71-102).
template <> struct PuzzlePatterns<5> {
    static constexpr int kNum = 4;
    __host__ __device__ static constexpr int count(int) { return 6; }
    __host__ __device__ static constexpr int tile(int p, int j) {
        constexpr int t[4][6] = {{3, 4, 5, 10, 15, 20}, {2, 1, 6, 11, 16, 21}, {7, 8, 9, 12, 17, 22},
                                 {13, 14, 18, 19, 23, 24}};
        return t[p][j];
    }
    __host__ __device__ static constexpr uint64_t offset(int p) { return (uint64_t)p * 127512000ull; }
};

template <int N> __host__ __device__ constexpr uint32_t pattern_mult(int p, int j) {
    // prod_{i=j}^{k-1} (N*N - i)
    uint32_t m = 1;
    for (int i = j; i < PuzzlePatterns<N>::count(p); ++i) m *= (uint32_t)(N * N - i);
    return m;
}
template <int N> __host__ __device__ constexpr int pattern_of_tile(int t) {
    for (int p = 0; p < PuzzlePatterns<N>::kNum; ++p)
        for (int j = 0; j < PuzzlePatterns<N>::count(p); ++j)
            if (PuzzlePatterns<N>::tile(p, j) == t) return p;
    return -1;
}

template <int N> struct PuzzleProblem : NarrowSlots {
    using Entry = PuzzleEntry;
    static constexpr int kMoves = 4;
    static constexpr int NN = N * N;
    // The slot's g word is g << 40 | (last move + 1) << 32 | prev: the relax
    // CAS sets the cost and the path link together, so the push phase checks
    // no winner (a candidate that lost is a stale entry, dropped at its pop).
    // The aux field keeps the pattern parts, which depend on the board alone:
    // the relaxer that claims the slot writes them.
    static constexpr int kLink = LINK_IN_G;
    __device__ static uint64_t g_word(uint64_t g, uint32_t prev, int mv) {
        return g << 40 | (uint64_t)(uint32_t)(mv + 1) << 32 | prev;
    }
    __device__ static uint64_t word_g(uint64_t w) { return w >> 40; }
    __device__ static uint64_t slot_g(const Slot *s) { return __ldcg(&s->g) >> 40; }
    __device__ static uint32_t slot_prev(const Slot *s) { return (uint32_t)__ldcg(&s->g); }
    __device__ static void set_link(Slot *s, uint32_t, uint32_t aux) { s->aux = aux & 0xffffu; }

    const uint8_t *pdb;   // concatenated tables
    uint64_t start;       // packed board: cell i at bits 4i
    uint64_t goal;

    __device__ static int cost_cmp(uint64_t a, uint64_t b) { return a < b ? -1 : (a > b ? 1 : 0); }

    __host__ __device__ static uint64_t goal_key() {
        uint64_t k = 0;
        for (int i = 0; i < NN; ++i) k |= (uint64_t)((i + 1) % NN) << (4 * i);
        return k;
    }
    // Inverse permutation: nibble t = cell of tile t.
    __device__ __forceinline__ static uint64_t inverse(uint64_t key) {
        uint64_t inv = 0;
#pragma unroll
        for (int i = 0; i < NN; ++i) inv |= (uint64_t)i << (4 * ((key >> (4 * i)) & 15));
        return inv;
    }
    template <int P> __device__ __forceinline__ static uint32_t rank(uint64_t inv) {
        uint32_t used = 0, code = 0;
#pragma unroll
        for (int j = 0; j < PuzzlePatterns<N>::count(P); ++j) {
            const uint32_t pos = (uint32_t)(inv >> (4 * PuzzlePatterns<N>::tile(P, j))) & 15u;
            const uint32_t v = pos - __popc(used & ((1u << pos) - 1u));
            code += v * pattern_mult<N>(P, j + 1);
            used |= 1u << pos;
        }
        return code;
    }
    __device__ __forceinline__ uint32_t part(int p, uint64_t inv) const {
        if (p == 0) return __ldg(pdb + PuzzlePatterns<N>::offset(0) + rank<0>(inv));
        if constexpr (PuzzlePatterns<N>::kNum > 1)
            return __ldg(pdb + PuzzlePatterns<N>::offset(1) + rank<1>(inv));
        return 0;
    }
    // aux = part0 | part1 << 8 | (last move + 1) << 16
    static constexpr uint32_t kLastMoveShift = 16;
    __device__ static uint32_t hsum(uint32_t aux) { return (aux & 0xff) + ((aux >> 8) & 0xff); }

    __device__ uint64_t start_key() const { return start; }
    __device__ uint32_t start_aux() const {
        const uint64_t inv = inverse(start);
        uint32_t a = part(0, inv);
        if (PuzzlePatterns<N>::kNum > 1) a |= part(1, inv) << 8;
        return a;
    }
    __device__ bool is_goal(uint64_t key) const { return key == goal; }
    __device__ __forceinline__ uint64_t f_of(uint64_t, uint64_t g, uint32_t aux) const {
        return g + hsum(aux);
    }
    __device__ __forceinline__ static int blank(uint64_t key) {
        constexpr uint64_t kPad = NN < 16 ? (~0ull << (4 * (NN < 16 ? NN : 0))) : 0ull;
        uint64_t z = ~(key | kPad);
        z = z & (z >> 1) & (z >> 2) & (z >> 3) & 0x1111111111111111ull;
        return (__ffsll((long long)z) - 1) >> 2;
    }
    // Blank moves 0..3 = DX/DY[0..3] of src/utils.hpp:120-121.  The move that
    // would undo the parent's move is skipped: it leads back to the parent,
    // whose g is already lower, so it never improves a slot.
    __device__ uint32_t moves(uint64_t key, uint32_t aux) const {
        const int b = blank(key), bx = b / N, by = b % N;
        uint32_t m = 0;
        if (bx + 1 < N) m |= 1u;
        if (bx > 0) m |= 2u;
        if (by + 1 < N) m |= 4u;
        if (by > 0) m |= 8u;
        const uint32_t last = aux >> 16;
        if (last) m &= ~(1u << ((last - 1) ^ 1));
        return m;
    }
    __device__ void apply(uint64_t key, uint64_t g, uint32_t aux, int mv, uint64_t &nkey,
                          uint64_t &ng, uint32_t &naux, uint64_t &nf) const {
        const int b = blank(key);
        const int q = b + (mv == 0 ? N : mv == 1 ? -N : mv == 2 ? 1 : -1);
        const uint64_t t = (key >> (4 * q)) & 15;
        nkey = (key & ~(15ull << (4 * q))) | (t << (4 * b));
        const uint64_t inv = inverse(nkey);
        uint32_t a = aux & 0xffffu;
        if (pattern_of_tile<N>((int)t) == 0)
            a = (a & 0xff00u) | part(0, inv);
        else
            a = (a & 0x00ffu) | (part(1, inv) << 8);
        naux = a | ((uint32_t)(mv + 1) << 16);
        ng = g + 1;
        nf = ng + hsum(naux);
    }
    // Two-step successor (see GridProblem::Succ): the first step computes the
    // board and issues the load of the moved tile's pattern entry, the second
    // (after the table CAS) folds it into aux and f.
    struct Succ {
        uint64_t key, g;
        uint32_t part;  // the loaded pattern entry
        uint32_t which; // its pattern
    };
    __device__ __forceinline__ void succ_begin(uint64_t key, uint64_t g, uint32_t, int mv, Succ &s) const {
        const int b = blank(key);
        const int q = b + (mv == 0 ? N : mv == 1 ? -N : mv == 2 ? 1 : -1);
        const uint64_t t = (key >> (4 * q)) & 15;
        s.key = (key & ~(15ull << (4 * q))) | (t << (4 * b));
        s.g = g + 1;
        s.which = (uint32_t)pattern_of_tile<N>((int)t);
        s.part = part((int)s.which, inverse(s.key));
    }
    __device__ __forceinline__ void succ_end(const Succ &s, uint32_t aux, int mv, uint32_t &naux,
                                             uint64_t &nf) const {
        uint32_t a = aux & 0xffffu;
        if (s.which == 0)
            a = (a & 0xff00u) | s.part;
        else
            a = (a & 0x00ffu) | (s.part << 8);
        naux = a | ((uint32_t)(mv + 1) << 16);
        nf = s.g + hsum(naux);
    }
    static constexpr bool kEntryKey = false;
    __device__ __forceinline__ Entry make_entry(uint64_t f, uint64_t g, uint32_t slot, uint32_t) const {
        Entry e;
        e.key = ((uint32_t)f << 16) | (0xffffu - (uint32_t)g);
        e.slot = slot;
        return e;
    }
    __device__ __forceinline__ static uint64_t entry_cost(const Entry &e) { return e.key >> 16; }
    __device__ __forceinline__ static bool less(const Entry &a, const Entry &b) { return a.key < b.key; }
    __device__ __forceinline__ static Entry load(const Entry *p) {
        const uint2 u = __ldcg(reinterpret_cast<const uint2 *>(p));
        Entry e;
        e.key = u.x;
        e.slot = u.y;
        return e;
    }
    __device__ __forceinline__ static void store(Entry *p, const Entry &e) {
        *reinterpret_cast<uint2 *>(p) = make_uint2(e.key, e.slot);
    }
    __device__ __forceinline__ static void load_node(const Slot *s, uint64_t &key, uint64_t &g,
                                                     uint32_t &aux) {
        const ulonglong2 v = __ldcg(reinterpret_cast<const ulonglong2 *>(s));
        key = v.x;
        g = v.y >> 40;
        aux = (__ldcg(&s->aux) & 0xffffu) | ((uint32_t)(v.y >> 32) & 0xffu) << kLastMoveShift;
    }
};

// ------------------------------------------------------- 24-puzzle ---
// 5x5 board, 128-bit key: cells 0..11 in `lo` and 12..23 in `hi`, 5 bits
// each; cell 24 is implied (the tiles 0..24 sum to 300), so every state has
// one key and bits 60..63 of both words stay zero (the all-ones empty key is
// never a board).  aux = the four pattern parts, 7 bits each, | (last move +
// 1) << 28.
template <> struct PuzzleProblem<5> : WideSlots {
    using Entry = PuzzleEntry;
    static constexpr int kMoves = 4;
    static constexpr int N = 5;
    static constexpr int NN = 25;
    static constexpr uint64_t kFieldLow = 0x0084210842108421ull;  // bit 0 of each of 12 fields

    const uint8_t *pdb;  // four concatenated tables
    Key128 start;
    Key128 goal;

    __device__ static int cost_cmp(uint64_t a, uint64_t b) { return a < b ? -1 : (a > b ? 1 : 0); }

    __host__ __device__ static uint32_t field(const Key128 &k, int i) {
        if (i < 12) return (uint32_t)(k.lo >> (5 * i)) & 31u;
        if (i < 24) return (uint32_t)(k.hi >> (5 * (i - 12))) & 31u;
        uint32_t sum = 0;
        for (int c = 0; c < 12; ++c) sum += (uint32_t)(k.lo >> (5 * c)) & 31u;
        for (int c = 0; c < 12; ++c) sum += (uint32_t)(k.hi >> (5 * c)) & 31u;
        return 300u - sum;
    }
    __host__ __device__ static void set_field(Key128 &k, int i, uint32_t v) {
        if (i < 12)
            k.lo = (k.lo & ~(31ull << (5 * i))) | ((uint64_t)v << (5 * i));
        else if (i < 24)
            k.hi = (k.hi & ~(31ull << (5 * (i - 12)))) | ((uint64_t)v << (5 * (i - 12)));
        // cell 24 is implied
    }
    __host__ __device__ static Key128 pack(const uint8_t *tiles) {
        Key128 k{0, 0};
        for (int i = 0; i < 24; ++i) set_field(k, i, tiles[i]);
        return k;
    }
    __host__ __device__ static Key128 goal_key() {
        Key128 k{0, 0};
        for (int i = 0; i < 24; ++i) set_field(k, i, (uint32_t)(i + 1));
        return k;
    }
    // index of the zero field of a 60-bit word of 5-bit fields (12 if none)
    __device__ __forceinline__ static int zero_field(uint64_t w) {
        const uint64_t t = w | (w >> 1) | (w >> 2) | (w >> 3) | (w >> 4);
        const uint64_t z = ~t & kFieldLow;
        return z ? (__ffsll((long long)z) - 1) / 5 : 12;
    }
    __device__ __forceinline__ static int blank(const Key128 &k) {
        const int a = zero_field(k.lo);
        if (a < 12) return a;
        const int b = zero_field(k.hi);
        return b < 12 ? 12 + b : 24;
    }
    // cell of each tile, 5 bits per tile, in a 128-bit word
    __device__ __forceinline__ static unsigned __int128 inverse(const Key128 &k) {
        unsigned __int128 inv = 0;
        uint32_t sum = 0;
#pragma unroll
        for (int i = 0; i < 24; ++i) {
            const uint32_t t = i < 12 ? (uint32_t)(k.lo >> (5 * i)) & 31u : (uint32_t)(k.hi >> (5 * (i - 12))) & 31u;
            sum += t;
            inv |= (unsigned __int128)i << (5 * t);
        }
        inv |= (unsigned __int128)24 << (5 * (300u - sum));
        return inv;
    }
    template <int P> __device__ __forceinline__ static uint32_t rank(unsigned __int128 inv) {
        uint32_t used = 0, code = 0;
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            const uint32_t pos = (uint32_t)(inv >> (5 * PuzzlePatterns<5>::tile(P, j))) & 31u;
            const uint32_t v = pos - __popc(used & ((1u << pos) - 1u));
            code += v * pattern_mult<5>(P, j + 1);
            used |= 1u << pos;
        }
        return code;
    }
    __device__ __forceinline__ uint32_t part(int p, unsigned __int128 inv) const {
        switch (p) {
        case 0: return __ldg(pdb + PuzzlePatterns<5>::offset(0) + rank<0>(inv));
        case 1: return __ldg(pdb + PuzzlePatterns<5>::offset(1) + rank<1>(inv));
        case 2: return __ldg(pdb + PuzzlePatterns<5>::offset(2) + rank<2>(inv));
        default: return __ldg(pdb + PuzzlePatterns<5>::offset(3) + rank<3>(inv));
        }
    }
    // aux = four 7-bit pattern parts | (last move + 1) << 28
    static constexpr uint32_t kLastMoveShift = 28;
    __device__ static uint32_t hsum(uint32_t aux) {
        return (aux & 127u) + ((aux >> 7) & 127u) + ((aux >> 14) & 127u) + ((aux >> 21) & 127u);
    }

    __device__ Key128 start_key() const { return start; }
    __device__ uint32_t start_aux() const {
        const unsigned __int128 inv = inverse(start);
        return part(0, inv) | part(1, inv) << 7 | part(2, inv) << 14 | part(3, inv) << 21;
    }
    __device__ bool is_goal(const Key128 &k) const { return k.lo == goal.lo && k.hi == goal.hi; }
    __device__ __forceinline__ uint64_t f_of(const Key128 &, uint64_t g, uint32_t aux) const { return g + hsum(aux); }
    // Blank moves 0..3 = DX/DY[0..3]; the move undoing the parent's is skipped.
    __device__ uint32_t moves(const Key128 &k, uint32_t aux) const {
        const int b = blank(k), bx = b / N, by = b % N;
        uint32_t m = 0;
        if (bx + 1 < N) m |= 1u;
        if (bx > 0) m |= 2u;
        if (by + 1 < N) m |= 4u;
        if (by > 0) m |= 8u;
        const uint32_t last = aux >> 28;
        if (last) m &= ~(1u << ((last - 1) ^ 1));
        return m;
    }
    struct Succ {
        Key128 key;
        uint64_t g;
        uint32_t part;   // the moved tile's pattern entry
        uint32_t which;  // its pattern
    };
    __device__ __forceinline__ void succ_begin(const Key128 &key, uint64_t g, uint32_t, int mv, Succ &s) const {
        const int b = blank(key);
        const int q = b + (mv == 0 ? N : mv == 1 ? -N : mv == 2 ? 1 : -1);
        const uint32_t t = field(key, q);
        s.key = key;
        set_field(s.key, b, t);
        set_field(s.key, q, 0);
        s.g = g + 1;
        s.which = (uint32_t)pattern_of_tile<5>((int)t);
        s.part = part((int)s.which, inverse(s.key));
    }
    __device__ __forceinline__ void succ_end(const Succ &s, uint32_t aux, int mv, uint32_t &naux,
                                             uint64_t &nf) const {
        const uint32_t sh = 7u * s.which;
        uint32_t a = (aux & 0x0fffffffu & ~(127u << sh)) | (s.part << sh);
        naux = a | ((uint32_t)(mv + 1) << 28);
        nf = s.g + hsum(naux);
    }
    static constexpr bool kEntryKey = false;
    __device__ __forceinline__ Entry make_entry(uint64_t f, uint64_t g, uint32_t slot, uint32_t) const {
        Entry e;
        e.key = ((uint32_t)f << 16) | (0xffffu - (uint32_t)g);
        e.slot = slot;
        return e;
    }
    __device__ __forceinline__ static uint64_t entry_cost(const Entry &e) { return e.key >> 16; }
    __device__ __forceinline__ static bool less(const Entry &a, const Entry &b) { return a.key < b.key; }
    __device__ __forceinline__ static Entry load(const Entry *p) {
        const uint2 u = __ldcg(reinterpret_cast<const uint2 *>(p));
        Entry e;
        e.key = u.x;
        e.slot = u.y;
        return e;
    }
    __device__ __forceinline__ static void store(Entry *p, const Entry &e) {
        *reinterpret_cast<uint2 *>(p) = make_uint2(e.key, e.slot);
    }
    __device__ __forceinline__ static void load_node(const Slot *s, Key128 &key, uint64_t &g, uint32_t &aux) {
        const ulonglong2 v = __ldcg(reinterpret_cast<const ulonglong2 *>(s));
        const ulonglong2 w = __ldcg(reinterpret_cast<const ulonglong2 *>(s) + 1);
        key.lo = v.x;
        key.hi = v.y;
        g = w.x;
        aux = (uint32_t)w.y;
    }
};

}  // namespace uastar

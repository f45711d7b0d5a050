"""The cache-line-blocked binary heap of the search kernel
(ga_search.cuh BrickHeap / heap_sift_down / heap_push / heap_push_run /
heap_geometry),
restated in Python and fuzzed against heapq: the index -> global offset map
is a bijection into the heap's block, and pops return the minimum."""
from __future__ import annotations

import heapq
import random

import pytest


def geometry(D, L, want):
    BE = 1 << D
    levels = 0
    while levels < 30 and (1 << levels) - 1 < want:
        levels += 1
    nbl = (levels - L + D - 1) // D if levels > L else 1
    nbl = max(nbl, 1)
    while L + nbl * D > 31:
        nbl -= 1
    bricks = (((1 << (nbl * D)) - 1) << L) // (BE - 1)
    reserve = ((1 << L) + BE - 1) // BE * BE
    return bricks * BE + reserve, (1 << (L + nbl * D)) - 1, reserve


def off(i, D, L):
    BE = 1 << D
    l = i.bit_length() - 1
    r = l - L
    bl, d = divmod(r, D)
    root = i >> d
    local = (1 << d) | (i & ((1 << d) - 1))
    first = (((1 << (bl * D)) - 1) << L) // (BE - 1)
    return (first + (root - (1 << (L + bl * D)))) * BE + local


class BrickHeap:
    def __init__(self, D, L, want):
        self.D, self.L = D, L
        self.stride, self.hcap, self.reserve = geometry(D, L, want)
        self.g = [None] * self.stride
        self.s = [None] * (1 << L)
        self.size = 0
        self.loads = 0

    def topn(self):
        return (1 << self.L) - 1

    def ld(self, i):
        if i <= self.topn():
            return self.s[i]
        self.loads += 1
        return self.g[self.reserve + off(i, self.D, self.L)]

    def st(self, i, v):
        if i <= self.topn():
            self.s[i] = v
        else:
            self.g[self.reserve + off(i, self.D, self.L)] = v

    def fetch(self, root):
        base = self.reserve + off(root, self.D, self.L) - 1
        self.loads += 1
        return self.g[base:base + (1 << self.D)]

    def push(self, v):
        assert self.size + 1 <= self.hcap
        self.size += 1
        now = self.size
        while now > 1:
            par = now >> 1
            pv = self.ld(par)
            if not v < pv:
                break
            self.st(now, pv)
            now = par
        self.st(now, v)

    def climb(self, now, v):
        """heap_climb: fill the vacant position `now` with v."""
        while now > 1:
            par = now >> 1
            pv = self.ld(par)
            if not v < pv:
                break
            self.st(now, pv)
            now = par
        self.st(now, v)

    def push_run(self, vals):
        """heap_push_run: the bottom brick read once and kept across the run."""
        D, L, topn = self.D, self.L, self.topn()
        cached, b = None, None

        def flush():
            nonlocal cached
            if cached is not None:
                base = self.reserve + off(cached, D, L) - 1
                self.g[base:base + (1 << D)] = b
                cached = None

        for x in vals:
            now = self.size + 1
            if now <= topn:
                self.push(x)
                continue
            self.size = now
            r = now.bit_length() - 1 - L
            d = r % D
            root = now >> d
            if root != cached:
                flush()
                # a bottom position that roots its own brick: nothing to read
                b = list(self.fetch(root)) if d > 0 else [None] * (1 << D)
                cached = root
            loc = (1 << d) | (now & ((1 << d) - 1))
            while loc > 1:
                pv = b[loc >> 1]
                if not x < pv:
                    break
                b[loc] = pv
                loc >>= 1
                now >>= 1
            if loc > 1:
                b[loc] = x
                continue
            pv = self.ld(now >> 1)
            if not x < pv:
                b[1] = x
                continue
            b[1] = pv
            flush()
            self.climb(now >> 1, x)
        flush()

    def pop(self):
        out = self.s[1]
        last = self.ld(self.size)
        self.size -= 1
        if self.size:
            self.sift(self.size, last)
        return out

    def pop_chores(self, run):
        """A pop followed by the owner's chores (ga_search.cuh): a root taken
        from the heap is refilled by the run's least entry when there is a run
        (heapreplace: one sift-down, the last entry stays), else by the last
        entry; the rest of the run is pushed as one run."""
        out = self.s[1]
        self.size -= 1
        run = sorted(run)
        if self.size and run:
            self.size += 1
            self.sift(self.size, run[0])
            run = run[1:]
        elif self.size:
            self.sift(self.size, self.ld(self.size + 1))
        self.push_run(run)
        return out

    def sift(self, size, last):
        D, topn = self.D, self.topn()
        now = 1
        while True:
            c = now << 1
            if c > size or c > topn:
                break
            a = self.s[c]
            if c < size and self.s[c + 1] < a:
                a = self.s[c + 1]
                c += 1
            if not a < last:
                self.s[now] = last
                return
            self.s[now] = a
            now = c
        if (now << 1) > size:
            self.st(now, last)
            return
        half, depth, scr = -1, 0, [None, None]
        while True:
            c = now << 1
            if c > size:
                break
            two = c < size
            if half >= 0 and depth + 1 < D:
                la = (1 << (depth + 1)) | (c & ((1 << (depth + 1)) - 1))
                a = scr[half][la]
                b = scr[half][la + 1] if two else None
            else:
                scr[0] = self.fetch(c)
                if two:
                    scr[1] = self.fetch(c + 1)
                a = scr[0][1]
                b = scr[1][1] if two else None
            right = two and b < a
            if right:
                a = b
            if not a < last:
                break
            self.st(now, a)
            if half >= 0 and depth + 1 < D:
                depth += 1
            else:
                half = 1 if right else 0
                depth = 0
            now = c + (1 if right else 0)
        self.st(now, last)


@pytest.mark.parametrize("D,L,want", [(3, 1, 100), (3, 7, 8192), (4, 5, 5000), (4, 1, 70), (3, 4, 3)])
def test_offsets_are_a_bijection_into_the_block(D, L, want):
    stride, hcap, reserve = geometry(D, L, want)
    assert hcap >= min(want, (1 << 31) - 1)
    seen = set()
    for i in range((1 << L), hcap + 1):
        o = off(i, D, L)
        assert reserve + o < stride and o % (1 << D) != 0
        seen.add(o)
    assert len(seen) == hcap + 1 - (1 << L)
    # a brick root sits at local slot 1 of a 128-byte-aligned brick
    assert off(1 << L, D, L) == 1


@pytest.mark.parametrize("D,L", [(3, 1), (3, 3), (4, 2), (4, 5), (3, 7)])
def test_pops_match_heapq(D, L):
    rng = random.Random(D * 100 + L)
    h = BrickHeap(D, L, 3000)
    ref = []
    for step in range(20000):
        if ref and (rng.random() < 0.45 or h.size >= h.hcap - 1):
            assert h.pop() == heapq.heappop(ref)
        else:
            v = (rng.randrange(1000), rng.randrange(1 << 20))
            h.push(v)
            heapq.heappush(ref, v)
        assert h.size == len(ref)
    while ref:
        assert h.pop() == heapq.heappop(ref)


def test_sift_waits_on_global_memory_once_per_brick():
    h = BrickHeap(3, 4, 1 << 14)
    rng = random.Random(5)
    for _ in range(10000):
        h.push((rng.random(),))
    h.loads = 0
    for _ in range(100):
        h.pop()
    # depth ~13 with 4 shared levels: ~3 brick bursts + the tail load per pop,
    # against ~9 dependent loads for an unblocked layout
    assert h.loads / 100 <= 2 * 4 + 1


@pytest.mark.parametrize("D,L", [(3, 1), (3, 3), (4, 2), (4, 5), (3, 7)])
def test_pushed_runs_match_heapq(D, L):
    # drains of 1..8 entries between pops, as the owners' chores do
    rng = random.Random(D * 7 + L)
    h = BrickHeap(D, L, 4000)
    ref = []
    for step in range(6000):
        if ref and rng.random() < 0.4:
            assert h.pop() == heapq.heappop(ref)
        elif h.size + 8 < h.hcap:
            run = [(rng.randrange(500), rng.randrange(1 << 20)) for _ in range(rng.randrange(1, 9))]
            h.push_run(run)
            for v in run:
                heapq.heappush(ref, v)
        assert h.size == len(ref)
    while ref:
        assert h.pop() == heapq.heappop(ref)


def test_a_run_reads_its_bottom_brick_once():
    # D = 4, L = 3: positions 64..127 sit at depth 3 of bricks of 8 siblings
    # (rooted at 8..15); large entries climb nowhere, so a run of 4 into
    # positions 73..76 reads one brick
    h = BrickHeap(4, 3, 1 << 14)
    for i in range(72):
        h.push((i,))
    h.loads = 0
    h.push_run([(10 ** 6 + i,) for i in range(4)])
    assert h.loads == 1
    # positions 3001..3004 each root a brick of their own: no brick read,
    # only the parent that each entry is compared with
    for i in range(72, 3000):
        h.push((i,))
    h.loads = 0
    h.push_run([(10 ** 6 + i,) for i in range(4)])
    assert h.loads == 4


@pytest.mark.parametrize("D,L", [(3, 1), (3, 7), (4, 5), (4, 1), (3, 4)])
def test_pop_with_replace_matches_heapq(D, L):
    # each round: a pop, then a drained run of 0..4 entries, the least of
    # which refills the popped root
    rng = random.Random(D * 11 + L)
    h = BrickHeap(D, L, 4000)
    ref = []
    for _ in range(64):
        v = (rng.randrange(500), rng.randrange(1 << 20))
        h.push(v)
        heapq.heappush(ref, v)
    for step in range(6000):
        run = [(rng.randrange(500), rng.randrange(1 << 20)) for _ in range(rng.randrange(0, 5))]
        if not ref or h.size + len(run) >= h.hcap:
            break
        assert h.pop_chores(run) == heapq.heappop(ref)
        for v in run:
            heapq.heappush(ref, v)
        assert h.size == len(ref)
    while ref:
        assert h.pop() == heapq.heappop(ref)

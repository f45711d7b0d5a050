"""The grid expansion's parent-neighbour pruning (GridProblem::entry_moves):
a node reached by move d skips every successor that is its parent or one of
the parent's neighbours.  Checked on the CPU: the packed mask table in the
kernel source equals that geometric rule, and an A* that applies the rule
(any expansion order, here sequential) returns the same exact optimum as one
that does not, on random grids with blocked and open goals."""
from __future__ import annotations

import heapq
import math
import re
from pathlib import Path

import numpy as np
import pytest

from uastar_gb300 import engine as E
from uastar_gb300 import workloads as WL

SRC = Path(__file__).resolve().parents[1] / "uastar_gb300" / "csrc" / "ga_problems.cuh"
# move i = (dx, dy): the reference's direction order (src/utils.hpp:120-122)
DX = [1, -1, 0, 0, 1, 1, -1, -1]
DY = [0, 0, 1, -1, 1, -1, 1, -1]


def pruned_by_rule(d: int) -> int:
    m = 0
    for j in range(8):
        if abs(DX[j] + DX[d]) <= 1 and abs(DY[j] + DY[d]) <= 1:
            m |= 1 << j
    return m


def test_mask_table_is_the_parent_neighbour_rule():
    text = SRC.read_text()
    consts = re.findall(r"0x([0-9a-f]{16})ull >> \(8 \* in\)", text)
    assert len(consts) == 1
    packed = int(consts[0], 16)
    for d in range(8):
        assert (packed >> (8 * d)) & 0xFF == pruned_by_rule(d), d
    # straight moves skip 5 successors, diagonal ones 3; never the move itself
    assert [bin(pruned_by_rule(d)).count("1") for d in range(8)] == [5] * 4 + [3] * 4
    assert all(not (pruned_by_rule(d) >> d) & 1 for d in range(8))


def cost_lt(a, b) -> bool:
    """(straight, diagonal) pairs compared exactly: a0 + a1*sqrt2 < b0 + b1*sqrt2."""
    x, y = a[0] - b[0], a[1] - b[1]
    if x <= 0 and y <= 0:
        return x < 0 or y < 0
    if x >= 0 and y >= 0:
        return False
    return (x * x < 2 * y * y) if y < 0 else (x * x > 2 * y * y and x < 0)


class Key:
    __slots__ = ("f",)

    def __init__(self, f):
        self.f = f

    def __lt__(self, o):
        return cost_lt(self.f, o.f)


def astar(cells: np.ndarray, start, goal, prune: bool):
    H, W = cells.shape

    def h(x, y):
        dx, dy = abs(x - goal[0]), abs(y - goal[1])
        return (max(dx, dy) - min(dx, dy), min(dx, dy))

    g = {start: (0, 0)}
    came = {start: -1}
    heap = [(Key(h(*start)), start, (0, 0))]
    while heap:
        _, node, gn = heapq.heappop(heap)
        if gn != g[node]:
            continue  # stale
        if node == goal:
            return gn
        x, y = node
        if not cells[x, y]:
            continue  # a blocked cell has no out-moves
        skip = pruned_by_rule(came[node]) if prune and came[node] >= 0 else 0
        for i in range(8):
            if (skip >> i) & 1:
                continue
            nx, ny = x + DX[i], y + DY[i]
            if not (0 <= nx < H and 0 <= ny < W) or not (cells[nx, ny] or (nx, ny) == goal):
                continue
            step = (1, 0) if i < 4 else (0, 1)
            ng = (gn[0] + step[0], gn[1] + step[1])
            if (nx, ny) not in g or cost_lt(ng, g[(nx, ny)]):
                g[(nx, ny)] = ng
                came[(nx, ny)] = i
                hh = h(nx, ny)
                heapq.heappush(heap, (Key((ng[0] + hh[0], ng[1] + hh[1])), (nx, ny), ng))
    return None


@pytest.mark.parametrize("seed", range(12))
def test_pruned_search_keeps_the_optimum(seed):
    rng = np.random.default_rng(seed)
    H, W = int(rng.integers(8, 40)), int(rng.integers(8, 40))
    cells = (rng.random((H, W)) >= rng.uniform(0.1, 0.4)).astype(np.uint8)
    start = (int(rng.integers(0, H)), int(rng.integers(0, W)))
    goal = (int(rng.integers(0, H)), int(rng.integers(0, W)))
    cells[start] = 1
    if seed % 3 == 0:
        cells[goal] = 0  # a blocked goal is still entered
    full = astar(cells, start, goal, prune=False)
    pruned = astar(cells, start, goal, prune=True)
    assert full == pruned, (seed, full, pruned)
    if full is not None:
        assert math.isfinite(full[0] + full[1] * math.sqrt(2))


def test_pruned_search_on_generated_grids_matches_the_engine_generator():
    for seed in range(3):
        sp = WL.screened_grid(48, 40, 0.3, 50 + seed, exact=True)
        words = sp.words()
        bits = (words[:, None] >> np.arange(64, dtype=np.uint64)) & np.uint64(1)
        cells = bits.reshape(-1)[: sp.H * sp.W].astype(np.uint8).reshape(sp.H, sp.W)
        assert (E.pack_words(cells) == words).all()
        assert astar(cells, sp.start, sp.goal, True) == astar(cells, sp.start, sp.goal, False) is not None

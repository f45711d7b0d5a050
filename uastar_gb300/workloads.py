"""Seeded synthetic workloads of the engine's benchmarks and parity tests.

No public dataset is involved: every instance is generated from a documented
seed by the engine's own generators, so the CPU oracle and the GPU engine see
identical inputs on any host.

  grid_1000      1000 x 1000 grid, 30 % blocked, start (0,0), goal (999,999)
  grid_20000     20000 x 20000 grid (4e8 cells, 50 MB bitmap), 30 % blocked,
                 opposite corners; solved with k = 8192 heaps and 2^28 slots
  puzzle15_x100  100 15-puzzles, each a 200-move random walk from the goal
  mixed_1024     768 15-puzzles (walks of 60..300 moves) + 256 grids (sides
                 256..4096, block rates 10..40 %)
  serve_stream   Poisson arrivals, 50 % 15-puzzle (walk 60..300), 50 % grid
                 (side 256..8192, block rate 10..40 %)

Meta-parameters are drawn from splitmix64 (the generator the C library uses),
so they do not depend on numpy's random streams.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

from . import engine as E

MASK64 = (1 << 64) - 1


def splitmix64(seed: int, i: int) -> int:
    """Output #i of the splitmix64 stream seeded with `seed` (as in host_utils.cpp)."""
    z = (seed + (i + 1) * 0x9E3779B97F4A7C15) & MASK64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return z ^ (z >> 31)


def uniform(seed: int, i: int) -> float:
    return (splitmix64(seed, i) >> 11) * (1.0 / (1 << 53))


def randint(seed: int, i: int, lo: int, hi: int) -> int:
    """Uniform integer in [lo, hi]."""
    return lo + ((splitmix64(seed, i) >> 32) * (hi - lo + 1) >> 32)


@dataclass(frozen=True)
class GridSpec:
    H: int
    W: int
    rate: float
    seed: int

    @property
    def start(self):
        return (0, 0)

    @property
    def goal(self):
        return (self.H - 1, self.W - 1)

    def words(self):
        return E.gen_grid(self.seed, self.H, self.W, self.rate, self.start, self.goal)

    def instance(self, est_nodes: int = 0) -> E.GridInstance:
        return E.GridInstance(self.words(), self.H, self.W, self.start, self.goal, est_nodes)


@dataclass(frozen=True)
class PuzzleSpec:
    n: int
    walk: int
    seed: int

    def tiles(self):
        return E.gen_puzzle(self.seed, self.n, self.walk)

    def instance(self, est_nodes: int = 0) -> E.PuzzleInstance:
        return E.PuzzleInstance(self.n, self.tiles(), est_nodes)


def screened_grid(H: int, W: int, rate: float, seed: int, limit: int = 200_000, exact: bool = False) -> GridSpec:
    """First seed >= `seed` whose corners are connected (proven, or presumed
    when both bounded searches outgrow `limit` cells)."""
    s = seed
    while True:
        spec = GridSpec(H, W, rate, s)
        w = spec.words()
        ok = E.grid_reachable(w, H, W, spec.start, spec.goal) if exact else \
            E.grid_screen(w, H, W, spec.start, spec.goal, limit) != 0
        if ok:
            return spec
        s += 1


# Seeds below were screened once with grid_reachable (the 1000^2 case) and by
# the reference CPU solver (the 20000^2 case); the fixtures record them.
GRID_1000 = GridSpec(1000, 1000, 0.30, 1)
GRID_20000 = GridSpec(20000, 20000, 0.30, 7)


def puzzle15_x100(count: int = 100, walk: int = 200, seed0: int = 1000):
    return [PuzzleSpec(4, walk, seed0 + i) for i in range(count)]


MIX_SEED = 0x5EED0C4


def mixed_1024(n_puzzles: int = 768, n_grids: int = 256, seed: int = MIX_SEED, max_side: int = 4096):
    """The batched workload: puzzles first, then grids (order is irrelevant to
    the engine, which sorts by estimated work)."""
    specs = []
    for i in range(n_puzzles):
        walk = randint(seed, 3 * i, 60, 300)
        specs.append(PuzzleSpec(4, walk, splitmix64(seed ^ 0xA5A5, i)))
    for j in range(n_grids):
        side = randint(seed + 1, 3 * j, 256, max_side)
        rate = 0.10 + 0.30 * uniform(seed + 1, 3 * j + 1)
        specs.append(screened_grid(side, side, round(rate, 4), splitmix64(seed ^ 0x5A5A, j) & 0xFFFFFFFF))
    return specs


def serve_stream(count: int, rate_per_s: float, seed: int = 0x5E57E, max_side: int = 8192,
                 walks: tuple = (60, 300), min_side: int = 256, workers: int = 0):
    """(arrival offset in seconds, spec) pairs: Poisson arrivals at `rate_per_s`.

    The request mix does not depend on the rate, only the arrival times do.
    Grid seeds are screened for connected corners on `workers` threads (0 =
    every host core; the screen runs in the C library, outside the GIL)."""
    t = 0.0
    times, jobs = [], []
    table = _screen_table(seed, max_side, walks, min_side)
    for i in range(count):
        u = uniform(seed, 4 * i)
        t += -math.log(1.0 - u) / rate_per_s
        times.append(t)
        if uniform(seed, 4 * i + 1) < 0.5:
            jobs.append(PuzzleSpec(4, randint(seed, 4 * i + 2, walks[0], walks[1]), splitmix64(seed ^ 0x77, i)))
        else:
            side = randint(seed, 4 * i + 2, min_side, max_side)
            r = round(0.10 + 0.30 * uniform(seed, 4 * i + 3), 4)
            s0 = splitmix64(seed ^ 0x99, i) & 0xFFFFFFFF
            if table is not None and i < table[0]:
                jobs.append(GridSpec(side, side, r, s0 + table[1].get(i, 0)))
            else:
                jobs.append((side, r, s0))
    specs = parallel_map(lambda j: j if isinstance(j, (PuzzleSpec, GridSpec)) else
                         screened_grid(j[0], j[0], j[1], j[2]), jobs, workers)
    return list(zip(times, specs))


_SCREEN = {}


def _screen_table(seed, max_side, walks, min_side):
    """(count, {index: seeds skipped}) of the recorded screen of the default
    serving stream (serve_stream_screen.json, made by screened_grid on every
    grid of its first `count` requests; a test re-screens a sample), or None
    for any other stream."""
    import json
    from pathlib import Path
    if "t" not in _SCREEN:
        p = Path(__file__).with_name("serve_stream_screen.json")
        _SCREEN["t"] = json.loads(p.read_text()) if p.exists() else None
    t = _SCREEN["t"]
    if t is None or t["stream"] != {"seed": seed, "max_side": max_side, "min_side": min_side,
                                    "walks": list(walks)}:
        return None
    return t["count"], {int(k): v for k, v in t["offsets"].items()}


def parallel_map(fn, items, workers: int = 0):
    """fn over items on a thread pool, results in order (the generators and
    screens are C calls that release the GIL)."""
    import os
    from concurrent.futures import ThreadPoolExecutor
    items = list(items)
    n = workers if workers > 0 else (os.cpu_count() or 1)
    if n <= 1 or len(items) < 2:
        return [fn(x) for x in items]
    with ThreadPoolExecutor(min(n, len(items))) as ex:
        return list(ex.map(fn, items))

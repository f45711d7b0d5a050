"""The reference's Problem interface, backed by the GB300 engine.

Mirrors ``class Problem`` (src/problem.hpp:6-24) and its two instances,
``Pathway`` (src/pathway/pathway.{hpp,cpp}) and ``Puzzle``
(src/puzzle/puzzle.{cuh,cu}), with the same method names, option names and
check semantics, so a caller of the reference's problem API can switch over.
The GPU half (gpuInitialize / gpuSolve) runs on the engine.  This package
ships no CPU solver: cpuInitialize / cpuSolve call the ``cpu_solver`` object
the caller injects (or do nothing, like the reference's --no-cpu).

Options are the reference's vm_options keys (src/main.cpp:117-143): "width",
"height", "input-module" (custom | zigzag | random), "block-rate" (percent,
random module), "seed", "ordinal", "no-cpu", "no-gpu".
"""
from __future__ import annotations

import abc
import io
import os
import struct
import sys
from pathlib import Path
from typing import Callable, Optional

import numpy as np

from . import engine as E

SQRT2_F32 = np.float32(1.4142135623731)  # src/utils.hpp:119


def float_equal(a: float, b: float, max_diff: float = 1e-3, max_ulps: int = 200) -> bool:
    """The reference's float comparison (src/utils.hpp:86-111)."""
    a32, b32 = np.float32(a), np.float32(b)
    if abs(np.float32(a32 - b32)) <= np.float32(max_diff):
        return True
    ia = struct.unpack("<i", struct.pack("<f", float(a32)))[0]
    ib = struct.unpack("<i", struct.pack("<f", float(b32)))[0]
    if (ia < 0) != (ib < 0):
        return False
    return abs(ia - ib) <= max_ulps


class Problem(abc.ABC):
    """src/problem.hpp:6-24."""

    @abc.abstractmethod
    def problemName(self) -> str: ...

    @abc.abstractmethod
    def prepare(self) -> None: ...

    @abc.abstractmethod
    def cpuInitialize(self) -> None: ...

    @abc.abstractmethod
    def gpuInitialize(self) -> None: ...

    @abc.abstractmethod
    def cpuSolve(self) -> None: ...

    @abc.abstractmethod
    def gpuSolve(self) -> None: ...

    @abc.abstractmethod
    def output(self) -> bool: ...


def _read_ints(stream, count: int) -> list[int]:
    out: list[int] = []
    while len(out) < count:
        line = stream.readline()
        if not line:
            raise ValueError(f"expected {count} integers on the input, got {len(out)}")
        out.extend(int(t) for t in line.split())
    return out


# -------------------------------------------------------------------- grid
class Pathway(Problem):
    """8-direction grid pathfinding (src/pathway/pathway.hpp:10-62)."""

    def __init__(self, options: dict, stdin: Optional[io.TextIOBase] = None,
                 cpu_solver: Optional[Callable] = None, engine: Optional[E.Engine] = None,
                 solution_dir: Optional[str] = None):
        if "width" not in options or "height" not in options:
            raise ValueError("Please set the width and height for your graph.")
        self.opts = dict(options)
        self.m_width = int(options["width"])
        self.m_height = int(options["height"])
        self.m_inputModule = options.get("input-module", "custom")
        self.stdin = stdin if stdin is not None else sys.stdin
        self.cpu_solver = cpu_solver
        self.engine = engine
        self.solution_dir = solution_dir
        self.words: Optional[np.ndarray] = None
        self.cpuSolved = self.gpuSolved = False
        self.cpuSuccessful = self.gpuSuccessful = False
        self.cpuOptimal = self.gpuOptimal = 0.0
        self.cpuSolution: list[int] = []
        self.gpuSolution: list[int] = []
        self.gpuResult: Optional[E.GridSolution] = None

    def problemName(self) -> str:
        return "Pathway Finding"

    # geometry helpers (pathway.hpp:64-119)
    def width(self) -> int:
        return self.m_width

    def height(self) -> int:
        return self.m_height

    def size(self) -> int:
        return self.m_width * self.m_height

    def toID(self, x: int, y: int) -> int:
        return x * self.m_width + y

    def toXY(self, i: int) -> tuple[int, int]:
        return divmod(i, self.m_width)

    def inrange(self, x: int, y: int) -> bool:
        return 0 <= x < self.m_height and 0 <= y < self.m_width

    def prepare(self) -> None:
        H, W = self.m_height, self.m_width
        if self.m_inputModule == "custom":
            # src/pathway/input/custom.cpp:14-26: "sx sy ex ey", then H*W ints, 0 = obstacle
            v = _read_ints(self.stdin, 4 + H * W)
            self.m_sx, self.m_sy, self.m_ex, self.m_ey = v[:4]
            cells = np.array(v[4:], dtype=np.int64).reshape(H, W) != 0
            self.words = E.pack_words(cells.astype(np.uint8))
        elif self.m_inputModule == "zigzag":
            gap = _read_ints(self.stdin, 1)[0]
            self.words, (self.m_sx, self.m_sy), (self.m_ex, self.m_ey) = E.gen_zigzag(H, W, gap)
        elif self.m_inputModule == "random":
            rate = float(self.opts.get("block-rate", 50)) / 100.0
            seed = int(self.opts.get("seed", 0))
            self.m_sx, self.m_sy, self.m_ex, self.m_ey = 0, 0, H - 1, W - 1
            self.words = E.gen_grid(seed, H, W, rate, (0, 0), (H - 1, W - 1))
        else:
            raise ValueError("Please set your input-module parameter correctly.")

    def cpuInitialize(self) -> None:
        pass

    def gpuInitialize(self) -> None:
        if self.engine is None:
            self.engine = E.Engine(int(self.opts.get("ordinal", 0)))
        self.engine.grid_load(self.words, self.m_height, self.m_width)

    def cpuSolve(self) -> None:
        if self.cpu_solver is None:
            return
        solved, cost, path = self.cpu_solver(self.words, self.m_height, self.m_width,
                                             (self.m_sx, self.m_sy), (self.m_ex, self.m_ey))
        self.cpuSuccessful, self.cpuOptimal, self.cpuSolution = bool(solved), float(cost), list(path)
        self.cpuSolved = True

    def gpuSolve(self) -> None:
        r = self.engine.grid_solve_loaded((self.m_sx, self.m_sy), (self.m_ex, self.m_ey))
        self.gpuResult = r
        self.gpuSuccessful = r.ok
        if r.ok:
            self.gpuSolution = self.engine.grid_path().tolist()
            _, _, self.gpuOptimal = E.validate_grid_path(self.words, self.m_height, self.m_width,
                                                         (self.m_sx, self.m_sy), (self.m_ex, self.m_ey),
                                                         self.gpuSolution)
        self.gpuSolved = True

    def output(self) -> bool:
        """Pathway::output (src/pathway/pathway.cpp:89-130)."""
        if self.cpuSolved and self.gpuSolved and self.cpuSuccessful != self.gpuSuccessful:
            return False
        if self.cpuSolved and self.cpuSuccessful:
            self.printSolution(self.cpuSolution, "solutionCPU.txt")
            print(f" > Optimal distance from CPU: {self.cpuOptimal:.3f}")
        if self.gpuSolved and self.gpuSuccessful:
            self.printSolution(self.gpuSolution, "solutionGPU.txt")
            print(f" > Optimal distance from GPU: {self.gpuOptimal:.3f}")
        elif self.gpuSolved:
            print("No solution from GPU.")
        if self.cpuSolved and self.gpuSolved and self.cpuSuccessful:
            return float_equal(self.cpuOptimal, self.gpuOptimal)
        return True

    def printSolution(self, path: list[int], filename: str) -> None:
        """Solution file in the reference's layout (pathway.cpp:141-174), with
        the straight/diagonal counts taken over the path's moves."""
        if self.solution_dir is None:
            return
        parts = []
        straight = diagonal = 0
        for k, v in enumerate(path):
            x, y = self.toXY(v)
            if k:
                px, py = self.toXY(path[k - 1])
                if abs(px - x) + abs(py - y) == 2:
                    diagonal += 1
                else:
                    straight += 1
            parts.append(("\n\t" if (k + 1) % 6 == 0 else "") + f"({x} {y})")
        Path(self.solution_dir, filename).write_text(" -> ".join(parts))
        print(f" > Number of -: {straight}, +: {diagonal}")


# ------------------------------------------------------------------ puzzle
# src/puzzle/CPU-solver.hpp:43-102, in the reference's tracked order (it fixes the rank)
PARTITIONS = {3: [[1, 2, 3, 4, 5, 6, 7, 8]],
              4: [[1, 2, 3, 4, 5, 6, 9, 13], [7, 8, 10, 11, 12, 14, 15]],
              5: [[3, 4, 5, 10, 15, 20], [2, 1, 6, 11, 16, 21], [7, 8, 9, 12, 17, 22], [13, 14, 18, 19, 23, 24]]}


def pdb_cache_names(n: int) -> list[str]:
    """database_<n>_<tiles>.bin, the reference's cache names (database.cpp:86-90)."""
    return ["database_%d_%s.bin" % (n, "_".join(map(str, t))) for t in PARTITIONS[n]]


def load_or_build_pdb(engine: E.Engine, n: int, cache_dir: Optional[str]) -> str:
    """Use the reference-compatible cache files when present, else build on the
    GPU (and write the cache files, as fetchDatabase does, database.cpp:86-122)."""
    names = pdb_cache_names(n)
    if cache_dir is not None:
        paths = [Path(cache_dir, nm) for nm in names]
        if all(p.exists() for p in paths):
            data = np.concatenate([np.fromfile(p, dtype=np.uint8) for p in paths])
            if data.size == E.Engine.pdb_bytes(n):
                engine.pdb_load(n, data)
                return "cache"
    engine.pdb_build(n)
    if cache_dir is not None:
        data = engine.pdb_fetch(n)
        off = 0
        for nm, tiles in zip(names, PARTITIONS[n]):
            size = 1
            for i in range(len(tiles)):
                size *= n * n - i
            data[off:off + size].tofile(Path(cache_dir, nm))
            off += size
    return "gpu"


class Puzzle(Problem):
    """Sliding-tile puzzle (src/puzzle/puzzle.cuh:7-46)."""

    def __init__(self, options: dict, stdin: Optional[io.TextIOBase] = None,
                 cpu_solver: Optional[Callable] = None, engine: Optional[E.Engine] = None,
                 pdb_cache_dir: Optional[str] = None, solution_dir: Optional[str] = None):
        w, h = options.get("width"), options.get("height")
        if w is None and h is None:
            raise ValueError("Please set the width or height for your graph.")
        if w is not None and h is not None and int(w) != int(h):
            raise ValueError("Currently we force width must equeal to height.")
        self.n = int(w if w is not None else h)
        if self.n not in (3, 4, 5):
            raise ValueError("This engine solves N=3, N=4 and N=5 puzzles")
        self.opts = dict(options)
        self.stdin = stdin if stdin is not None else sys.stdin
        self.cpu_solver = cpu_solver
        self.engine = engine
        self.pdb_cache_dir = pdb_cache_dir
        self.solution_dir = solution_dir
        self.m_initialState: list[int] = []
        self.cpuSolved = self.gpuSolved = False
        self.cpuSuccessful = self.gpuSuccessful = False
        self.cpuOptimal = self.gpuOptimal = 0
        self.cpuSolution: list[int] = []
        self.gpuSolution: list[int] = []
        self.gpuResult: Optional[E.PuzzleSolution] = None

    def problemName(self) -> str:
        return "Tile Puzzle"

    def length(self) -> int:
        return self.n

    def size(self) -> int:
        return self.n * self.n

    def initialState(self) -> list[int]:
        return list(self.m_initialState)

    def prepare(self) -> None:
        self.m_initialState = _read_ints(self.stdin, self.n * self.n)

    def cpuInitialize(self) -> None:
        pass

    def gpuInitialize(self) -> None:
        if self.engine is None:
            self.engine = E.Engine(int(self.opts.get("ordinal", 0)))
        load_or_build_pdb(self.engine, self.n, self.pdb_cache_dir)

    def cpuSolve(self) -> None:
        if self.cpu_solver is None:
            return
        solved, steps, moves = self.cpu_solver(self.n, self.m_initialState)
        self.cpuSuccessful, self.cpuOptimal, self.cpuSolution = bool(solved), int(steps), list(moves)
        self.cpuSolved = True

    def gpuSolve(self) -> None:
        r = self.engine.puzzle_solve(self.n, self.m_initialState)
        self.gpuResult = r
        self.gpuSuccessful = r.ok
        if r.ok:
            self.gpuOptimal = r.steps
            self.gpuSolution = self.engine.puzzle_moves()
        self.gpuSolved = True

    def output(self) -> bool:
        """Puzzle::output (src/puzzle/puzzle.cu:162-220): exact step equality."""
        if self.cpuSolved and self.gpuSolved and self.cpuSuccessful != self.gpuSuccessful:
            return False
        if self.cpuSolved and self.cpuSuccessful:
            print(f" > Optimal steps from CPU: {self.cpuOptimal}")
        if self.gpuSolved and self.gpuSuccessful:
            print(f" > Optimal steps from GPU: {self.gpuOptimal}")
            self.printSolution(self.gpuSolution, "solutionGPU.txt")
        if self.cpuSolved and self.gpuSolved and self.cpuSuccessful:
            return self.cpuOptimal == self.gpuOptimal
        return True

    def printSolution(self, moves: list[int], filename: str) -> None:
        """Board after every move, in the reference's layout (puzzle.cu:222-259)."""
        if self.solution_dir is None:
            return
        n = self.n
        state = list(self.m_initialState)
        dx, dy = (1, -1, 0, 0), (0, 0, 1, -1)

        def fmt(s):
            return "".join("".join("%4d" % s[i * n + j] for j in range(n)) + "\n" for i in range(n)) + "\n"

        out = [fmt(state)]
        for d in moves:
            b = state.index(0)
            bx, by = divmod(b, n)
            q = (bx + dx[d]) * n + by + dy[d]
            state[b], state[q] = state[q], state[b]
            out.append(fmt(state))
        Path(self.solution_dir, filename).write_text("".join(out))


def solve_problem(problem: Problem, use_cpu: bool = True, use_gpu: bool = True) -> bool:
    """solve_problem of the reference driver (src/main.cpp:60-110)."""
    problem.prepare()
    if use_cpu:
        problem.cpuInitialize()
    if use_gpu:
        problem.gpuInitialize()
    if use_cpu:
        problem.cpuSolve()
    if use_gpu:
        problem.gpuSolve()
    if use_cpu or use_gpu:
        if not problem.output():
            print("ERROR: Output of the CPU and GPU is not consistent!")
            return False
    return True

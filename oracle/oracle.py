"""ctypes binding of oracle/liboracle.so, the CPU restatement of the
reference's A* solvers and PDB generator (oracle/uastar_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the engine package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"


def build() -> Path:
    src = HERE / "uastar_oracle.cpp"
    if not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-f", str(HERE / "Makefile"), "-C", str(HERE.parent)], check=True)
    return LIB


class GridResult(C.Structure):
    _fields_ = [("solved", C.c_int), ("capped", C.c_int), ("cost", C.c_float), ("straight", C.c_int64),
                ("diagonal", C.c_int64), ("generated", C.c_int64), ("expanded", C.c_int64),
                ("path_len", C.c_int64), ("solve_seconds", C.c_double)]


class PuzzleResult(C.Structure):
    _fields_ = [("solved", C.c_int), ("capped", C.c_int), ("steps", C.c_int), ("stored", C.c_int64),
                ("expanded", C.c_int64), ("solve_seconds", C.c_double)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        l = C.CDLL(os.fspath(LIB))
        u64p, i32p = C.POINTER(C.c_uint64), C.POINTER(C.c_int32)
        l.oracle_grid_astar.argtypes = [C.c_int, C.c_int, u64p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int64,
                                        i32p, C.c_int64, C.POINTER(GridResult)]
        l.oracle_grid_astar_exact.argtypes = [C.c_int, C.c_int, u64p, C.c_int, C.c_int, C.c_int, C.c_int,
                                              C.POINTER(GridResult)]
        l.oracle_float_equal.argtypes = [C.c_float, C.c_float]
        l.oracle_pattern_size.restype = C.c_uint64
        l.oracle_pattern_size.argtypes = [C.c_int, i32p, C.c_int]
        l.oracle_pattern_encode.restype = C.c_uint64
        l.oracle_pattern_encode.argtypes = [C.c_int, i32p, C.c_int, C.POINTER(C.c_uint8)]
        l.oracle_pattern_decode.argtypes = [C.c_int, i32p, C.c_int, C.c_uint64, C.POINTER(C.c_uint8)]
        l.oracle_pdb_build.restype = C.c_uint64
        l.oracle_pdb_build.argtypes = [C.c_int, i32p, C.c_int, C.POINTER(C.c_uint8)]
        l.oracle_puzzle_astar.argtypes = [C.c_int, C.POINTER(C.c_uint8), C.POINTER(C.POINTER(C.c_uint8)),
                                          C.c_int64, i32p, C.c_int64, C.POINTER(PuzzleResult)]
        l.oracle_gen_grid.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int,
                                      C.c_int, u64p]
        _lib = l
    return _lib


def gen_grid(seed: int, H: int, W: int, rate: float, start=(0, 0), goal=None) -> np.ndarray:
    """The benchmarks' seeded Bernoulli grid (1 = open), built by the oracle
    library alone (the same bits as the engine's generator)."""
    goal = (H - 1, W - 1) if goal is None else goal
    words = np.zeros((H * W + 63) // 64, dtype=np.uint64)
    if lib().oracle_gen_grid(seed & (2**64 - 1), H, W, float(rate), start[0], start[1], goal[0], goal[1],
                             words.ctypes.data_as(C.POINTER(C.c_uint64))):
        raise ValueError("bad grid parameters")
    return words


def grid_astar(words: np.ndarray, H: int, W: int, start, goal, max_expansions: int = 0, want_path=True):
    """Reference-semantics float32 A* (CPU-solver.cpp). Returns (GridResult, path ndarray or None)."""
    w = np.ascontiguousarray(words, dtype=np.uint64)
    r = GridResult()
    cap = H * W if want_path else 0
    path = np.zeros(max(cap, 1), dtype=np.int32)
    lib().oracle_grid_astar(H, W, w.ctypes.data_as(C.POINTER(C.c_uint64)), start[0], start[1], goal[0], goal[1],
                            max_expansions, path.ctypes.data_as(C.POINTER(C.c_int32)) if want_path else None,
                            cap, C.byref(r))
    return r, (path[: r.path_len].copy() if (want_path and r.solved) else None)


def grid_astar_exact(words: np.ndarray, H: int, W: int, start, goal) -> GridResult:
    w = np.ascontiguousarray(words, dtype=np.uint64)
    r = GridResult()
    lib().oracle_grid_astar_exact(H, W, w.ctypes.data_as(C.POINTER(C.c_uint64)), start[0], start[1], goal[0],
                                  goal[1], C.byref(r))
    return r


def float_equal(a: float, b: float) -> bool:
    return bool(lib().oracle_float_equal(a, b))


def _i32(a):
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.int32))
    return arr, arr.ctypes.data_as(C.POINTER(C.c_int32))


PARTITIONS = {3: [[1, 2, 3, 4, 5, 6, 7, 8]],
              4: [[1, 2, 3, 4, 5, 6, 9, 13], [7, 8, 10, 11, 12, 14, 15]],
              5: [[3, 4, 5, 10, 15, 20], [2, 1, 6, 11, 16, 21], [7, 8, 9, 12, 17, 22], [13, 14, 18, 19, 23, 24]]}


def pattern_size(n: int, tracked) -> int:
    t, p = _i32(tracked)
    return int(lib().oracle_pattern_size(n, p, len(t)))


def pattern_encode(n: int, tracked, conf) -> int:
    t, p = _i32(tracked)
    c = np.ascontiguousarray(np.asarray(conf, dtype=np.uint8))
    return int(lib().oracle_pattern_encode(n, p, len(t), c.ctypes.data_as(C.POINTER(C.c_uint8))))


def pattern_decode(n: int, tracked, code: int) -> np.ndarray:
    t, p = _i32(tracked)
    out = np.zeros(n * n, dtype=np.uint8)
    lib().oracle_pattern_decode(n, p, len(t), code, out.ctypes.data_as(C.POINTER(C.c_uint8)))
    return out


def pdb_build(n: int, tracked) -> np.ndarray:
    t, p = _i32(tracked)
    out = np.zeros(pattern_size(n, tracked), dtype=np.uint8)
    lib().oracle_pdb_build(n, p, len(t), out.ctypes.data_as(C.POINTER(C.c_uint8)))
    return out


def puzzle_astar(n: int, tiles, tables: list[np.ndarray], max_expansions: int = 0):
    """Returns (PuzzleResult, moves list)."""
    t = np.ascontiguousarray(np.asarray(tiles, dtype=np.uint8))
    ptrs = (C.POINTER(C.c_uint8) * len(tables))(*[tb.ctypes.data_as(C.POINTER(C.c_uint8)) for tb in tables])
    moves = np.zeros(1024, dtype=np.int32)
    r = PuzzleResult()
    lib().oracle_puzzle_astar(n, t.ctypes.data_as(C.POINTER(C.c_uint8)), ptrs, max_expansions,
                              moves.ctypes.data_as(C.POINTER(C.c_int32)), 1024, C.byref(r))
    return r, (moves[: r.steps].tolist() if r.solved else [])

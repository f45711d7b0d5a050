"""uastar_gb300: a GB300-native (sm_103a) GA*-style parallel A* engine that
drops in behind uAstar's Problem API.

The search runs in hand-written CUDA kernels (csrc/) exposed through the C ABI
in include/uastar_gpu.h and bound here with ctypes.  There is no CPU fallback:
if the CUDA library is missing, using the engine raises.
"""
from ._lib import LIB_PATH, STATUS_NAMES  # noqa: F401
from .engine import (Engine, EngineError, GridInstance, GridSolution, PuzzleInstance,  # noqa: F401
                     PuzzleSolution, gen_grid, gen_puzzle, gen_zigzag, grid_reachable, now_s,
                     pack_words, unpack_words, validate_grid_path, validate_puzzle_moves)
from .problem import Pathway, Problem, Puzzle, float_equal, solve_problem  # noqa: F401

__all__ = [
    "Engine", "EngineError", "GridInstance", "PuzzleInstance", "GridSolution", "PuzzleSolution",
    "gen_grid", "gen_puzzle", "gen_zigzag", "grid_reachable", "validate_grid_path", "validate_puzzle_moves",
    "pack_words", "unpack_words", "now_s", "Problem", "Pathway", "Puzzle", "float_equal", "solve_problem",
]

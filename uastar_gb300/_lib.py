"""ctypes binding of the engine's C ABI (include/uastar_gpu.h).

The shared library is built in-tree (``python -m uastar_gb300.build``) and
loaded from this package directory.  There is no fallback: if the library is
missing, importing the engine fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libuastar_gb300.so"

# status codes (uastar_gpu.h)
OK, NO_SOLUTION, HEAP_OVERFLOW, ARENA_FULL, HASH_FULL, ITER_LIMIT, CUDA_ERROR, BAD_INPUT, \
    TIMEOUT, RUNNING, CANCELLED, REJECTED = range(12)
STATUS_NAMES = {
    OK: "OK", NO_SOLUTION: "NO_SOLUTION", HEAP_OVERFLOW: "HEAP_OVERFLOW", ARENA_FULL: "ARENA_FULL",
    HASH_FULL: "HASH_FULL", ITER_LIMIT: "ITER_LIMIT", CUDA_ERROR: "CUDA_ERROR", BAD_INPUT: "BAD_INPUT",
    TIMEOUT: "TIMEOUT", RUNNING: "RUNNING", CANCELLED: "CANCELLED", REJECTED: "REJECTED",
}
KIND_GRID, KIND_PUZZLE = 1, 2


class Config(C.Structure):
    _fields_ = [("heaps", C.c_int32), ("block_threads", C.c_int32), ("heap_capacity", C.c_int32),
                ("hash_log2_slots", C.c_int32), ("max_load", C.c_double), ("max_rounds", C.c_int64),
                ("wait_timeout_s", C.c_double), ("threads_per_heap", C.c_int32), ("heap_top_levels", C.c_int32),
                ("dedup", C.c_int32), ("exact_ms", C.c_int32)]


class GridResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("table_grows", C.c_int32), ("straight", C.c_int64),
                ("diagonal", C.c_int64), ("cost", C.c_float), ("pad", C.c_float),
                ("cost_exact", C.c_double), ("expanded", C.c_int64), ("generated", C.c_int64),
                ("pushed", C.c_int64), ("rounds", C.c_int64), ("table_used", C.c_int64),
                ("path_len", C.c_int64), ("kernel_ms", C.c_double), ("solve_ms", C.c_double)]


class PuzzleResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("steps", C.c_int32), ("expanded", C.c_int64),
                ("generated", C.c_int64), ("pushed", C.c_int64), ("rounds", C.c_int64),
                ("table_used", C.c_int64), ("kernel_ms", C.c_double), ("solve_ms", C.c_double),
                ("table_grows", C.c_int32), ("reserved", C.c_int32)]


class BoundedResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("steps", C.c_int32), ("lower_bound", C.c_int32), ("segments", C.c_int32),
                ("expanded", C.c_int64), ("generated", C.c_int64), ("kernel_ms", C.c_double), ("solve_ms", C.c_double),
                ("exact_passes", C.c_int32), ("exact_optimal", C.c_int32), ("exact_nodes", C.c_int64),
                ("exact_ms", C.c_double)]


class Instance(C.Structure):
    _fields_ = [("kind", C.c_int32), ("n", C.c_int32), ("H", C.c_int32), ("W", C.c_int32),
                ("sx", C.c_int32), ("sy", C.c_int32), ("ex", C.c_int32), ("ey", C.c_int32),
                ("words", C.POINTER(C.c_uint64)), ("tiles", C.c_uint8 * 16), ("est_nodes", C.c_int64)]


class InstanceResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("steps", C.c_int32), ("straight", C.c_int64),
                ("diagonal", C.c_int64), ("cost", C.c_float), ("pad", C.c_float),
                ("expanded", C.c_int64), ("generated", C.c_int64), ("rounds", C.c_int64),
                ("attempts", C.c_int32), ("migrations", C.c_int32), ("latency_ms", C.c_double),
                ("device_ms", C.c_double), ("start_ms", C.c_double)]


class BatchConfig(C.Structure):
    _fields_ = [("threads_per_instance", C.c_int32), ("threads_per_heap", C.c_int32),
                ("heap_capacity", C.c_int32), ("load_factor", C.c_double), ("ctas", C.c_int32),
                ("use_graph", C.c_int32), ("tier1_rounds", C.c_int32), ("tier2_puzzle_rounds", C.c_int32),
                ("cluster_size", C.c_int32), ("reserved", C.c_int32)]


class BatchStats(C.Structure):
    _fields_ = [("wall_ms", C.c_double), ("kernel_ms", C.c_double), ("expanded", C.c_int64),
                ("generated", C.c_int64), ("waves", C.c_int32), ("escalated", C.c_int32),
                ("ctas", C.c_int32), ("threads_per_instance", C.c_int32), ("heap_capacity", C.c_int32),
                ("load_factor", C.c_double), ("partition_bytes", C.c_int64)]


class ServeConfig(C.Structure):
    _fields_ = [("hbm_budget_gb", C.c_double), ("slots", C.c_int32), ("threads_per_instance", C.c_int32),
                ("threads_per_heap", C.c_int32), ("heap_capacity", C.c_int32), ("rounds_per_quantum", C.c_int32),
                ("load_factor", C.c_double), ("cluster_slots", C.c_int32), ("quantum_us", C.c_int32)]


class ServeCompletion(C.Structure):
    _fields_ = [("id", C.c_int64), ("result", InstanceResult)]


class ServeStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("rejected", C.c_int64),
                ("cancelled", C.c_int64), ("quanta", C.c_int64), ("busy_ms", C.c_double),
                ("peak_budget_gb", C.c_double), ("peak_resident", C.c_int32), ("reserved", C.c_int32)]


class NoallocGridResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("reserved", C.c_int32), ("straight", C.c_int64),
                ("diagonal", C.c_int64), ("expanded", C.c_int64), ("generated", C.c_int64),
                ("rounds", C.c_int64), ("path_len", C.c_int64)]


# (name, restype, argtypes) for every entry point of uastar_gpu.h
_P = C.c_void_p
_U64P = C.POINTER(C.c_uint64)
_U8P = C.POINTER(C.c_uint8)
_I32P = C.POINTER(C.c_int32)
_I64P = C.POINTER(C.c_int64)
_DP = C.POINTER(C.c_double)
SIGNATURES = [
    ("uastar_create", _P, [C.c_int32, C.POINTER(Config)]),
    ("uastar_destroy", None, [_P]),
    ("uastar_last_error", C.c_char_p, [_P]),
    ("uastar_set_stream", C.c_int32, [_P, _P]),
    ("uastar_kernel_launches", C.c_int64, [_P]),
    ("uastar_build_info", C.c_char_p, []),
    ("uastar_round_floor", C.c_int32, [_P, C.c_int32, _DP, _DP]),
    ("uastar_grid_load", C.c_int32, [_P, _U64P, C.c_int32, C.c_int32]),
    ("uastar_grid_solve_loaded", C.c_int32, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                             C.POINTER(GridResult)]),
    ("uastar_grid_solve", C.c_int32, [_P, _U64P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                      C.c_int32, C.POINTER(GridResult)]),
    ("uastar_grid_path", C.c_int64, [_P, _I32P, C.c_int64]),
    ("uastar_sort_keys", C.c_int32, [_P, C.POINTER(C.c_uint32), C.c_int64, C.c_int32, C.POINTER(C.c_uint32)]),
    ("uastar_pdb_build", C.c_int32, [_P, C.c_int32, _DP]),
    ("uastar_pdb_bytes", C.c_int64, [C.c_int32]),
    ("uastar_pdb_load", C.c_int32, [_P, C.c_int32, _U8P, C.c_int64]),
    ("uastar_pdb_fetch", C.c_int32, [_P, C.c_int32, _U8P, C.c_int64]),
    ("uastar_puzzle_solve", C.c_int32, [_P, C.c_int32, _U8P, C.POINTER(PuzzleResult)]),
    ("uastar_puzzle_moves", C.c_int64, [_P, _I32P, C.c_int64]),
    ("uastar_puzzle_solve_bounded", C.c_int32, [_P, C.c_int32, _U8P, C.c_int32, C.POINTER(BoundedResult)]),
    ("uastar_batch_solve", C.c_int32, [_P, C.POINTER(Instance), C.c_int32, C.POINTER(BatchConfig),
                                       C.POINTER(InstanceResult), C.POINTER(BatchStats)]),
    ("uastar_autotune", C.c_int32, [_P, C.POINTER(Instance), C.c_int32, C.POINTER(BatchConfig)]),
    ("uastar_serve_start", C.c_int32, [_P, C.POINTER(ServeConfig)]),
    ("uastar_serve_submit", C.c_int64, [_P, C.POINTER(Instance), C.c_double]),
    ("uastar_serve_poll", C.c_int32, [_P, C.POINTER(ServeCompletion), C.c_int32]),
    ("uastar_serve_cancel", C.c_int32, [_P, C.c_int64]),
    ("uastar_serve_stop", C.c_int32, [_P, C.c_double, C.POINTER(ServeStats)]),
    ("uastar_now_s", C.c_double, []),
    ("uastar_grid_solve_noalloc", C.c_int32, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                              C.c_int32, _P, C.c_int64, _P, _P]),
    ("uastar_gen_grid", C.c_int32, [C.c_uint64, C.c_int32, C.c_int32, C.c_double, C.c_int32, C.c_int32,
                                    C.c_int32, C.c_int32, _U64P]),
    ("uastar_gen_puzzle", C.c_int32, [C.c_uint64, C.c_int32, C.c_int32, _U8P]),
    ("uastar_gen_zigzag", C.c_int32, [C.c_int32, C.c_int32, C.c_int32, _U64P, _I32P, _I32P, _I32P, _I32P]),
    ("uastar_grid_reachable", C.c_int32, [_U64P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                          C.c_int32]),
    ("uastar_grid_screen", C.c_int32, [_U64P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                       C.c_int32, C.c_int64]),
    ("uastar_validate_grid_path", C.c_int32, [_U64P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                              C.c_int32, _I32P, C.c_int64, _I64P, _I64P,
                                              C.POINTER(C.c_float)]),
    ("uastar_validate_puzzle_moves", C.c_int32, [C.c_int32, _U8P, _I32P, C.c_int64]),
]

_lib = None


def load() -> C.CDLL:
    """Load the in-tree engine library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build the CUDA engine first (python -m uastar_gb300.build); "
            "there is no CPU fallback")
    lib = C.CDLL(os.fspath(LIB_PATH))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib

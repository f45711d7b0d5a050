"""Python face of the GA* engine: an ``Engine`` object over the C ABI plus the
host utilities (seeded generators, reachability screen, path validators).

All search work runs in the CUDA library; this module only marshals buffers.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Iterable, Sequence

import numpy as np

from . import _lib as L


class EngineError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{L.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def _u64p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_uint64))


def _u8p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_uint8))


def _i32p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def grid_words(H: int, W: int) -> int:
    return (H * W + 63) // 64


def _bitmap(words, H: int, W: int) -> np.ndarray:
    """The bitmap as contiguous uint64 words, checked to cover H x W cells:
    the C side reads ceil(H*W/64) words from the pointer it is given."""
    w = np.ascontiguousarray(words, dtype=np.uint64)
    if H > 0 and W > 0 and w.size < grid_words(H, W):
        raise ValueError(f"bitmap of {w.size} words is short of the {grid_words(H, W)} a {H}x{W} grid needs")
    return w


# ------------------------------------------------------------ host utilities
def gen_grid(seed: int, H: int, W: int, block_rate: float, start=(0, 0), goal=None) -> np.ndarray:
    """Seeded Bernoulli grid bitmap (1 = open) with start and goal forced open."""
    lib = L.load()
    goal = (H - 1, W - 1) if goal is None else goal
    words = np.zeros(grid_words(H, W), dtype=np.uint64)
    rc = lib.uastar_gen_grid(seed & (2**64 - 1), H, W, float(block_rate), start[0], start[1], goal[0], goal[1],
                             _u64p(words))
    if rc:
        raise EngineError(rc, "gen_grid")
    return words


def gen_puzzle(seed: int, n: int, walk_len: int) -> np.ndarray:
    """Seeded random walk of blank moves from the goal (no immediate reversal)."""
    lib = L.load()
    tiles = np.zeros(n * n, dtype=np.uint8)
    rc = lib.uastar_gen_puzzle(seed & (2**64 - 1), n, walk_len, _u8p(tiles))
    if rc:
        raise EngineError(rc, "gen_puzzle")
    return tiles


def gen_zigzag(H: int, W: int, height_gap: int):
    """The reference's zig-zag maze; returns (words, (sx, sy), (ex, ey))."""
    lib = L.load()
    words = np.zeros(grid_words(H, W), dtype=np.uint64)
    v = [C.c_int32() for _ in range(4)]
    rc = lib.uastar_gen_zigzag(H, W, height_gap, _u64p(words), *[C.byref(x) for x in v])
    if rc:
        raise EngineError(rc, "gen_zigzag")
    return words, (v[0].value, v[1].value), (v[2].value, v[3].value)


def grid_reachable(words: np.ndarray, H: int, W: int, start, goal) -> bool:
    lib = L.load()
    w = _bitmap(words, H, W)
    return bool(lib.uastar_grid_reachable(_u64p(w), H, W, start[0], start[1], goal[0], goal[1]))


def grid_screen(words: np.ndarray, H: int, W: int, start, goal, limit: int = 200_000) -> int:
    """1 = reachable, 0 = unreachable (proven), 2 = presumed reachable (both sides large)."""
    lib = L.load()
    w = _bitmap(words, H, W)
    return int(lib.uastar_grid_screen(_u64p(w), H, W, start[0], start[1], goal[0], goal[1], limit))


def validate_grid_path(words: np.ndarray, H: int, W: int, start, goal, path: Sequence[int]):
    """Returns (straight, diagonal, float32 cost accumulated in path order) or raises."""
    lib = L.load()
    p = np.ascontiguousarray(np.asarray(path, dtype=np.int32))
    a, b, c = C.c_int64(), C.c_int64(), C.c_float()
    w = _bitmap(words, H, W)
    rc = lib.uastar_validate_grid_path(_u64p(w), H, W, start[0], start[1], goal[0], goal[1], _i32p(p),
                                       len(p), C.byref(a), C.byref(b), C.byref(c))
    if rc:
        raise EngineError(rc, "grid path failed validation")
    return a.value, b.value, c.value


def validate_puzzle_moves(n: int, tiles: Sequence[int], moves: Sequence[int]) -> bool:
    lib = L.load()
    t = np.ascontiguousarray(np.asarray(tiles, dtype=np.uint8))
    m = np.ascontiguousarray(np.asarray(moves, dtype=np.int32))
    return lib.uastar_validate_puzzle_moves(n, _u8p(t), _i32p(m), len(m)) == L.OK


def pack_words(grid01: np.ndarray) -> np.ndarray:
    """(H, W) array of 0/1 (1 = open) -> bitmap words (bit id&63 of word id>>6)."""
    flat = np.asarray(grid01, dtype=np.uint8).reshape(-1)
    nbits = flat.size
    pad = (-nbits) % 64
    bits = np.concatenate([flat, np.zeros(pad, dtype=np.uint8)]).reshape(-1, 64)
    return np.packbits(bits[:, ::-1], axis=1).view(">u8").astype(np.uint64).reshape(-1)


def unpack_words(words: np.ndarray, H: int, W: int) -> np.ndarray:
    b = np.unpackbits(np.asarray(words, dtype=np.uint64).astype(">u8").view(np.uint8).reshape(-1, 8), axis=1)
    b = b.reshape(-1, 64)[:, ::-1].reshape(-1)[: H * W]
    return b.reshape(H, W)


# ------------------------------------------------------------------ results
@dataclass
class GridSolution:
    status: int
    straight: int
    diagonal: int
    cost: float
    cost_exact: float
    expanded: int
    generated: int
    pushed: int
    rounds: int
    table_used: int
    path_len: int
    kernel_ms: float
    solve_ms: float
    table_grows: int = 0

    @property
    def ok(self) -> bool:
        return self.status == L.OK


@dataclass
class PuzzleSolution:
    status: int
    steps: int
    expanded: int
    generated: int
    pushed: int
    rounds: int
    table_used: int
    kernel_ms: float
    solve_ms: float
    table_grows: int = 0

    @property
    def ok(self) -> bool:
        return self.status == L.OK


@dataclass
class GridInstance:
    words: np.ndarray
    H: int
    W: int
    start: tuple
    goal: tuple
    est_nodes: int = 0


@dataclass
class PuzzleInstance:
    n: int
    tiles: np.ndarray
    est_nodes: int = 0


def _to_struct(inst, keep: list) -> L.Instance:
    s = L.Instance()
    if isinstance(inst, GridInstance):
        w = _bitmap(inst.words, inst.H, inst.W)
        keep.append(w)
        s.kind = L.KIND_GRID
        s.H, s.W = inst.H, inst.W
        s.sx, s.sy = inst.start
        s.ex, s.ey = inst.goal
        s.words = _u64p(w)
    else:
        s.kind = L.KIND_PUZZLE
        s.n = inst.n
        for i, t in enumerate(np.asarray(inst.tiles, dtype=np.uint8)):
            s.tiles[i] = int(t)
    s.est_nodes = int(getattr(inst, "est_nodes", 0))
    return s


def _result_dict(r: L.InstanceResult) -> dict:
    return {k: getattr(r, k) for k, _ in L.InstanceResult._fields_ if k not in ("pad", "reserved")}


# ------------------------------------------------------------------- engine
class Engine:
    """One GA* engine on one GPU (drop-in for GPUPathwaySolver / GPUPuzzleSolver)."""

    def __init__(self, ordinal: int = 0, *, heaps: int = 0, block_threads: int = 0, heap_capacity: int = 0,
                 hash_log2_slots: int = 0, max_load: float = 0.0, max_rounds: int = 0,
                 wait_timeout_s: float = 0.0, threads_per_heap: int = 0, heap_top_levels: int = 0,
                 dedup: int = 0, exact_ms: int = 0):
        self._lib = L.load()
        cfg = L.Config(heaps, block_threads, heap_capacity, hash_log2_slots, max_load, max_rounds,
                       wait_timeout_s, threads_per_heap, heap_top_levels, dedup, exact_ms)
        self._h = self._lib.uastar_create(ordinal, C.byref(cfg))
        if not self._h:
            raise EngineError(L.CUDA_ERROR, f"cannot create an engine on CUDA device {ordinal}")

    # lifecycle
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.uastar_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def last_error(self) -> str:
        return self._lib.uastar_last_error(self._h).decode()

    @property
    def kernel_launches(self) -> int:
        return int(self._lib.uastar_kernel_launches(self._h))

    def round_floor(self, rounds: int = 2000) -> tuple[float, float]:
        """Microseconds per round of a bare team barrier, and of one dependent
        16-byte table CAS per thread plus the barrier, on this engine's plain
        launch geometry (uastar_round_floor)."""
        a, b = C.c_double(), C.c_double()
        self._check(self._lib.uastar_round_floor(self._h, rounds, C.byref(a), C.byref(b)), "round_floor")
        return a.value, b.value

    def set_stream(self, stream_ptr: int | None) -> None:
        self._lib.uastar_set_stream(self._h, C.c_void_p(stream_ptr or 0))

    def _check(self, rc: int, what: str, allow=(L.OK,)):
        if rc not in allow:
            raise EngineError(rc, f"{what}: {self.last_error}")

    # grid
    def grid_load(self, words: np.ndarray, H: int, W: int) -> None:
        w = _bitmap(words, H, W)
        self._check(self._lib.uastar_grid_load(self._h, _u64p(w), H, W), "grid_load")

    def _grid_sol(self, r: L.GridResult) -> GridSolution:
        return GridSolution(r.status, r.straight, r.diagonal, r.cost, r.cost_exact, r.expanded, r.generated,
                            r.pushed, r.rounds, r.table_used, r.path_len, r.kernel_ms, r.solve_ms,
                            r.table_grows)

    def grid_solve_loaded(self, start, goal) -> GridSolution:
        r = L.GridResult()
        self._lib.uastar_grid_solve_loaded(self._h, start[0], start[1], goal[0], goal[1], C.byref(r))
        if r.status in (L.CUDA_ERROR, L.BAD_INPUT, L.TIMEOUT):
            raise EngineError(r.status, self.last_error)
        return self._grid_sol(r)

    def grid_solve(self, words: np.ndarray, H: int, W: int, start, goal) -> GridSolution:
        w = _bitmap(words, H, W)
        r = L.GridResult()
        self._lib.uastar_grid_solve(self._h, _u64p(w), H, W, start[0], start[1], goal[0], goal[1], C.byref(r))
        if r.status in (L.CUDA_ERROR, L.BAD_INPUT, L.TIMEOUT):
            raise EngineError(r.status, self.last_error)
        return self._grid_sol(r)

    def grid_path(self) -> np.ndarray:
        n = self._lib.uastar_grid_path(self._h, None, 0)
        if n < 0:
            raise EngineError(-n, "no grid solution")
        out = np.zeros(n, dtype=np.int32)
        self._lib.uastar_grid_path(self._h, _i32p(out), n)
        return out

    def sort_keys(self, keys, key_bits: int = 0) -> np.ndarray:
        """Stable argsort of 32-bit keys by the sorted dedup mode's device
        radix sort (uastar_sort_keys)."""
        k = np.ascontiguousarray(np.asarray(keys, dtype=np.uint32))
        out = np.zeros(k.size, dtype=np.uint32)
        u32p = C.POINTER(C.c_uint32)
        self._check(self._lib.uastar_sort_keys(self._h, k.ctypes.data_as(u32p), k.size, key_bits,
                                               out.ctypes.data_as(u32p)), "sort_keys")
        return out

    # puzzle
    def pdb_build(self, n: int) -> float:
        ms = C.c_double()
        self._check(self._lib.uastar_pdb_build(self._h, n, C.byref(ms)), "pdb_build")
        return ms.value

    @staticmethod
    def pdb_bytes(n: int) -> int:
        return int(L.load().uastar_pdb_bytes(n))

    def pdb_load(self, n: int, tables: np.ndarray) -> None:
        t = np.ascontiguousarray(tables, dtype=np.uint8)
        self._check(self._lib.uastar_pdb_load(self._h, n, _u8p(t), t.size), "pdb_load")

    def pdb_fetch(self, n: int) -> np.ndarray:
        out = np.zeros(self.pdb_bytes(n), dtype=np.uint8)
        self._check(self._lib.uastar_pdb_fetch(self._h, n, _u8p(out), out.size), "pdb_fetch")
        return out

    def puzzle_solve(self, n: int, tiles: Sequence[int]) -> PuzzleSolution:
        t = np.ascontiguousarray(np.asarray(tiles, dtype=np.uint8))
        r = L.PuzzleResult()
        self._lib.uastar_puzzle_solve(self._h, n, _u8p(t), C.byref(r))
        if r.status in (L.CUDA_ERROR, L.BAD_INPUT, L.TIMEOUT):
            raise EngineError(r.status, self.last_error)
        return PuzzleSolution(r.status, r.steps, r.expanded, r.generated, r.pushed, r.rounds, r.table_used,
                              r.kernel_ms, r.solve_ms, r.table_grows)

    def puzzle_solve_bounded(self, n: int, tiles: Sequence[int], max_log2_slots: int) -> dict:
        """Memory-bounded solve (dedup table capped at 2^max_log2_slots slots):
        the returned solution's `steps`, a proven `lower_bound` on the optimum,
        the number of table-capped GA* `segments` (1: optimal) and the exact
        IDA* phase after them (`exact_passes`, `exact_optimal`,
        `exact_nodes`, `exact_ms`; its time is the engine's `exact_ms`)."""
        t = np.ascontiguousarray(np.asarray(tiles, dtype=np.uint8))
        r = L.BoundedResult()
        self._lib.uastar_puzzle_solve_bounded(self._h, n, _u8p(t), max_log2_slots, C.byref(r))
        if r.status in (L.CUDA_ERROR, L.BAD_INPUT, L.TIMEOUT):
            raise EngineError(r.status, self.last_error)
        return {k: getattr(r, k) for k, _ in L.BoundedResult._fields_}

    def puzzle_moves(self) -> list[int]:
        n = self._lib.uastar_puzzle_moves(self._h, None, 0)
        if n < 0:
            raise EngineError(-n, "no puzzle solution")
        out = np.zeros(n, dtype=np.int32)
        self._lib.uastar_puzzle_moves(self._h, _i32p(out), n)
        return out.tolist()

    # batched engine
    def batch_solve(self, instances: Iterable, *, threads_per_instance: int = 0, threads_per_heap: int = 0,
                    heap_capacity: int = 0, load_factor: float = 0.0, ctas: int = 0, use_graph: int = 1,
                    tier1_rounds: int = 0, tier2_puzzle_rounds: int = 0, cluster_size: int = 0):
        insts = list(instances)
        keep: list = []
        arr = (L.Instance * max(1, len(insts)))(*[_to_struct(i, keep) for i in insts])
        res = (L.InstanceResult * max(1, len(insts)))()
        cfg = L.BatchConfig(threads_per_instance, threads_per_heap, heap_capacity, load_factor, ctas, use_graph,
                            tier1_rounds, tier2_puzzle_rounds, cluster_size, 0)
        st = L.BatchStats()
        self._check(self._lib.uastar_batch_solve(self._h, arr, len(insts), C.byref(cfg), res, C.byref(st)),
                    "batch_solve")
        stats = {k: getattr(st, k) for k, _ in L.BatchStats._fields_}
        return [_result_dict(res[i]) for i in range(len(insts))], stats

    def autotune(self, sample: Iterable) -> dict:
        insts = list(sample)
        keep: list = []
        arr = (L.Instance * len(insts))(*[_to_struct(i, keep) for i in insts])
        best = L.BatchConfig()
        self._check(self._lib.uastar_autotune(self._h, arr, len(insts), C.byref(best)), "autotune")
        out = {k: getattr(best, k) for k, _ in L.BatchConfig._fields_}
        out["tried"] = out.pop("reserved")  # configurations timed
        return out

    # serving loop
    def serve_start(self, *, hbm_budget_gb: float = 120.0, slots: int = 0, threads_per_instance: int = 0,
                    threads_per_heap: int = 0, heap_capacity: int = 0, rounds_per_quantum: int = 0,
                    load_factor: float = 0.0, cluster_slots: int = 0, quantum_us: int = 0) -> None:
        cfg = L.ServeConfig(hbm_budget_gb, slots, threads_per_instance, threads_per_heap, heap_capacity,
                            rounds_per_quantum, load_factor, cluster_slots, quantum_us)
        self._check(self._lib.uastar_serve_start(self._h, C.byref(cfg)), "serve_start")

    def serve_submit(self, inst, arrival_s: float = 0.0) -> int:
        keep: list = []
        s = _to_struct(inst, keep)
        rid = self._lib.uastar_serve_submit(self._h, C.byref(s), float(arrival_s))
        if rid < 0:
            raise EngineError(-rid, f"serve_submit: {self.last_error}")
        return int(rid)

    def serve_poll(self, cap: int = 4096) -> list[tuple[int, dict]]:
        buf = (L.ServeCompletion * cap)()
        n = self._lib.uastar_serve_poll(self._h, buf, cap)
        return [(buf[i].id, _result_dict(buf[i].result)) for i in range(max(0, n))]

    def serve_cancel(self, rid: int) -> None:
        self._check(self._lib.uastar_serve_cancel(self._h, rid), "serve_cancel")

    def serve_stop(self, timeout_s: float = 60.0) -> dict:
        st = L.ServeStats()
        rc = self._lib.uastar_serve_stop(self._h, float(timeout_s), C.byref(st))
        self._check(rc, "serve_stop")
        return {k: getattr(st, k) for k, _ in L.ServeStats._fields_ if k != "reserved"}


def now_s() -> float:
    return float(L.load().uastar_now_s())

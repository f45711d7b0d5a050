"""The allocation-free grid solve (uastar_grid_solve_noalloc) through the C
ABI, against the regular engine entry point (uastar_grid_solve).

It serves callers that may not allocate device memory while they run: the
search runs out of a fixed device array the library reserves at load time.
This file is named to be collected last, so that a failure here comes after
every other test has run; it also passes on its own in a fresh process.
The test allocates the caller's device buffers with torch; the entry point
itself allocates nothing.

Tolerance: the exact optimum (straight, diagonal) must be identical to the
regular entry point's, the float32 cost within the reference's float_equal,
and both paths must re-validate on the host."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from uastar_gb300 import Engine
from uastar_gb300 import _lib as L
from uastar_gb300 import engine as E
from uastar_gb300 import workloads as WL
from uastar_gb300.problem import float_equal

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def solve_noalloc(words: np.ndarray, H: int, W: int, start, goal, path_cap: int):
    lib = L.load()
    dev = torch.device("cuda", 0)
    d_words = torch.from_numpy(words.view(np.int64).copy()).to(dev)
    d_path = torch.full((path_cap,), -1, dtype=torch.int32, device=dev)
    d_res = torch.zeros(C.sizeof(L.NoallocGridResult), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = lib.uastar_grid_solve_noalloc(C.c_void_p(d_words.data_ptr()), H, W, start[0], start[1], goal[0], goal[1],
                                       C.c_void_p(d_path.data_ptr()), path_cap, C.c_void_p(d_res.data_ptr()),
                                       C.c_void_p(stream.cuda_stream))
    assert rc == L.OK
    torch.cuda.synchronize(dev)
    res = L.NoallocGridResult.from_buffer_copy(d_res.cpu().numpy().tobytes())
    return res, d_path.cpu().numpy()[: max(0, res.path_len)]


def check_pair(words, H, W, start, goal, ref):
    res, path = solve_noalloc(words, H, W, start, goal, path_cap=H * W + 1)
    assert res.status == L.OK, res.status
    assert (res.straight, res.diagonal) == (ref.straight, ref.diagonal)
    a, b, cost = E.validate_grid_path(words, H, W, start, goal, path)
    assert (a, b) == (res.straight, res.diagonal)
    assert float_equal(cost, ref.cost)
    return res


def test_noalloc_matches_regular_entry_point_twice_in_a_row():
    # two different grids back to back: the second call must not see the
    # first call's leftovers in the shared array
    specs = [WL.screened_grid(600, 500, 0.3, 21, exact=True), WL.screened_grid(256, 301, 0.2, 5, exact=True)]
    with Engine(0) as eng:
        for sp in specs:
            w = sp.words()
            ref = eng.grid_solve(w, sp.H, sp.W, sp.start, sp.goal)
            assert ref.ok
            check_pair(w, sp.H, sp.W, sp.start, sp.goal, ref)
        # and the same grid twice
        sp = specs[0]
        w = sp.words()
        ref = eng.grid_solve(w, sp.H, sp.W, sp.start, sp.goal)
        r1 = check_pair(w, sp.H, sp.W, sp.start, sp.goal, ref)
        r2 = check_pair(w, sp.H, sp.W, sp.start, sp.goal, ref)
        assert (r1.straight, r1.diagonal) == (r2.straight, r2.diagonal)


def test_noalloc_rejects_oversized_grids_and_reports_unreachable():
    lib = L.load()
    dev = torch.device("cuda", 0)
    d_words = torch.zeros(16, dtype=torch.int64, device=dev)
    d_path = torch.zeros(16, dtype=torch.int32, device=dev)
    d_res = torch.zeros(C.sizeof(L.NoallocGridResult), dtype=torch.uint8, device=dev)
    rc = lib.uastar_grid_solve_noalloc(C.c_void_p(d_words.data_ptr()), 4096, 4096, 0, 0, 1, 1,
                                       C.c_void_p(d_path.data_ptr()), 16, C.c_void_p(d_res.data_ptr()), None)
    assert rc == L.BAD_INPUT  # 2^24 cells: above the fixed array's maximum of 2^22
    g = np.ones((40, 40), dtype=np.uint8)
    g[20, :] = 0
    res, path = solve_noalloc(E.pack_words(g), 40, 40, (0, 0), (39, 39), 64)
    assert res.status == L.NO_SOLUTION and res.path_len == 0


def test_noalloc_reports_a_short_path_buffer_and_a_full_table():
    # a solvable grid whose path is longer than the caller's buffer
    sp = WL.screened_grid(300, 300, 0.2, 8, exact=True)
    res, _ = solve_noalloc(sp.words(), sp.H, sp.W, sp.start, sp.goal, path_cap=50)
    assert res.status == L.ARENA_FULL and res.path_len == 0
    # a goal walled off from a start whose component (1500 x 2048 open
    # cells) is larger than the fixed table's 0.8 * 2^20 slots
    g = np.ones((2048, 2048), dtype=np.uint8)
    g[1500, :] = 0
    res, _ = solve_noalloc(E.pack_words(g), 2048, 2048, (0, 0), (2047, 2047), 64)
    assert res.status == L.HASH_FULL and res.path_len == 0

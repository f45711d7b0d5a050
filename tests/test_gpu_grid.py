"""GPU grid engine (plain, whole-GPU team) against the reference's results.

Parity bar: the same number of straight and diagonal
steps as the reference's CPU A*, its float32 cost within the reference's own
tolerance (float_equal: 1e-3 absolute or 200 ULPs, src/utils.hpp:86-111), and
a path that re-validates on the host."""
from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from conftest import golden
from uastar_gb300 import Engine, EngineError
from uastar_gb300 import _lib as L
from uastar_gb300 import engine as E
from uastar_gb300 import workloads as WL
from uastar_gb300.problem import float_equal

pytestmark = pytest.mark.gpu


def case_words(c):
    if c["kind"] == "custom":
        return E.pack_words(np.array(c["cells"], dtype=np.uint8).reshape(c["H"], c["W"]))
    if c["kind"] == "zigzag":
        return E.gen_zigzag(c["H"], c["W"], c["height_gap"])[0]
    return WL.GridSpec(c["H"], c["W"], c["rate"], c["seed"]).words()


def check_against(r, path, words, c):
    ref = c["ref"]
    assert r.ok == ref["solved"], c["name"]
    assert (r.straight, r.diagonal) == (ref["straight"], ref["diagonal"]), c["name"]
    assert float_equal(r.cost, ref["cost"]), (c["name"], r.cost, ref["cost"])
    a, b, fc = E.validate_grid_path(words, c["H"], c["W"], tuple(c["start"]), tuple(c["goal"]), path)
    assert (a, b) == (r.straight, r.diagonal)
    assert len(path) == r.path_len


@pytest.mark.parametrize("heaps,block,tph,levels", [(8192, 256, 4, 0), (8192, 128, 1, -1), (1024, 64, 2, 3),
                                                    (32, 32, 1, 2), (64, 512, 8, 0)])
def test_golden_small_grids(heaps, block, tph, levels):
    with Engine(0, heaps=heaps, block_threads=block, threads_per_heap=tph, heap_top_levels=levels) as eng:
        for c in golden("grid_small.json"):
            w = case_words(c)
            r = eng.grid_solve(w, c["H"], c["W"], tuple(c["start"]), tuple(c["goal"]))
            check_against(r, eng.grid_path(), w, c)


def test_grid_1000(engine):
    c = golden("grid_c1.json")
    w = case_words(c)
    r = engine.grid_solve(w, c["H"], c["W"], tuple(c["start"]), tuple(c["goal"]))
    check_against(r, engine.grid_path(), w, c)
    assert r.expanded > 0 and r.rounds >= r.path_len - 1


def test_grid_resident_bitmap_matches_host_call(engine):
    c = golden("grid_c1.json")
    w = case_words(c)
    engine.grid_load(w, c["H"], c["W"])
    r1 = engine.grid_solve_loaded(tuple(c["start"]), tuple(c["goal"]))
    p1 = engine.grid_path()
    r2 = engine.grid_solve(w, c["H"], c["W"], tuple(c["start"]), tuple(c["goal"]))
    assert (r1.straight, r1.diagonal) == (r2.straight, r2.diagonal)
    E.validate_grid_path(w, c["H"], c["W"], tuple(c["start"]), tuple(c["goal"]), p1)


@pytest.mark.parametrize("H,W,rate,seed", [(200, 300, 0.3, 5), (512, 512, 0.35, 9), (777, 333, 0.15, 2),
                                            (1, 500, 0.0, 1), (400, 1, 0.0, 1)])
def test_live_oracle(engine, H, W, rate, seed):
    sp = WL.screened_grid(H, W, rate, seed, exact=True)
    w = sp.words()
    r = engine.grid_solve(w, H, W, sp.start, sp.goal)
    ref, _ = O.grid_astar(w, H, W, sp.start, sp.goal, want_path=False)
    ex = O.grid_astar_exact(w, H, W, sp.start, sp.goal)
    assert r.ok and ref.solved
    assert (r.straight, r.diagonal) == (ex.straight, ex.diagonal) == (ref.straight, ref.diagonal)
    assert float_equal(r.cost, ref.cost)


def test_unreachable_goal(engine):
    g = np.ones((40, 40), dtype=np.uint8)
    g[20, :] = 0
    w = E.pack_words(g)
    r = engine.grid_solve(w, 40, 40, (0, 0), (39, 39))
    assert r.status == L.NO_SOLUTION
    with pytest.raises(EngineError):
        engine.grid_path()
    assert O.grid_astar(w, 40, 40, (0, 0), (39, 39))[0].solved == 0


def test_bad_inputs(engine):
    w = E.pack_words(np.ones((4, 4), dtype=np.uint8))
    with pytest.raises(EngineError):
        engine.grid_solve(w, 4, 4, (0, 0), (4, 4))
    with pytest.raises(EngineError):
        engine.grid_solve(w, 0, 4, (0, 0), (0, 0))
    big = np.zeros(E.grid_words(46341, 46341), dtype=np.uint64)  # untouched pages
    with pytest.raises(EngineError):  # 2^31 cells or more: path ids would not fit int32
        engine.grid_solve(big, 46341, 46341, (0, 0), (1, 1))
    with Engine(0, hash_log2_slots=32) as eng:  # above the 2^31-slot table limit
        with pytest.raises(EngineError):
            eng.grid_solve(w, 4, 4, (0, 0), (3, 3))


def test_small_fixed_table_reports_hash_full():
    sp = WL.screened_grid(300, 300, 0.2, 1, exact=True)
    with Engine(0, hash_log2_slots=10) as eng:
        r = eng.grid_solve(sp.words(), 300, 300, sp.start, sp.goal)
        assert r.status == L.HASH_FULL


def test_auto_table_grows_on_overflow():
    # the auto-sized table of the 1000^2 grid starts at 2^20 slots and is
    # moved to a 4x table in place when half full; the result is unchanged
    c = golden("grid_c1.json")
    w = case_words(c)
    with Engine(0) as eng:
        r = eng.grid_solve(w, c["H"], c["W"], tuple(c["start"]), tuple(c["goal"]))
        assert r.table_grows >= 1 and r.table_used > (1 << 19)
        check_against(r, eng.grid_path(), w, c)


def test_small_fixed_heaps_report_overflow():
    sp = WL.screened_grid(400, 400, 0.1, 1, exact=True)
    with Engine(0, heaps=32, block_threads=32, threads_per_heap=1, heap_capacity=3, heap_top_levels=-1) as eng:
        r = eng.grid_solve(sp.words(), 400, 400, sp.start, sp.goal)
        assert r.status == L.HEAP_OVERFLOW


def test_round_limit_reports_iter_limit():
    sp = WL.screened_grid(300, 300, 0.2, 1, exact=True)
    with Engine(0, max_rounds=5) as eng:
        r = eng.grid_solve(sp.words(), 300, 300, sp.start, sp.goal)
        assert r.status == L.ITER_LIMIT and r.rounds == 5


def test_problem_api_pathway(tmp_path):
    import io
    from uastar_gb300.problem import Pathway, solve_problem
    text = "0 0 4 4\n1 0 1 1 1\n1 0 1 1 1\n1 0 1 1 1\n1 1 1 0 1\n1 1 1 0 1\n"

    def cpu(words, H, W, s, g):
        r, path = O.grid_astar(words, H, W, s, g)
        return r.solved, r.cost, path.tolist()

    p = Pathway({"width": 5, "height": 5, "input-module": "custom"}, stdin=io.StringIO(text), cpu_solver=cpu,
                solution_dir=str(tmp_path))
    assert solve_problem(p)
    assert (tmp_path / "solutionGPU.txt").exists()
    assert abs(p.gpuOptimal - 8.243) < 1e-3


def test_grid_beyond_2_29_cells():
    """Grids above 2^29 cells carry no incoming move in their entries (all 8
    moves are expanded); cell ids above 2^29 must survive the entry round
    trip.  An open 24000^2 grid (576 M cells): on an open grid the optimum
    from (x0, y0) to (x1, y1) is min(dx, dy) diagonal + |dx - dy| straight."""
    H = W = 24000
    words = np.full((H * W + 63) // 64, np.uint64(0xFFFFFFFFFFFFFFFF), dtype=np.uint64)
    with Engine(0) as eng:
        eng.grid_load(words, H, W)
        for (s, g) in [((23990, 23950), (23999, 23999)), ((30, 40), (12, 3)), ((23999, 0), (23950, 7))]:
            r = eng.grid_solve_loaded(s, g)
            dx, dy = abs(s[0] - g[0]), abs(s[1] - g[1])
            assert r.ok and (r.straight, r.diagonal) == (abs(dx - dy), min(dx, dy)), (s, g)
            path = eng.grid_path()
            a, b, _ = E.validate_grid_path(words, H, W, s, g, path)
            assert (a, b) == (r.straight, r.diagonal)
            if s[0] * W > (1 << 29):
                assert int(path.min()) > (1 << 29)  # every cell id above 2^29

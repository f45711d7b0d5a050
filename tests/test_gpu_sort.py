"""The sorted dedup mode: the device radix sort that replaces the reference's
per-round MergesortPairs of the successor list (src/pathway/GPU-solver.cu:218)
and the grid search that removes a round's duplicates by sort + unique
instead of the table's atomic minimum.

The sort is checked against a stable argsort on the host (the reference's
sort library is not in its tree, so its results are pinned by definition);
the sorted search against the reference's golden grids, the live oracle and
the default mode."""
from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from conftest import golden
from test_gpu_grid import case_words, check_against
from uastar_gb300 import Engine, EngineError
from uastar_gb300 import _lib as L
from uastar_gb300 import workloads as WL
from uastar_gb300.problem import float_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def seng():
    with Engine(0, dedup=1) as eng:
        yield eng


def max_keys():
    import torch

    return 2048 * torch.cuda.get_device_properties(0).multi_processor_count


@pytest.mark.parametrize("n,bits,dist", [(1, 0, "uniform"), (2, 1, "uniform"), (1000, 8, "few"),
                                         (4099, 12, "uniform"), (100_000, 0, "uniform"),
                                         (100_000, 29, "few"), (65_536, 20, "equal"),
                                         (50_000, 16, "descending"), (-1, 29, "uniform")])
def test_sort_is_a_stable_argsort(seng, n, bits, dist):
    rng = np.random.default_rng(n + bits)
    if n < 0:
        n = max_keys()  # the largest sort one launch takes
    top = 1 << (bits or 32)
    if dist == "uniform":
        keys = rng.integers(0, top, n, dtype=np.uint64).astype(np.uint32)
    elif dist == "few":
        keys = rng.integers(0, 7, n, dtype=np.uint64).astype(np.uint32) * (top // 8)
    elif dist == "equal":
        keys = np.full(n, top - 1, dtype=np.uint32)
    else:
        keys = (top - 1 - np.arange(n, dtype=np.uint64) % top).astype(np.uint32)
    perm = seng.sort_keys(keys, bits)
    assert (perm == np.argsort(keys, kind="stable")).all()


def test_sort_edges(seng):
    assert seng.sort_keys(np.zeros(0, dtype=np.uint32)).size == 0
    with pytest.raises(EngineError):
        seng.sort_keys(np.array([5, 300], dtype=np.uint32), 8)  # 300 has bits above 8
    with pytest.raises(EngineError):
        seng.sort_keys(np.zeros(max_keys() + 1, dtype=np.uint32))


def test_sorted_golden_small_grids():
    for heaps, block, tph in [(8192, 256, 4), (1024, 64, 2), (64, 512, 8)]:
        with Engine(0, heaps=heaps, block_threads=block, threads_per_heap=tph, dedup=1) as eng:
            for c in golden("grid_small.json"):
                w = case_words(c)
                r = eng.grid_solve(w, c["H"], c["W"], tuple(c["start"]), tuple(c["goal"]))
                check_against(r, eng.grid_path(), w, c)


def test_sorted_grid_1000_equals_default_mode(seng):
    """The 1000x1000 grid (30 % blocked) in both modes: the reference's step counts, and the table grows in
    place at least once from its 2^20-slot start in the sorted mode too."""
    c = golden("grid_c1.json")
    w = case_words(c)
    r = seng.grid_solve(w, c["H"], c["W"], tuple(c["start"]), tuple(c["goal"]))
    check_against(r, seng.grid_path(), w, c)
    with Engine(0) as e0:
        r0 = e0.grid_solve(w, c["H"], c["W"], tuple(c["start"]), tuple(c["goal"]))
    assert (r0.straight, r0.diagonal) == (r.straight, r.diagonal)
    assert r.generated > 0 and r.rounds >= r.path_len - 1
    assert r.table_grows >= 1 and r.table_used > (1 << 19)


@pytest.mark.parametrize("H,W,rate,seed", [(300, 200, 0.3, 6), (640, 480, 0.35, 3), (1, 700, 0.0, 1)])
def test_sorted_live_oracle(seng, H, W, rate, seed):
    sp = WL.screened_grid(H, W, rate, seed, exact=True)
    w = sp.words()
    r = seng.grid_solve(w, H, W, sp.start, sp.goal)
    ref, _ = O.grid_astar(w, H, W, sp.start, sp.goal, want_path=False)
    assert r.ok and ref.solved
    assert (r.straight, r.diagonal) == (ref.straight, ref.diagonal)
    assert float_equal(r.cost, ref.cost)


def test_sorted_full_table_and_blocked_goal():
    from uastar_gb300 import engine as E

    sp = WL.screened_grid(300, 300, 0.2, 1, exact=True)
    with Engine(0, hash_log2_slots=10, dedup=1) as eng:
        r = eng.grid_solve(sp.words(), 300, 300, sp.start, sp.goal)
        assert r.status == L.HASH_FULL
    with Engine(0, dedup=1) as eng:
        cells = np.ones((40, 40), dtype=np.uint8)
        cells[39, 38] = cells[38, 39] = cells[38, 38] = 0  # goal walled in
        r = eng.grid_solve(E.pack_words(cells), 40, 40, (0, 0), (39, 39))
        assert r.status == L.NO_SOLUTION


def test_puzzles_ignore_the_grid_sort_mode():
    with Engine(0, dedup=1) as eng:
        eng.pdb_build(3)
        r = eng.puzzle_solve(3, [8, 1, 3, 4, 0, 2, 7, 6, 5])
        assert r.ok and r.steps == 14


def test_bad_dedup_value_is_rejected():
    with Engine(0, dedup=7) as eng:
        with pytest.raises(EngineError):
            eng.grid_solve(np.zeros(1, dtype=np.uint64), 4, 4, (0, 0), (3, 3))

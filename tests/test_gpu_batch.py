"""Batched persistent engine (one CTA per instance, device work queue, CUDA
graph launch): every instance's result equals the plain engine's and the
reference's, alone and in the mix."""
from __future__ import annotations

import pytest

import oracle as O
from conftest import golden
from uastar_gb300 import Engine
from uastar_gb300 import _lib as L
from uastar_gb300 import engine as E
from uastar_gb300 import workloads as WL
from uastar_gb300.problem import float_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def beng():
    with Engine(0) as eng:
        eng.pdb_build(3)
        eng.pdb_build(4)
        yield eng


def small_mix():
    specs = []
    for i in range(24):
        specs.append(WL.PuzzleSpec(4, 20 + 5 * i, 900 + i))
    for i in range(8):
        specs.append(WL.PuzzleSpec(3, 10 + 4 * i, 50 + i))
    for i, side in enumerate([40, 64, 128, 200, 256, 333, 512, 640]):
        specs.append(WL.screened_grid(side, side + i, 0.1 + 0.04 * i, 7 + i, exact=True))
    return specs


def test_batch_matches_plain_engine(beng):
    specs = small_mix()
    insts = [s.instance() for s in specs]
    res, stats = beng.batch_solve(insts)
    assert stats["waves"] >= 1
    for s, inst, r in zip(specs, insts, res):
        if isinstance(s, WL.PuzzleSpec):
            p = beng.puzzle_solve(s.n, inst.tiles)
            assert r["status"] == L.OK and r["steps"] == p.steps, (s, r)
        else:
            p = beng.grid_solve(inst.words, s.H, s.W, s.start, s.goal)
            assert r["status"] == L.OK and (r["straight"], r["diagonal"]) == (p.straight, p.diagonal), (s, r)
            assert float_equal(r["cost"], p.cost)


@pytest.mark.parametrize("threads", [64, 128, 512])
def test_batch_geometries_agree(beng, threads):
    specs = small_mix()[::3]
    insts = [s.instance() for s in specs]
    base, _ = beng.batch_solve(insts, threads_per_instance=256)
    res, _ = beng.batch_solve(insts, threads_per_instance=threads, heap_capacity=512, load_factor=0.7)
    for a, b in zip(base, res):
        assert a["status"] == b["status"] == L.OK
        assert (a["steps"], a["straight"], a["diagonal"]) == (b["steps"], b["straight"], b["diagonal"])


def test_batch_overflow_retry_preserves_results(beng):
    # tiny partitions force HASH_FULL on the first wave; the retry waves must
    # still return the optimum
    specs = [WL.PuzzleSpec(4, 60, 77), WL.screened_grid(300, 300, 0.2, 3, exact=True)]
    insts = [s.instance(est_nodes=64) for s in specs]
    res, stats = beng.batch_solve(insts)
    assert stats["waves"] >= 2 or stats["escalated"] >= 1
    p = beng.puzzle_solve(4, insts[0].tiles)
    assert res[0]["status"] == L.OK and res[0]["steps"] == p.steps and res[0]["attempts"] >= 2
    ex = O.grid_astar_exact(insts[1].words, 300, 300, (0, 0), (299, 299))
    assert (res[1]["straight"], res[1]["diagonal"]) == (ex.straight, ex.diagonal)


def test_batch_handles_unsolvable_and_bad(beng):
    bad = E.PuzzleInstance(4, [2, 1] + list(range(3, 16)) + [0])
    g = E.GridInstance(E.pack_words(__import__("numpy").ones((3, 3), dtype="uint8")), 3, 3, (0, 0), (2, 2))
    res, _ = beng.batch_solve([bad, g])
    assert res[0]["status"] == L.NO_SOLUTION
    assert res[1]["status"] == L.OK and res[1]["diagonal"] == 2


def test_batch_puzzles_match_golden(beng):
    rows = golden("puzzle_c3.json")[:40]
    insts = [E.PuzzleInstance(4, r["tiles"]) for r in rows]
    res, _ = beng.batch_solve(insts)
    for row, r in zip(rows, res):
        assert r["status"] == L.OK and r["steps"] == row["ref"]["steps"]


def test_autotune_returns_a_working_config(beng):
    specs = small_mix()[::4]
    cfg = beng.autotune([s.instance() for s in specs])
    assert cfg["threads_per_instance"] in (128, 256, 512)
    res, _ = beng.batch_solve([s.instance() for s in specs], threads_per_instance=cfg["threads_per_instance"],
                              heap_capacity=cfg["heap_capacity"], load_factor=cfg["load_factor"])
    assert all(r["status"] == L.OK for r in res)

"""Serving loop (continuous batching): requests arriving while others are on
the device are admitted as slots and memory free up; each result is the same
alone (plain engine) and in the mix; cancellation and budget rejection are
reported on the host."""
from __future__ import annotations

import time

import pytest

from uastar_gb300 import Engine
from uastar_gb300 import _lib as L
from uastar_gb300 import workloads as WL
from uastar_gb300.problem import float_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def seng():
    with Engine(0) as eng:
        eng.pdb_build(4)
        yield eng


def drain(eng, n, timeout=120.0):
    got = {}
    t0 = time.time()
    while len(got) < n and time.time() - t0 < timeout:
        for rid, r in eng.serve_poll():
            got[rid] = r
        time.sleep(0.002)
    return got


def test_stream_results_equal_alone_and_in_mix(seng):
    # moderate instances: every one fits the 16 GB budget of this test
    stream = WL.serve_stream(60, rate_per_s=400.0, max_side=1024, walks=(20, 90), min_side=64)
    insts = [s.instance() for _, s in stream]
    seng.serve_start(hbm_budget_gb=16.0, slots=32, rounds_per_quantum=64)
    t0 = WL.E.now_s() + 0.05
    ids = [seng.serve_submit(inst, t0 + dt) for (dt, _), inst in zip(stream, insts)]
    got = drain(seng, len(ids))
    stats = seng.serve_stop(30.0)
    assert len(got) == len(ids)
    assert stats["completed"] == len(ids) and stats["quanta"] > 1
    assert stats["peak_resident"] > 1  # requests overlapped on the device
    for rid, (dt, spec), inst in zip(ids, stream, insts):
        r = got[rid]
        assert r["latency_ms"] > 0
        if isinstance(spec, WL.PuzzleSpec):
            p = seng.puzzle_solve(4, inst.tiles)
            assert r["status"] == L.OK and r["steps"] == p.steps
        else:
            p = seng.grid_solve(inst.words, spec.H, spec.W, spec.start, spec.goal)
            assert r["status"] == p.status
            if p.ok:
                assert (r["straight"], r["diagonal"]) == (p.straight, p.diagonal)
                assert float_equal(r["cost"], p.cost)


def test_cancel_and_reject(seng):
    # 100 MB: the 8000^2 grid's 8 MB bitmap cannot fit its 5 MB arena
    seng.serve_start(hbm_budget_gb=0.1, slots=4, rounds_per_quantum=16)
    big = WL.GridSpec(8000, 8000, 0.1, 1).instance()
    late = WL.PuzzleSpec(4, 200, 3).instance()
    r_big = seng.serve_submit(big)
    r_late = seng.serve_submit(late, WL.E.now_s() + 30.0)  # not yet arrived
    seng.serve_cancel(r_late)
    got = drain(seng, 2, timeout=30)
    seng.serve_stop(10.0)
    assert got[r_big]["status"] == L.REJECTED
    assert got[r_late]["status"] == L.CANCELLED


def test_wide_searches_move_to_cluster_slots(seng):
    # every request starts on a CTA slot; the 15-puzzles of 200-move walks
    # keep their CTA's heaps saturated and, the GPU being otherwise idle, move
    # to 8-CTA cluster slots with their search state (migrations); the large
    # sparse grids have thin frontiers and stay.  Both tiers' results equal
    # the plain engine's.
    specs = [WL.screened_grid(2100 + 100 * i, 2100 + 100 * i, 0.15, 40 + i, exact=True) for i in range(3)]
    specs += [WL.PuzzleSpec(4, 200, 1000 + i) for i in range(4)]
    specs += [WL.PuzzleSpec(4, 30 + 5 * i, 900 + i) for i in range(4)]
    insts = [s.instance() for s in specs]
    seng.serve_start(hbm_budget_gb=32.0, rounds_per_quantum=128)
    ids = [seng.serve_submit(inst) for inst in insts]
    got = drain(seng, len(ids), timeout=60)
    seng.serve_stop(30.0)
    assert len(got) == len(ids)
    assert max(got[i]["migrations"] for i in ids) >= 1
    for rid, spec, inst in zip(ids, specs, insts):
        r = got[rid]
        if isinstance(spec, WL.PuzzleSpec):
            p = seng.puzzle_solve(4, inst.tiles)
            assert r["status"] == L.OK and r["steps"] == p.steps
        else:
            p = seng.grid_solve(inst.words, spec.H, spec.W, spec.start, spec.goal)
            assert r["status"] == L.OK and p.ok
            assert (r["straight"], r["diagonal"]) == (p.straight, p.diagonal)
            assert float_equal(r["cost"], p.cost)


def test_serving_after_a_batch_and_a_failed_allocation():
    # A batch leaves its team regions cached on the engine; the serving loop
    # takes its budget after them, and a serving budget that cannot be had
    # fails alone: the engine keeps working.
    from uastar_gb300 import EngineError
    with Engine(0) as eng:
        eng.pdb_build(4)
        insts = [s.instance() for s in WL.mixed_1024()[::8]]
        res, _ = eng.batch_solve(insts, load_factor=0.35)
        assert all(r["status"] == L.OK for r in res)
        with pytest.raises(EngineError):
            eng.serve_start(hbm_budget_gb=1e6)
        row = WL.puzzle15_x100(count=1)[0]
        assert eng.puzzle_solve(4, row.tiles()).ok
        eng.serve_start(hbm_budget_gb=120.0)
        reqs = [s.instance() for _, s in WL.serve_stream(16, 1000.0, max_side=512, walks=(20, 60))]
        ids = [eng.serve_submit(inst) for inst in reqs]
        got = drain(eng, len(ids))
        eng.serve_stop(30.0)
        assert len(got) == len(ids) and all(r["status"] == L.OK for r in got.values())
        res2, _ = eng.batch_solve(insts[:32])  # and a batch after serving
        assert all(r["status"] == L.OK for r in res2)

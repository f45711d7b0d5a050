"""GPU pattern-database build and sliding-tile search against the reference.

PDBs must equal the reference's generator byte for byte (sha256 of the
reference's database_<n>_<tiles>.bin files); solves must return the exact
optimal move count of the reference's CPU A*, with moves that replay to the
goal on the host."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

import oracle as O
from conftest import golden
from uastar_gb300 import Engine, EngineError
from uastar_gb300 import _lib as L
from uastar_gb300 import engine as E
from uastar_gb300 import workloads as WL
from uastar_gb300.problem import PARTITIONS, pdb_cache_names

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def peng():
    with Engine(0) as eng:
        eng.pdb_build(3)
        eng.pdb_build(4)
        eng.pdb_build(5)
        yield eng


def test_pdb3_equals_oracle_and_reference(peng):
    t = peng.pdb_fetch(3)
    assert (t == O.pdb_build(3, PARTITIONS[3][0])).all()
    sums = golden("pdb_sha256.json")
    assert hashlib.sha256(t.tobytes()).hexdigest() == sums["database_3_1_2_3_4_5_6_7_8.bin"]["sha256"]


def test_pdb4_equals_reference_files(peng):
    sums = golden("pdb_sha256.json")
    t = peng.pdb_fetch(4)
    off = 0
    for name in pdb_cache_names(4):
        if name not in sums:
            pytest.skip("15-puzzle reference tables not in the fixture")
        n = sums[name]["bytes"]
        assert hashlib.sha256(t[off:off + n].tobytes()).hexdigest() == sums[name]["sha256"], name
        off += n
    assert off == t.size


def test_pdb_load_roundtrip(peng):
    t = peng.pdb_fetch(3)
    with Engine(0) as e2:
        e2.pdb_load(3, t)
        r = e2.puzzle_solve(3, [8, 1, 3, 4, 0, 2, 7, 6, 5])
        assert r.ok and r.steps == 14


def test_puzzle8_golden(peng):
    for row in golden("puzzle3_small.json"):
        r = peng.puzzle_solve(3, row["tiles"])
        assert r.ok and r.steps == row["ref"]["steps"], row
        mv = peng.puzzle_moves()
        assert len(mv) == r.steps and E.validate_puzzle_moves(3, row["tiles"], mv)


def test_puzzle15_small_golden(peng):
    for row in golden("puzzle4_small.json"):
        r = peng.puzzle_solve(4, row["tiles"])
        assert r.ok and r.steps == row["ref"]["steps"], row
        assert E.validate_puzzle_moves(4, row["tiles"], peng.puzzle_moves())


def test_puzzle15_x100_golden(peng):
    rows = golden("puzzle_c3.json")
    assert len(rows) == 100
    for row in rows:
        assert E.gen_puzzle(row["seed"], 4, row["walk"]).tolist() == row["tiles"]
        r = peng.puzzle_solve(4, row["tiles"])
        assert r.ok and r.steps == row["ref"]["steps"], row
        assert E.validate_puzzle_moves(4, row["tiles"], peng.puzzle_moves())


def test_puzzle15_live_oracle(peng):
    tables = peng.pdb_fetch(4)
    t0, t1 = tables[:518918400], tables[518918400:]
    for seed in range(6):
        tiles = E.gen_puzzle(seed + 500, 4, 40 + 10 * seed)
        r = peng.puzzle_solve(4, tiles)
        ref, _ = O.puzzle_astar(4, tiles, [t0, t1])
        assert r.ok and ref.solved and r.steps == ref.steps


def test_unsolvable_and_bad_boards(peng):
    r = peng.puzzle_solve(3, [2, 1, 3, 4, 5, 6, 7, 8, 0])  # one swap: odd permutation
    assert r.status == L.NO_SOLUTION
    r = peng.puzzle_solve(4, [2, 1] + list(range(3, 16)) + [0])
    assert r.status == L.NO_SOLUTION
    with pytest.raises(EngineError):
        peng.puzzle_solve(4, [1, 1] + list(range(3, 16)) + [0])
    r = peng.puzzle_solve(5, [2, 1] + list(range(3, 25)) + [0])  # odd permutation, n odd
    assert r.status == L.NO_SOLUTION
    with pytest.raises(EngineError):
        peng.puzzle_solve(6, list(range(36)))


def test_goal_board_is_zero_moves(peng):
    r = peng.puzzle_solve(4, list(range(1, 16)) + [0])
    assert r.ok and r.steps == 0 and peng.puzzle_moves() == []


def test_missing_pdb_is_reported():
    with Engine(0) as e:
        with pytest.raises(EngineError):
            e.puzzle_solve(3, [8, 1, 3, 4, 0, 2, 7, 6, 5])


def test_table_grows_in_place_hard_puzzle(peng):
    """A hard 15-puzzle (63 moves, ~4e7 expansions) outgrows the auto-sized
    2^22-slot starting table several times; the paused search is moved to a
    4x table each time and resumed, and still returns the reference's optimum."""
    row = golden("mixed_c4.json")[127]
    tiles = E.gen_puzzle(row["seed"], 4, row["walk"])
    r = peng.puzzle_solve(4, tiles)
    assert r.ok and r.steps == row["ref"]["steps"] == 63
    assert r.table_grows >= 2
    assert r.table_used > (1 << 22)
    assert E.validate_puzzle_moves(4, tiles, peng.puzzle_moves())


def test_memory_bounded_mode(peng):
    """Bounded mode: with room to spare one exact segment (the optimum, its
    own lower bound); with the table capped far below the search's needs
    several segments, a valid solution no shorter than the reference's
    optimum, and a lower bound no higher than it."""
    rows = golden("puzzle_c3.json")
    row = rows[0]
    r = peng.puzzle_solve_bounded(4, row["tiles"], 28)
    assert r["status"] == L.OK and r["segments"] == 1
    assert r["steps"] == r["lower_bound"] == row["ref"]["steps"]
    hard = golden("mixed_c4.json")[127]  # 63 moves, ~7.5e7 states
    tiles = E.gen_puzzle(hard["seed"], 4, hard["walk"])
    r = peng.puzzle_solve_bounded(4, tiles, 20)  # 2^20 slots
    opt = hard["ref"]["steps"]
    assert r["status"] == L.OK and r["segments"] > 1
    assert r["lower_bound"] <= opt <= r["steps"]
    assert r["lower_bound"] > 40
    mv = peng.puzzle_moves()
    assert len(mv) == r["steps"] and E.validate_puzzle_moves(4, tiles, mv)


def test_memory_bounded_mode_exact_phase():
    """After the table-capped segments, iterative-deepening passes (memory
    bounded by the search depth, not by the table) reach the reference's
    optimum and prove it: the same answer at every table cap, lower bound =
    length.  Without the exact phase the segments' answer keeps its bound."""
    hard = golden("mixed_c4.json")[127]  # 63 moves
    tiles = E.gen_puzzle(hard["seed"], 4, hard["walk"])
    opt = hard["ref"]["steps"]
    with Engine(0, exact_ms=60000) as e:
        e.pdb_build(4)
        for log2 in (20, 22):
            r = e.puzzle_solve_bounded(4, tiles, log2)
            assert r["status"] == L.OK and r["segments"] > 1
            assert r["exact_optimal"] == 1 and r["exact_passes"] >= 1
            assert r["steps"] == r["lower_bound"] == opt
            mv = e.puzzle_moves()
            assert len(mv) == opt and E.validate_puzzle_moves(4, tiles, mv)
    with Engine(0, exact_ms=-1) as e:
        e.pdb_build(4)
        r = e.puzzle_solve_bounded(4, tiles, 20)
        assert r["status"] == L.OK and r["exact_passes"] == 0
        assert r["lower_bound"] <= opt <= r["steps"]


def test_pdb5_equals_reference_files(peng):
    """The four 6-tile tables of the 5x5 puzzle, byte for byte the reference's
    database_5_<tiles>.bin files (tracked order of CPU-solver.hpp:71-102)."""
    sums = golden("pdb_sha256.json")
    t = peng.pdb_fetch(5)
    off = 0
    for name in pdb_cache_names(5):
        if name not in sums:
            pytest.skip("24-puzzle reference tables not in the fixture")
        n = sums[name]["bytes"]
        assert hashlib.sha256(t[off:off + n].tobytes()).hexdigest() == sums[name]["sha256"], name
        off += n
    assert off == t.size


def test_puzzle24_golden(peng):
    """5x5 boards (16-byte state keys): exact optimal move counts of the
    reference's CPU A*, moves that replay to the goal."""
    for row in golden("puzzle5_small.json"):
        if row["seed"] is not None:
            assert E.gen_puzzle(row["seed"], 5, row["walk"]).tolist() == row["tiles"]
        r = peng.puzzle_solve(5, row["tiles"])
        assert r.ok and r.steps == row["ref"]["steps"], row
        mv = peng.puzzle_moves()
        assert len(mv) == r.steps and E.validate_puzzle_moves(5, row["tiles"], mv)


def test_memory_bounded_24_puzzle(peng):
    """The mode the reference's README describes for puzzles beyond A*'s
    memory: a 5x5 board 400 random moves from the goal, table capped at
    2^23 slots (256 MB) — a valid solution and a proven lower bound under it."""
    tiles = E.gen_puzzle(77, 5, 400)
    r = peng.puzzle_solve_bounded(5, tiles, 23)
    assert r["status"] == L.OK
    assert 0 < r["lower_bound"] <= r["steps"]
    mv = peng.puzzle_moves()
    assert len(mv) == r["steps"] and E.validate_puzzle_moves(5, tiles, mv)


def test_pdb5_load_checks_the_field_width(peng):
    """Loaded 5x5 tables (the reference's cache files) work like built ones;
    an entry above the 7 bits the search keeps per table is refused, and the
    engine then holds no 5x5 tables."""
    t = peng.pdb_fetch(5)
    row = golden("puzzle5_small.json")[0]
    with Engine(0) as e2:
        e2.pdb_load(5, t)
        r = e2.puzzle_solve(5, row["tiles"])
        assert r.ok and r.steps == row["ref"]["steps"]
        bad = t.copy()
        bad[123457] = 200
        with pytest.raises(EngineError):
            e2.pdb_load(5, bad)
        with pytest.raises(EngineError):
            e2.puzzle_solve(5, row["tiles"])

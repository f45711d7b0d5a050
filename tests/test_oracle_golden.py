"""The oracle restatement (oracle/uastar_oracle.cpp) against the golden
fixtures produced by the reference's own CPU solvers.  CPU only."""
from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from conftest import golden
from uastar_gb300 import engine as E
from uastar_gb300 import workloads as WL


def case_words(c):
    if c["kind"] == "custom":
        return E.pack_words(np.array(c["cells"], dtype=np.uint8).reshape(c["H"], c["W"]))
    if c["kind"] == "zigzag":
        return E.gen_zigzag(c["H"], c["W"], c["height_gap"])[0]
    return WL.GridSpec(c["H"], c["W"], c["rate"], c["seed"]).words()


def test_grid_small_cases():
    cases = golden("grid_small.json")
    assert len(cases) >= 20
    for c in cases:
        w = case_words(c)
        s, g = tuple(c["start"]), tuple(c["goal"])
        r, path = O.grid_astar(w, c["H"], c["W"], s, g)
        ref = c["ref"]
        assert r.solved == ref["solved"], c["name"]
        # Equal-f entries leave the reference's queue in node-address order
        # (pair<float, node_t*>, CPU-solver.hpp:22-25), so paths and node counts
        # may differ between runs; the optimum may not.
        assert (r.straight, r.diagonal) == (ref["straight"], ref["diagonal"]), c["name"]
        assert O.float_equal(r.cost, ref["cost"]), c["name"]
        assert E.validate_grid_path(w, c["H"], c["W"], s, g, path)[:2] == (r.straight, r.diagonal)
        ex = O.grid_astar_exact(w, c["H"], c["W"], s, g)
        assert (ex.straight, ex.diagonal) == (ref["straight"], ref["diagonal"]), c["name"]


def test_grid_1000_case():
    c = golden("grid_c1.json")
    w = case_words(c)
    r, path = O.grid_astar(w, c["H"], c["W"], tuple(c["start"]), tuple(c["goal"]))
    assert O.float_equal(r.cost, c["ref"]["cost"])
    assert (r.straight, r.diagonal) == (c["ref"]["straight"], c["ref"]["diagonal"])
    assert E.validate_grid_path(w, c["H"], c["W"], tuple(c["start"]), tuple(c["goal"]), path)[:2] == \
        (r.straight, r.diagonal)


def test_readme_example():
    # README.md:15-23 of the reference: 4 straight + 3 diagonal = 8.243
    c = next(x for x in golden("grid_small.json") if x["name"] == "readme5")
    assert c["ref"]["straight"] == 4 and c["ref"]["diagonal"] == 3
    assert abs(c["ref"]["cost"] - 8.2426) < 1e-3


def test_unreachable_goal_is_no_solution():
    # the reference reads an empty queue here (CPU-solver.cpp:84-87); the
    # restatement reports "not solved" instead
    w = E.pack_words(np.vstack([np.ones((1, 5), np.uint8), np.zeros((1, 5), np.uint8), np.ones((3, 5), np.uint8)]))
    r, _ = O.grid_astar(w, 5, 5, (0, 0), (4, 4))
    assert r.solved == 0
    assert O.grid_astar_exact(w, 5, 5, (0, 0), (4, 4)).solved == 0


def test_float_equal_matches_reference_rule():
    assert O.float_equal(1.0, 1.0005)
    assert not O.float_equal(1.0, 1.01)
    big = np.float32(30000.0)
    assert O.float_equal(float(big), float(np.nextafter(big, np.float32(1e9), dtype=np.float32)))


def test_puzzle8_small_cases():
    rows = golden("puzzle3_small.json")
    table = O.pdb_build(3, O.PARTITIONS[3][0])
    for row in rows:
        r, moves = O.puzzle_astar(3, row["tiles"], [table])
        assert r.solved == row["ref"]["solved"]
        assert r.steps == row["ref"]["steps"]
        assert E.validate_puzzle_moves(3, row["tiles"], moves) and len(moves) == r.steps


def test_pdb8_matches_reference_checksum():
    sums = golden("pdb_sha256.json")
    import hashlib
    t = O.pdb_build(3, O.PARTITIONS[3][0])
    assert hashlib.sha256(t.tobytes()).hexdigest() == sums["database_3_1_2_3_4_5_6_7_8.bin"]["sha256"]


def test_pattern_rank_roundtrip():
    rng = np.random.default_rng(3)
    for n, tracked in [(3, O.PARTITIONS[3][0]), (4, O.PARTITIONS[4][0]), (4, O.PARTITIONS[4][1])]:
        size = O.pattern_size(n, tracked)
        for code in list(rng.integers(0, size, 200)) + [0, size - 1]:
            conf = O.pattern_decode(n, tracked, int(code))
            assert O.pattern_encode(n, tracked, conf) == int(code)

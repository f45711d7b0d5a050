"""Host utilities of the engine library: generators, screens, validators.
They run on the CPU (no kernel launches)."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

from conftest import golden
from uastar_gb300 import engine as E
from uastar_gb300 import workloads as WL


def sha(w):
    return hashlib.sha256(np.asarray(w, dtype="<u8").tobytes()).hexdigest()


def test_generators_reproduce_fixture_instances():
    # the fixtures were generated on another host: identical bitmaps here
    for c in golden("grid_small.json"):
        if c["kind"] == "random":
            assert sha(WL.GridSpec(c["H"], c["W"], c["rate"], c["seed"]).words()) == c["words_sha256"], c["name"]
        if c["kind"] == "zigzag":
            assert sha(E.gen_zigzag(c["H"], c["W"], c["height_gap"])[0]) == c["words_sha256"]
    c1 = golden("grid_c1.json")
    assert sha(WL.GRID_1000.words()) == c1["words_sha256"]


def test_gen_grid_rate_and_forced_endpoints():
    w = E.gen_grid(11, 300, 301, 0.3, (5, 6), (299, 300))
    g = E.unpack_words(w, 300, 301)
    assert g[5, 6] == 1 and g[299, 300] == 1
    assert abs(1.0 - g.mean() - 0.3) < 0.01
    assert (E.unpack_words(E.gen_grid(1, 10, 10, 0.0), 10, 10) == 1).all()
    full = E.unpack_words(E.gen_grid(1, 10, 10, 1.0), 10, 10)
    assert full.sum() == 2  # only the forced corners stay open


def test_gen_puzzle_walk_properties():
    for seed in range(20):
        t = E.gen_puzzle(seed, 4, 200)
        assert sorted(t.tolist()) == list(range(16))
    assert E.gen_puzzle(3, 4, 0).tolist() == list(range(1, 16)) + [0]
    assert (E.gen_puzzle(9, 3, 31) == E.gen_puzzle(9, 3, 31)).all()
    for seed in range(5):
        t = E.gen_puzzle(seed, 5, 60)
        assert sorted(t.tolist()) == list(range(25))


def test_puzzle24_walk_replays():
    # a 5x5 walk undone by the reversed moves reaches the goal (validator on 25 cells)
    t = E.gen_puzzle(7, 5, 0).tolist()
    assert t == list(range(1, 25)) + [0]
    assert E.validate_puzzle_moves(5, t, [])
    assert E.validate_puzzle_moves(5, [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20,
                                       21, 22, 23, 0, 24], [2])
    assert not E.validate_puzzle_moves(5, t, [0])  # off the board


def test_pack_unpack_roundtrip():
    rng = np.random.default_rng(0)
    for H, W in [(1, 1), (1, 64), (3, 65), (17, 33), (64, 64)]:
        g = (rng.random((H, W)) < 0.6).astype(np.uint8)
        assert (E.unpack_words(E.pack_words(g), H, W) == g).all()


def test_reachability_and_screen():
    g = np.ones((6, 6), dtype=np.uint8)
    g[3, :] = 0
    w = E.pack_words(g)
    # row 3 is blocked: cells of row 3 can be entered but not left
    assert not E.grid_reachable(w, 6, 6, (0, 0), (5, 5))
    assert E.grid_reachable(w, 6, 6, (0, 0), (3, 2))  # entering a blocked cell is allowed
    assert E.grid_screen(w, 6, 6, (0, 0), (5, 5), 1000) == 0
    open_ = E.pack_words(np.ones((50, 50), dtype=np.uint8))
    assert E.grid_screen(open_, 50, 50, (0, 0), (49, 49), 10) == 2
    assert E.grid_screen(open_, 50, 50, (0, 0), (49, 49), 100000) == 1


def test_validate_grid_path():
    g = np.ones((4, 4), dtype=np.uint8)
    g[1, 1] = 0
    w = E.pack_words(g)
    with pytest.raises(E.EngineError):
        E.validate_grid_path(w, 4, 4, (0, 0), (3, 3), [0, 5, 10, 15])  # leaves blocked (1,1)
    with pytest.raises(E.EngineError):
        E.validate_grid_path(w, 4, 4, (0, 0), (3, 3), [0, 2, 3, 15])  # not adjacent
    with pytest.raises(E.EngineError):
        E.validate_grid_path(w, 4, 4, (0, 0), (3, 3), [1, 6, 11, 15])  # wrong start
    a, b, c = E.validate_grid_path(w, 4, 4, (0, 0), (3, 3), [0, 1, 6, 11, 15])
    assert (a, b) == (2, 2)
    assert np.float32(c) == np.float32(np.float32(np.float32(np.float32(1) + np.float32(1.4142135623731))
                                                  + np.float32(1.4142135623731)) + np.float32(1))


def test_validate_puzzle_moves():
    t = [1, 2, 3, 4, 5, 6, 7, 0, 8]
    assert E.validate_puzzle_moves(3, t, [2])
    assert not E.validate_puzzle_moves(3, t, [3])
    assert not E.validate_puzzle_moves(3, t, [0])  # off the board
    assert not E.validate_puzzle_moves(3, [1, 1, 3, 4, 5, 6, 7, 0, 8], [2])  # not a permutation


def test_short_bitmaps_are_refused_before_the_c_side():
    """The C functions read ceil(H*W/64) words from the pointer they get; the
    Python wrappers check the array covers the grid first."""
    short = np.zeros(3, dtype=np.uint64)  # 192 cells
    with pytest.raises(ValueError):
        E.grid_reachable(short, 20, 20, (0, 0), (19, 19))
    with pytest.raises(ValueError):
        E.grid_screen(short, 20, 20, (0, 0), (19, 19))
    with pytest.raises(ValueError):
        E.validate_grid_path(short, 20, 20, (0, 0), (19, 19), [0, 21])
    # a list of Python ints is converted, not misread
    words = E.pack_words(np.ones((8, 8), dtype=np.uint8))
    assert E.grid_reachable([int(x) for x in words], 8, 8, (0, 0), (7, 7))


def test_serving_stream_screen_table_matches_the_screen():
    # the recorded screen of the 20000-request serving stream equals a fresh
    # screen on a sample of its grids (those skipped past their first seed
    # and others), and the stream built from it is the screened stream
    import json
    from pathlib import Path
    table = json.loads((Path(WL.__file__).with_name("serve_stream_screen.json")).read_text())
    offsets = {int(k): v for k, v in table["offsets"].items()}
    stream = WL.serve_stream(table["count"], 1.0)
    grids = [i for i, (_, s) in enumerate(stream) if isinstance(s, WL.GridSpec)]
    skipped = sorted(offsets)[::max(1, len(offsets) // 12)][:12]
    plain = [i for i in grids if i not in offsets][::max(1, len(grids) // 12)][:12]
    for i in skipped + plain:
        s = stream[i][1]
        base = WL.splitmix64(0x5E57E ^ 0x99, i) & 0xFFFFFFFF
        assert s.seed == base + offsets.get(i, 0)
        assert WL.screened_grid(s.H, s.W, s.rate, base).seed == s.seed, i


def test_oracle_generator_equals_engine_generator():
    import oracle as O
    for seed, H, W, rate in [(7, 300, 333, 0.3), (1, 1000, 1000, 0.3), (5, 17, 5, 0.9), (3, 1, 70, 0.5)]:
        assert (O.gen_grid(seed, H, W, rate) == E.gen_grid(seed, H, W, rate)).all()

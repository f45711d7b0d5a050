"""The 20000 x 20000 grid (4e8 cells, 30 % blocked) with k = 8192 heaps and a
2^28-slot dedup table, against the reference CPU A* result recorded in the
fixture.  Parity: identical (straight, diagonal) and float_equal cost."""
from __future__ import annotations

import pytest

from conftest import golden
from uastar_gb300 import Engine
from uastar_gb300 import engine as E
from uastar_gb300 import workloads as WL
from uastar_gb300.problem import float_equal

pytestmark = pytest.mark.gpu


def test_grid_20000():
    c = golden("grid_c2.json")
    sp = WL.GRID_20000
    assert (c["H"], c["seed"]) == (sp.H, sp.seed)
    w = sp.words()
    with Engine(0, heaps=8192, block_threads=256, threads_per_heap=4, hash_log2_slots=28) as eng:
        r = eng.grid_solve(w, sp.H, sp.W, sp.start, sp.goal)
        path = eng.grid_path()
    assert r.ok
    ref = c["ref"]
    assert (r.straight, r.diagonal) == (ref["straight"], ref["diagonal"]), (r, ref)
    assert float_equal(r.cost, ref["cost"]), (r.cost, ref["cost"])
    assert E.validate_grid_path(w, sp.H, sp.W, sp.start, sp.goal, path)[:2] == (r.straight, r.diagonal)

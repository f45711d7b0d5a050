"""Host logic of the reference-API mirror (uastar_gb300.problem): input
modules, the result check and the solution-file format.  CPU only."""
from __future__ import annotations

import io

import numpy as np
import pytest

from conftest import golden
from uastar_gb300 import engine as E
from uastar_gb300.problem import Pathway, Puzzle, float_equal, pdb_cache_names

README_INPUT = """0 0 4 4
1 0 1 1 1
1 0 1 1 1
1 0 1 1 1
1 1 1 0 1
1 1 1 0 1
"""


def test_custom_module_parses_reference_format():
    p = Pathway({"width": 5, "height": 5, "input-module": "custom"}, stdin=io.StringIO(README_INPUT))
    p.prepare()
    assert (p.m_sx, p.m_sy, p.m_ex, p.m_ey) == (0, 0, 4, 4)
    c = next(x for x in golden("grid_small.json") if x["name"] == "readme5")
    assert (E.unpack_words(p.words, 5, 5).reshape(-1) == np.array(c["cells"])).all()


def test_zigzag_module():
    p = Pathway({"width": 15, "height": 20, "input-module": "zigzag"}, stdin=io.StringIO("3\n"))
    p.prepare()
    assert (p.m_sx, p.m_sy, p.m_ex, p.m_ey) == (0, 7, 19, 7)
    g = E.unpack_words(p.words, 20, 15)
    assert g[3].tolist() == [0] * 14 + [1] and g[6].tolist() == [1] + [0] * 14


def test_random_module_uses_block_rate_and_seed():
    p = Pathway({"width": 64, "height": 48, "input-module": "random", "block-rate": 25, "seed": 4})
    p.prepare()
    assert (E.gen_grid(4, 48, 64, 0.25) == p.words).all()


def test_bad_options_rejected():
    with pytest.raises(ValueError):
        Pathway({"width": 5})
    with pytest.raises(ValueError):
        Pathway({"width": 5, "height": 5, "input-module": "nope"}).prepare()
    with pytest.raises(ValueError):
        Puzzle({"width": 4, "height": 3})
    with pytest.raises(ValueError):
        Puzzle({"width": 6})


def test_float_equal_rule():
    assert float_equal(8.242641, 8.2426405)
    assert float_equal(20000.0, 20000.3)              # 154 float32 ULPs: within 200
    assert not float_equal(20000.0, 20002.0)
    assert not float_equal(1.0, -1.0)


def test_pdb_cache_names_match_reference():
    assert pdb_cache_names(4) == ["database_4_1_2_3_4_5_6_9_13.bin", "database_4_7_8_10_11_12_14_15.bin"]
    assert pdb_cache_names(3) == ["database_3_1_2_3_4_5_6_7_8.bin"]


def test_output_check_logic_without_gpu():
    p = Pathway({"width": 5, "height": 5}, stdin=io.StringIO(README_INPUT))
    p.cpuSolved = p.gpuSolved = True
    p.cpuSuccessful = p.gpuSuccessful = True
    p.cpuOptimal, p.gpuOptimal = 8.2426414, 8.2426405
    assert p.output()
    p.gpuOptimal = 9.0
    assert not p.output()
    p.gpuSuccessful = False
    assert not p.output()

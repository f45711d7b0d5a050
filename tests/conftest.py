"""Shared test setup: the `gpu` marker, in-tree builds and golden fixtures."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the engine's kernels")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from uastar_gb300 import build as B
    B.build()
    import oracle as O
    O.build()
    yield


def golden(name: str):
    p = GOLDEN / name
    if not p.exists():
        pytest.skip(f"fixture {name} not generated")
    return json.loads(p.read_text())


@pytest.fixture(scope="session")
def engine():
    from uastar_gb300 import Engine
    eng = Engine(0)
    yield eng
    eng.close()

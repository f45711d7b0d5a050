"""The C-ABI library loads and exports every entry point include/uastar_gpu.h
declares, and the ctypes layouts match the header.  No kernel is launched."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

from uastar_gb300 import _lib as L

HEADER = Path(__file__).resolve().parents[1] / "include" / "uastar_gpu.h"


def declared():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(uastar_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    names = declared()
    assert len(names) >= 30
    lib = L.load()
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", str(L.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (uastar_\w+)", out))
    assert set(names) <= exported


def test_bindings_cover_header():
    assert {n for n, _, _ in L.SIGNATURES} == set(declared())


def test_struct_sizes_match_c_layout():
    # sizes computed from the header's field lists (natural alignment, x86-64 / aarch64)
    assert C.sizeof(L.Config) == 56
    assert C.sizeof(L.GridResult) == 104
    assert C.sizeof(L.PuzzleResult) == 72
    assert C.sizeof(L.Instance) == 64
    assert C.sizeof(L.InstanceResult) == 88
    assert C.sizeof(L.ServeCompletion) == 96
    assert C.sizeof(L.BoundedResult) == 72
    assert C.sizeof(L.ServeConfig) == 48


def test_status_codes_match_header():
    text = HEADER.read_text()
    for name, val in [("UASTAR_OK", L.OK), ("UASTAR_NO_SOLUTION", L.NO_SOLUTION),
                      ("UASTAR_HEAP_OVERFLOW", L.HEAP_OVERFLOW), ("UASTAR_HASH_FULL", L.HASH_FULL),
                      ("UASTAR_ITER_LIMIT", L.ITER_LIMIT), ("UASTAR_TIMEOUT", L.TIMEOUT),
                      ("UASTAR_REJECTED", L.REJECTED)]:
        assert re.search(rf"{name}\s*=\s*{val}\b", text), name


def test_build_info_and_pdb_sizes():
    lib = L.load()
    assert b"sm_103a" in lib.uastar_build_info()
    assert lib.uastar_pdb_bytes(3) == 362880
    assert lib.uastar_pdb_bytes(4) == 16 * 15 * 14 * 13 * 12 * 11 * 10 * 9 + 16 * 15 * 14 * 13 * 12 * 11 * 10
    assert lib.uastar_pdb_bytes(5) == 4 * (25 * 24 * 23 * 22 * 21 * 20)
    assert lib.uastar_pdb_bytes(6) == 0

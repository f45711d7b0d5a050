"""The bench's reference arm (the reference's CPU A* on the headline query,
restated in oracle/) on a short bounded sample: it prints the bench line's
keys and loads no library of the engine package.  CPU only."""
from __future__ import annotations

import json
import subprocess
import sys

from conftest import ROOT

PROBE = """
import runpy, sys
sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3',
            '--ref-cap', '200000', '--ref-full-solve', '0']
runpy.run_path('bench.py', run_name='__main__')
maps = open('/proc/self/maps').read()
print('ENGINE_LIBRARY_LOADED', 'libuastar_gb300' in maps)
"""


def test_reference_arm_runs_on_the_oracle_alone():
    out = subprocess.run([sys.executable, "-c", PROBE], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.strip().splitlines() if l.strip()]
    assert lines[-1] == "ENGINE_LIBRARY_LOADED False"
    rec = json.loads(lines[-2])
    assert rec["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "config", "cpu_baseline", "e2e"):
        assert key in rec, key
    assert rec["value"] > 0 and rec["warmup"] >= 3
    assert rec["e2e"]["value"] == rec["value"] and rec["e2e"]["h2d_bytes_per_step"] == 0
    assert rec["cpu_baseline"]["kind"] in ("port", "reference")

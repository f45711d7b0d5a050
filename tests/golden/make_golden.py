"""Generate the golden fixtures of the parity tests by running the reference's
own CPU solvers (built unmodified from the reference sources by
oracle/Makefile.ref into oracle/_ref/) on the engine's seeded instances.

    python tests/golden/make_golden.py small c1      # seconds
    python tests/golden/make_golden.py c3 c4 c2      # minutes (c2 needs ~10 GB RAM)
    python tests/golden/make_golden.py c5            # ~30 min: the serving stream's 512-request sample
    python tests/golden/make_golden.py pdb           # after `ref_puzzle pdb 4` (and 5) cached the tables
    python tests/golden/make_golden.py p24small      # after `ref_puzzle pdb 5`

Each part writes tests/golden/<part>.json.  Grid fixtures store the instance
parameters and a sha256 of the generated bitmap (so a test can check that the
generator reproduces the instance on another host), the reference's float32
cost, the straight/diagonal counts replayed from the reference's path, and the
path itself when it is short.  Only this script reads the reference build;
the tests read the JSON files.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import json
import os
import struct
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from uastar_gb300 import engine as E  # noqa: E402
from uastar_gb300 import workloads as WL  # noqa: E402

GOLDEN = Path(__file__).resolve().parent
REF = ROOT / "oracle" / "_ref"
WORK = Path(tempfile.gettempdir()) / "uastar_golden"
WORK.mkdir(exist_ok=True)
PDB_DIR = REF / "pdb"


def sha(words: np.ndarray) -> str:
    return hashlib.sha256(np.asarray(words, dtype="<u8").tobytes()).hexdigest()


def write_grid(path: Path, words, H, W, s, g):
    with open(path, "wb") as f:
        f.write(b"UAG1")
        f.write(struct.pack("<6i", H, W, s[0], s[1], g[0], g[1]))
        f.write(struct.pack("<Q", len(words)))
        f.write(np.asarray(words, dtype="<u8").tobytes())


def ref_grid(words, H, W, s, g, tag: str, keep_path: bool):
    gp, jp = WORK / f"{tag}.grid", WORK / f"{tag}.json"
    write_grid(gp, words, H, W, s, g)
    subprocess.run([str(REF / "ref_grid"), str(gp), str(jp)], check=True, capture_output=True)
    r = json.loads(jp.read_text())
    out = {"solved": r["solved"], "solve_seconds": r["solve_seconds"]}
    if r["solved"]:
        a, b, c = E.validate_grid_path(words, H, W, s, g, r["path"])
        out.update(cost=r["cost"], straight=a, diagonal=b, generated=r["generated"], path_len=len(r["path"]))
        if keep_path:
            out["path"] = r["path"]
    gp.unlink()
    jp.unlink()
    return out


def grid_case(name, words, H, W, s, g, params, keep_path=True):
    rec = {"name": name, "H": H, "W": W, "start": list(s), "goal": list(g), "words_sha256": sha(words)}
    rec.update(params)
    rec["ref"] = ref_grid(words, H, W, s, g, name, keep_path)
    return rec


def part_small():
    cases = []
    # README example (README.md:15-23): cost 8.243 with corner-cutting past (3,3)
    readme = np.array([[1, 0, 1, 1, 1], [1, 0, 1, 1, 1], [1, 0, 1, 1, 1], [1, 1, 1, 0, 1], [1, 1, 1, 0, 1]],
                      dtype=np.uint8)
    cases.append(grid_case("readme5", E.pack_words(readme), 5, 5, (0, 0), (4, 4),
                           {"kind": "custom", "cells": readme.reshape(-1).tolist()}))
    # blocked goal: the reference may enter a blocked cell (it only cannot leave it)
    bg = np.ones((6, 7), dtype=np.uint8)
    bg[5, 6] = 0
    bg[2, 1:6] = 0
    cases.append(grid_case("blocked_goal", E.pack_words(bg), 6, 7, (0, 0), (5, 6),
                           {"kind": "custom", "cells": bg.reshape(-1).tolist()}))
    # start == goal
    one = np.ones((3, 3), dtype=np.uint8)
    cases.append(grid_case("start_is_goal", E.pack_words(one), 3, 3, (1, 1), (1, 1),
                           {"kind": "custom", "cells": one.reshape(-1).tolist()}))
    # single row / column, ragged sizes
    row = np.ones((1, 37), dtype=np.uint8)
    cases.append(grid_case("one_row", E.pack_words(row), 1, 37, (0, 3), (0, 36),
                           {"kind": "custom", "cells": row.reshape(-1).tolist()}))
    for H, W, gap in [(9, 9, 2), (20, 15, 3), (64, 33, 4), (101, 7, 5)]:
        words, s, g = E.gen_zigzag(H, W, gap)
        cases.append(grid_case(f"zigzag_{H}x{W}_g{gap}", words, H, W, s, g,
                               {"kind": "zigzag", "height_gap": gap}))
    for (H, W, rate, seeds) in [(16, 16, 0.3, range(1, 6)), (33, 65, 0.25, range(1, 4)),
                                (64, 64, 0.3, range(1, 6)), (128, 96, 0.2, range(1, 3)),
                                (100, 100, 0.4, range(1, 4)), (256, 256, 0.3, range(1, 4)),
                                (300, 200, 0.1, range(1, 2))]:
        for sd in seeds:
            sp = WL.screened_grid(H, W, rate, sd, exact=True)
            cases.append(grid_case(f"random_{H}x{W}_r{rate}_s{sp.seed}", sp.words(), H, W, sp.start, sp.goal,
                                   {"kind": "random", "rate": rate, "seed": sp.seed}))
    (GOLDEN / "grid_small.json").write_text(json.dumps(cases, indent=0))

    # puzzles: 8-puzzle walks and the survey's probe board; short 15-puzzle walks
    pz = []
    boards = [(3, [8, 1, 3, 4, 0, 2, 7, 6, 5], None, None)]
    for sd in range(20):
        boards.append((3, E.gen_puzzle(sd, 3, 5 + 3 * sd).tolist(), sd, 5 + 3 * sd))
    boards.append((3, [1, 2, 3, 4, 5, 6, 7, 8, 0], None, 0))
    res = ref_puzzle(3, [b[1] for b in boards], "small3")
    for (nn, tiles, sd, walk), r in zip(boards, res):
        pz.append({"n": nn, "tiles": tiles, "seed": sd, "walk": walk, "ref": r})
    (GOLDEN / "puzzle3_small.json").write_text(json.dumps(pz, indent=0))


def part_p15small():
    boards = [(4, E.gen_puzzle(100 + sd, 4, 10 + 2 * sd).tolist(), 100 + sd, 10 + 2 * sd) for sd in range(24)]
    boards.append((4, list(range(1, 16)) + [0], None, 0))
    res = ref_puzzle(4, [b[1] for b in boards], "small4")
    pz = [{"n": nn, "tiles": tiles, "seed": sd, "walk": walk, "ref": r} for (nn, tiles, sd, walk), r in zip(boards, res)]
    (GOLDEN / "puzzle4_small.json").write_text(json.dumps(pz, indent=0))


def part_p24small():
    # 5x5 boards from short random walks: the reference's CPU A* (4 x 6-tile
    # PDB, src/puzzle/CPU-solver.hpp:71-102) solves them in seconds
    boards = [(5, E.gen_puzzle(200 + sd, 5, 8 + 4 * sd).tolist(), 200 + sd, 8 + 4 * sd) for sd in range(16)]
    boards.append((5, list(range(1, 25)) + [0], None, 0))
    res = ref_puzzle_parallel(5, [b[1] for b in boards], "small5", 4)
    pz = [{"n": nn, "tiles": tiles, "seed": sd, "walk": walk, "ref": r} for (nn, tiles, sd, walk), r in zip(boards, res)]
    (GOLDEN / "puzzle5_small.json").write_text(json.dumps(pz, indent=0))


def ref_puzzle(n: int, boards, tag: str):
    inp, outp = WORK / f"{tag}.txt", WORK / f"{tag}.jsonl"
    inp.write_text("".join(" ".join(map(str, b)) + "\n" for b in boards))
    subprocess.run([str(REF / "ref_puzzle"), "solve", str(n), str(PDB_DIR), str(inp), str(outp)], check=True,
                   capture_output=True)
    rows = [json.loads(x) for x in outp.read_text().splitlines() if x.strip()]
    assert len(rows) == len(boards)
    return rows


def ref_puzzle_parallel(n, boards, tag, jobs):
    chunks = [boards[i::jobs] for i in range(jobs)]
    with cf.ThreadPoolExecutor(jobs) as ex:
        outs = list(ex.map(lambda ic: ref_puzzle(n, ic[1], f"{tag}_{ic[0]}") if ic[1] else [],
                           enumerate(chunks)))
    res = [None] * len(boards)
    for i in range(jobs):
        for j, r in enumerate(outs[i]):
            res[i + j * jobs] = r
    return res


def part_c1():
    sp = WL.GRID_1000
    rec = grid_case("grid_1000", sp.words(), sp.H, sp.W, sp.start, sp.goal,
                    {"kind": "random", "rate": sp.rate, "seed": sp.seed})
    (GOLDEN / "grid_c1.json").write_text(json.dumps(rec))


def part_c2():
    sp = WL.GRID_20000
    rec = grid_case("grid_20000", sp.words(), sp.H, sp.W, sp.start, sp.goal,
                    {"kind": "random", "rate": sp.rate, "seed": sp.seed}, keep_path=False)
    (GOLDEN / "grid_c2.json").write_text(json.dumps(rec))


def part_c3(jobs=8):
    specs = WL.puzzle15_x100()
    boards = [s.tiles().tolist() for s in specs]
    res = ref_puzzle_parallel(4, boards, "c3", jobs)
    rows = [{"seed": s.seed, "walk": s.walk, "tiles": b, "ref": {k: r[k] for k in ("solved", "steps", "stored",
                                                                                   "solve_seconds")}}
            for s, b, r in zip(specs, boards, res)]
    (GOLDEN / "puzzle_c3.json").write_text(json.dumps(rows, indent=0))


def part_c4(jobs=8):
    specs = WL.mixed_1024()
    pz = [s for s in specs if isinstance(s, WL.PuzzleSpec)]
    gr = [s for s in specs if isinstance(s, WL.GridSpec)]
    pres = ref_puzzle_parallel(4, [s.tiles().tolist() for s in pz], "c4p", jobs)
    rows = []
    for s, r in zip(pz, pres):
        rows.append({"kind": "puzzle", "seed": s.seed, "walk": s.walk,
                     "ref": {k: r[k] for k in ("solved", "steps", "stored", "solve_seconds")}})

    def one(s):
        rec = grid_case(f"c4_{s.H}_{s.seed}", s.words(), s.H, s.W, s.start, s.goal,
                        {"kind": "random", "rate": s.rate, "seed": s.seed}, keep_path=False)
        rec["kind"] = "grid"
        return rec

    with cf.ThreadPoolExecutor(jobs) as ex:
        rows.extend(ex.map(one, gr))
    (GOLDEN / "mixed_c4.json").write_text(json.dumps(rows, indent=0))


def serve_sample(stream, n_big: int = 64, n_long: int = 64, n_rest: int = 384):
    """Indices of the serving stream's golden sample: its n_big largest grids,
    its n_long longest puzzle walks and n_rest more in a seeded order."""
    grids = sorted((i for i, (_, s) in enumerate(stream) if isinstance(s, WL.GridSpec)),
                   key=lambda i: (-stream[i][1].H, i))[:n_big]
    walks = sorted((i for i, (_, s) in enumerate(stream) if isinstance(s, WL.PuzzleSpec)),
                   key=lambda i: (-stream[i][1].walk, i))[:n_long]
    chosen = set(grids) | set(walks)
    rest = sorted((i for i in range(len(stream)) if i not in chosen), key=lambda i: WL.splitmix64(0xC5C5, i))
    return sorted(chosen | set(rest[:n_rest]))


def ref_puzzle_one(n: int, board, tag: str, timeout_s: float, mem_gb: float):
    """The reference's CPU A* on one board in its own process, bounded in
    time and address space; None when it does not finish within them."""
    import resource

    def limit():
        b = int(mem_gb * (1 << 30))
        resource.setrlimit(resource.RLIMIT_AS, (b, b))

    inp, outp = WORK / f"{tag}.txt", WORK / f"{tag}.jsonl"
    inp.write_text(" ".join(map(str, board)) + "\n")
    try:
        subprocess.run([str(REF / "ref_puzzle"), "solve", str(n), str(PDB_DIR), str(inp), str(outp)], check=True,
                       capture_output=True, timeout=timeout_s, preexec_fn=limit)
        rows = [json.loads(x) for x in outp.read_text().splitlines() if x.strip()]
        return rows[0] if rows and rows[0].get("solved") else None
    except (subprocess.CalledProcessError, subprocess.TimeoutExpired):
        return None
    finally:
        inp.unlink(missing_ok=True)
        outp.unlink(missing_ok=True)


def part_c5(jobs=6, puzzle_jobs=4, timeout_s=900.0, mem_gb=12.0):
    """The serving stream's golden sample.  Each puzzle is solved by the
    reference in its own process within `timeout_s` and `mem_gb`; a board
    that needs more is recorded as skipped (ref.solved false, with the
    reason) and left out of the comparisons."""
    stream = WL.serve_stream(20000, 1.0)
    idx = serve_sample(stream)
    pz = [i for i in idx if isinstance(stream[i][1], WL.PuzzleSpec)]
    gr = [i for i in idx if isinstance(stream[i][1], WL.GridSpec)]
    rows = {}

    def one_puzzle(i):
        s = stream[i][1]
        r = ref_puzzle_one(4, s.tiles().tolist(), f"c5p_{i}", timeout_s, mem_gb)
        ref = ({k: r[k] for k in ("solved", "steps", "stored", "solve_seconds")} if r else
               {"solved": False, "skipped": f"the reference's CPU A* needs more than {timeout_s:.0f} s or "
                                             f"{mem_gb:.0f} GB for this board"})
        return {"index": i, "kind": "puzzle", "seed": s.seed, "walk": s.walk, "ref": ref}

    def one_grid(i):
        s = stream[i][1]
        rec = grid_case(f"c5_{i}", s.words(), s.H, s.W, s.start, s.goal,
                        {"kind": "random", "rate": s.rate, "seed": s.seed}, keep_path=False)
        rec["kind"] = "grid"
        rec["index"] = i
        return rec

    with cf.ThreadPoolExecutor(puzzle_jobs) as ex:
        for rec in ex.map(one_puzzle, pz):
            rows[rec["index"]] = rec
            print("puzzle", rec["index"], rec["ref"].get("steps"), flush=True)
    with cf.ThreadPoolExecutor(jobs) as ex:
        for rec in ex.map(one_grid, gr):
            rows[rec["index"]] = rec
    (GOLDEN / "serve_c5_sample.json").write_text(json.dumps([rows[i] for i in idx], indent=0))


def part_pdb():
    out = {}
    for p in sorted(PDB_DIR.glob("database_*.bin")):
        out[p.name] = {"bytes": p.stat().st_size, "sha256": hashlib.sha256(p.read_bytes()).hexdigest()}
    (GOLDEN / "pdb_sha256.json").write_text(json.dumps(out, indent=1))


PARTS = {"small": part_small, "p15small": part_p15small, "p24small": part_p24small, "c1": part_c1, "c2": part_c2,
         "c3": part_c3, "c4": part_c4, "c5": part_c5, "pdb": part_pdb}

if __name__ == "__main__":
    if not (REF / "ref_grid").exists():
        subprocess.run(["make", "-f", "oracle/Makefile.ref"], cwd=ROOT, check=True)
    for name in sys.argv[1:] or ["small", "c1"]:
        print("part", name, flush=True)
        PARTS[name]()

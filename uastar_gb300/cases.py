"""Run one named workload case on the engine (for profiling and quick checks).

    python -m uastar_gb300.cases grid_1000 [--repeat 2]
    python -m uastar_gb300.cases grid_20000 [--repeat 2] [--dedup 1]
    python -m uastar_gb300.cases puzzle15 [--count 10]
    python -m uastar_gb300.cases mixed_small [--repeat 1]
    python -m uastar_gb300.cases cluster_small [--repeat 1]
    python -m uastar_gb300.cases pdb4 [--repeat 1]
    python -m uastar_gb300.cases sort [--repeat 3]

Each repeat solves the case once and prints one line of results; profilers
capture the second launch of the search kernel (`-s 1 -c 1`).
"""
from __future__ import annotations

import argparse
import time

from . import Engine
from . import workloads as WL


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["grid_1000", "grid_20000", "puzzle15", "mixed_small", "cluster_small", "pdb4",
                                     "sort"])
    ap.add_argument("--repeat", type=int, default=2)
    ap.add_argument("--count", type=int, default=10)
    ap.add_argument("--dedup", type=int, default=0, help="grids: 0 table minimum, 1 per-round sort + unique")
    args = ap.parse_args()

    if args.case in ("grid_1000", "grid_20000"):
        sp = WL.GRID_1000 if args.case == "grid_1000" else WL.GRID_20000
        # fixed tables: one search launch per solve (no in-place growth)
        kw = {"hash_log2_slots": 28 if args.case == "grid_20000" else 22, "dedup": args.dedup}
        words = sp.words()
        with Engine(0, heaps=8192, block_threads=256, threads_per_heap=4, **kw) as eng:
            for _ in range(args.repeat):
                r = eng.grid_solve(words, sp.H, sp.W, sp.start, sp.goal)
                print(f"{args.case}: {r.straight}+{r.diagonal}*sqrt2 cost {r.cost:.4f} expanded {r.expanded} "
                      f"generated {r.generated} rounds {r.rounds} kernel {r.kernel_ms:.1f} ms", flush=True)
    elif args.case == "puzzle15":
        with Engine(0, hash_log2_slots=25) as eng:  # fixed table: one launch per solve
            eng.pdb_build(4)
            for _ in range(args.repeat):
                t0 = time.perf_counter()
                steps = [eng.puzzle_solve(4, s.tiles()).steps for s in WL.puzzle15_x100(count=args.count)]
                print(f"puzzle15: {len(steps)} solves in {time.perf_counter() - t0:.3f} s, steps {steps}", flush=True)
    elif args.case == "sort":
        # the sorted dedup mode's team sort on its own: the largest launch
        # (2048 keys per SM) of 29-bit keys, the 20000^2 grid's cell width
        import numpy as np
        import torch
        n = 2048 * torch.cuda.get_device_properties(0).multi_processor_count
        keys = np.random.default_rng(1).integers(0, 1 << 29, n, dtype=np.uint64).astype(np.uint32)
        with Engine(0) as eng:
            for _ in range(args.repeat):
                t0 = time.perf_counter()
                perm = eng.sort_keys(keys, 29)
                ok = bool((keys[perm][1:] >= keys[perm][:-1]).all())
                print(f"sort: {n} keys, sorted {ok}, {1e3 * (time.perf_counter() - t0):.2f} ms with copies", flush=True)
    elif args.case == "pdb4":
        with Engine(0) as eng:
            for _ in range(args.repeat):
                print(f"pdb4: built in {eng.pdb_build(4):.1f} ms", flush=True)
    elif args.case == "cluster_small":
        # 36 15-puzzles of 120-move walks and 4 grids of 2200^2: a 64-round
        # budget on the single-CTA tier sends most of them to 8-CTA clusters
        specs = [WL.PuzzleSpec(4, 120, 8000 + i) for i in range(36)]
        specs += [WL.screened_grid(2200, 2200, 0.25, 21 + i, exact=True) for i in range(4)]
        insts = [s.instance() for s in specs]
        with Engine(0) as eng:
            eng.pdb_build(4)
            for _ in range(args.repeat):
                res, st = eng.batch_solve(insts, tier1_rounds=64)
                print(f"cluster_small: {sum(r['status'] == 0 for r in res)}/{len(res)} ok, "
                      f"{st['wall_ms']:.1f} ms, waves {st['waves']}", flush=True)
    else:
        specs = [WL.PuzzleSpec(4, 60 + i, 7000 + i) for i in range(48)]
        specs += [WL.screened_grid(256 + 32 * i, 256 + 32 * i, 0.25, 11 + i, exact=True) for i in range(8)]
        insts = [s.instance() for s in specs]
        with Engine(0) as eng:
            eng.pdb_build(4)
            for _ in range(args.repeat):
                res, st = eng.batch_solve(insts)
                print(f"mixed_small: {sum(r['status'] == 0 for r in res)}/{len(res)} ok, "
                      f"{st['wall_ms']:.1f} ms, waves {st['waves']}", flush=True)


if __name__ == "__main__":
    main()

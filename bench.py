"""Benchmark of the GA* engine on one GB300 (or N replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--sections c3,c4,c5,mb,dedup | --headline-only]

Headline (one JSON line on rank 0): expanded nodes/s of the plain engine on
the 20000 x 20000 grid (4e8 cells, 30 % blocked, corner to corner, k = 8192
heaps, 2^28-slot dedup table).  A step = one complete solve of that query
with the bitmap resident in HBM (search + path extraction + host
re-validation).  `e2e` is the same metric through the C-ABI call that takes a
pinned host bitmap (H2D copy, search, path D2H inside the timed region).
The line also carries the 15-puzzle x 100 solves/s (plain engine), the mixed
1024-instance batch solves/s (batched persistent engine) against the plain
engine on the same mix, the serving stream's solves/s with p50/p99
latency, the memory-bounded mode's lengths and lower bounds, and the two
grid dedup modes (table minimum vs per-round sort + unique).  All inputs are seeded synthetic instances (uastar_gb300.workloads).

--impl reference times the reference's CPU A* (the oracle restatement of
src/pathway/CPU-solver.cpp, built from oracle/) on this host's cores: every
core runs the same 20000^2 query, each stopped after a fixed number of
expansions, and the line reports their aggregate expanded nodes/s.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "expanded nodes/s (GA* on the 20000x20000 grid, 30% blocked)"
UNIT = "nodes/s"
WORKLOAD = "grid_20000"
# algorithmic bytes per unit of work (sector-granular, 32 B per random access):
# grid 160 B per expansion + 32 B per generated successor + 64 B per heap push
GRID_BYTES = (160, 32, 64)


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# ----------------------------------------------------------------- our arm
def run_ours(args, rank, world, local_rank):
    import numpy as np
    import torch
    from uastar_gb300 import Engine, replicas, workloads as WL
    from uastar_gb300 import engine as E

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.Stream(device=dev)
    sp = WL.GRID_20000
    words = sp.words()
    pinned = torch.empty(words.size, dtype=torch.int64, pin_memory=True)
    pinned.numpy().view(np.uint64)[:] = words
    host_words = pinned.numpy().view(np.uint64)

    eng = Engine(local_rank, heaps=8192, block_threads=256, threads_per_heap=4, hash_log2_slots=28)
    eng.set_stream(stream.cuda_stream)
    eng.grid_load(words, sp.H, sp.W)

    def solve():
        r = eng.grid_solve_loaded(sp.start, sp.goal)
        assert r.ok, r
        return r

    for _ in range(args.warmup):
        solve()
    ref_pair = None
    c2 = ROOT / "tests" / "golden" / "grid_c2.json"
    if c2.exists():
        ref = json.loads(c2.read_text())["ref"]
        ref_pair = (ref["straight"], ref["diagonal"])

    launches0 = eng.kernel_launches
    results = []
    kernel_ms = []
    replicas.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clocks:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            r = solve()
            results.append(r)
            kernel_ms.append(r.kernel_ms)
        ev1.record(stream)
        torch.cuda.synchronize()
    replicas.barrier()
    launches = eng.kernel_launches - launches0
    elapsed_ms = ev0.elapsed_time(ev1)
    elapsed_ms = replicas.max_over_ranks(elapsed_ms)
    expanded = sum(r.expanded for r in results)
    total_expanded = replicas.sum_over_ranks(expanded)
    value = total_expanded / (elapsed_ms / 1e3)
    r0 = results[-1]
    parity = None
    if ref_pair is not None:
        parity = (r0.straight, r0.diagonal) == ref_pair

    # roofline of the search kernel (one launch per solve)
    peak, peak_kind = measured_peaks()
    per_launch_bytes = [GRID_BYTES[0] * r.expanded + GRID_BYTES[1] * r.generated + GRID_BYTES[2] * r.pushed
                        for r in results]
    mean_kernel_ms = sum(kernel_ms) / len(kernel_ms)
    achieved = (sum(per_launch_bytes) / len(per_launch_bytes)) / (mean_kernel_ms / 1e3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        t = json.loads(tf.read_text()).get(WORKLOAD)
        if t:
            traffic = t.get("dram_bytes_per_launch")

    # e2e: through the host-buffer C-ABI call, H2D + search + path D2H per step
    torch.cuda.synchronize()
    e2e_steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    e2e_exp = 0
    for _ in range(e2e_steps):
        r = eng.grid_solve(host_words, sp.H, sp.W, sp.start, sp.goal)
        assert r.ok
        path = eng.grid_path()
        e2e_exp += r.expanded
    torch.cuda.synchronize()
    e2e_s = replicas.max_over_ranks(time.perf_counter() - t0)
    e2e_value = replicas.sum_over_ranks(e2e_exp) / e2e_s
    d2h = int(path.nbytes) + 104

    line = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(elapsed_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int64", "data": "synthetic (seeded generator)",
        "config": {"workload": WORKLOAD, "grid": "20000x20000", "block_rate": 0.30, "seed": sp.seed,
                   "heaps": 8192, "block_threads": 256, "threads_per_heap": 4, "hash_slots": 2 ** 28,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2: each solve rewrites its 8.6 GB dedup table first",
                   "step": "one full solve (search + path walk + host validation), bitmap resident"},
        "result": {"straight": r0.straight, "diagonal": r0.diagonal, "cost": r0.cost,
                   "expanded": r0.expanded, "generated": r0.generated, "pushed": r0.pushed,
                   "rounds": r0.rounds, "path_len": r0.path_len, "matches_reference": parity},
        "e2e": {"value": round(e2e_value, 1), "unit": UNIT, "h2d_bytes_per_step": int(words.nbytes),
                "d2h_bytes_per_step": d2h, "steps": e2e_steps},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 5), "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": "k_plain_search<GridProblem>", "kernel_ms_mean": round(mean_kernel_ms, 3),
                     "bytes_per_launch": int(sum(per_launch_bytes) / len(per_launch_bytes)),
                     "bytes_model": "160*expanded + 32*generated + 64*pushed"},
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
    }
    return eng, line


def cpu_baseline(args):
    """Oracle (reference-semantics CPU A*) on one host core, bounded sample of the same query."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    from uastar_gb300 import workloads as WL
    sp = WL.GRID_20000
    words = sp.words()
    cap = args.cpu_cap
    t0 = time.perf_counter()
    r, _ = O.grid_astar(words, sp.H, sp.W, sp.start, sp.goal, max_expansions=cap, want_path=False)
    dt = time.perf_counter() - t0
    return {"value": round(r.expanded / r.solve_seconds, 1), "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"reference-semantics CPU A* on the same 20000^2 query, stopped after {r.expanded} "
                      f"expansions ({r.solve_seconds:.1f} s of search, {dt:.1f} s wall incl. setup)"}


# ----------------------------------------------------------- extra sections
def section_c3(eng, args):
    """15-puzzle x 100 (200-move walks), plain engine one at a time."""
    from uastar_gb300 import workloads as WL
    t_pdb = eng.pdb_build(4)
    eng._bench_pdb = True
    specs = WL.puzzle15_x100(count=args.c3_count)
    golden = {}
    gp = ROOT / "tests" / "golden" / "puzzle_c3.json"
    if gp.exists():
        golden = {r["seed"]: r["ref"]["steps"] for r in json.loads(gp.read_text())}
    boards = [s.tiles() for s in specs]
    for b in boards[:3]:
        eng.puzzle_solve(4, b)
    t0 = time.perf_counter()
    res = [eng.puzzle_solve(4, b) for b in boards]
    dt = time.perf_counter() - t0
    agree = [golden[s.seed] == r.steps for s, r in zip(specs, res) if s.seed in golden]
    return {"instances": len(specs), "solves_per_s": round(len(specs) / dt, 2),
            "expanded_per_s": round(sum(r.expanded for r in res) / dt, 1),
            "mean_solve_ms": round(1e3 * dt / len(specs), 3), "pdb_build_ms": round(t_pdb, 1),
            "all_ok": all(r.ok for r in res),
            "optimal_agreement": (f"{sum(agree)}/{len(agree)}" if agree else None)}


def ensure_pdb(eng):
    """The 15-puzzle tables, built once per engine (any section may run first)."""
    if not getattr(eng, "_bench_pdb", False):
        eng.pdb_build(4)
        eng._bench_pdb = True


def section_c4(eng, args):
    """Mixed 1024 (768 puzzles + 256 grids): batched engine vs plain engine."""
    from uastar_gb300 import workloads as WL
    ensure_pdb(eng)
    specs = WL.mixed_1024()
    insts = [s.instance() for s in specs]
    cfg = {}
    if args.autotune:
        cfg = eng.autotune(insts[::16])
    res, st = eng.batch_solve(insts, threads_per_instance=cfg.get("threads_per_instance", 0),
                              heap_capacity=cfg.get("heap_capacity", 0), load_factor=cfg.get("load_factor", 0.0))
    t0 = time.perf_counter()
    res, st = eng.batch_solve(insts, threads_per_instance=cfg.get("threads_per_instance", 0),
                              heap_capacity=cfg.get("heap_capacity", 0), load_factor=cfg.get("load_factor", 0.0))
    dt = time.perf_counter() - t0
    batched = len(insts) / dt
    # plain engine on a sample of the same mix, one instance at a time
    sample = list(range(0, len(specs), max(1, len(specs) // args.plain_sample)))
    t0 = time.perf_counter()
    plain_ok = 0
    for i in sample:
        s, inst = specs[i], insts[i]
        if isinstance(s, WL.PuzzleSpec):
            r = eng.puzzle_solve(4, inst.tiles)
            plain_ok += int(r.ok and r.steps == res[i]["steps"])
        else:
            r = eng.grid_solve(inst.words, s.H, s.W, s.start, s.goal)
            plain_ok += int(r.ok and (r.straight, r.diagonal) == (res[i]["straight"], res[i]["diagonal"]))
    plain = len(sample) / (time.perf_counter() - t0)
    agree = None
    gp = ROOT / "tests" / "golden" / "mixed_c4.json"
    if gp.exists():
        rows = json.loads(gp.read_text())
        ok = 0
        for row, r in zip(rows, res):
            if row["kind"] == "puzzle":
                ok += int(r["steps"] == row["ref"]["steps"])
            else:
                ok += int((r["straight"], r["diagonal"]) == (row["ref"]["straight"], row["ref"]["diagonal"]))
        agree = f"{ok}/{len(rows)}"
    return {"instances": len(insts), "batched_solves_per_s": round(batched, 1),
            "plain_solves_per_s": round(plain, 2), "speedup_vs_plain": round(batched / plain, 2),
            "expanded_per_s": round(st["expanded"] / dt, 1), "waves": st["waves"],
            "threads_per_instance": st["threads_per_instance"], "heap_capacity": st["heap_capacity"],
            "load_factor": st["load_factor"], "all_ok": all(r["status"] == 0 for r in res),
            "plain_agrees": f"{plain_ok}/{len(sample)}", "optimal_agreement": agree}


def section_c5(eng, args):
    """Serving: Poisson stream, admission against a 120 GB budget."""
    from uastar_gb300 import workloads as WL
    ensure_pdb(eng)
    out = []
    for rate in args.serve_rates:
        stream = WL.serve_stream(args.serve_count, rate)
        insts = [s.instance() for _, s in stream]
        eng.serve_start(hbm_budget_gb=120.0)
        t0 = WL.E.now_s() + 0.05
        ids = [eng.serve_submit(inst, t0 + dt) for (dt, _), inst in zip(stream, insts)]
        got = {}
        deadline = time.time() + args.serve_timeout
        while len(got) < len(ids) and time.time() < deadline:
            for rid, r in eng.serve_poll():
                got[rid] = r
            time.sleep(0.001)
        st = eng.serve_stop(10.0)
        lat = sorted(r["latency_ms"] for r in got.values() if r["status"] == 0)
        span = max(stream[-1][0], 1e-9)
        done_t = (max(r["latency_ms"] / 1e3 + stream[i][0] for i, r in enumerate(got[x] for x in ids if x in got))
                  if got else span)
        out.append({"rate_per_s": rate, "requests": len(ids), "completed_ok": len(lat),
                    "solves_per_s": round(len(lat) / max(done_t, 1e-9), 1),
                    "p50_ms": round(lat[len(lat) // 2], 3) if lat else None,
                    "p99_ms": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 3) if lat else None,
                    "quanta": st["quanta"], "peak_resident": st["peak_resident"],
                    "peak_budget_gb": round(st["peak_budget_gb"], 2)})
    # the plain engine, one request at a time, on a sample of the same stream
    # (the request mix does not depend on the rate)
    stream = WL.serve_stream(args.serve_count, 1.0)
    sample = stream[::max(1, len(stream) // args.plain_sample)]
    t0 = time.perf_counter()
    for _, spec in sample:
        if isinstance(spec, WL.PuzzleSpec):
            eng.puzzle_solve(4, spec.tiles())
        else:
            eng.grid_solve(spec.words(), spec.H, spec.W, spec.start, spec.goal)
    plain = len(sample) / (time.perf_counter() - t0)
    for row in out:
        row["plain_solves_per_s"] = round(plain, 2)
        row["speedup_vs_plain"] = round(row["solves_per_s"] / plain, 2)
    return out


def section_mb(eng, args):
    """Memory-bounded mode on the hardest 15-puzzle of the mixed batch (63
    moves, ~7.5e7 states when solved exactly): the returned length next to
    the proven lower bound, for dedup tables capped at 2^20 .. 2^24 slots."""
    from uastar_gb300 import workloads as WL
    from uastar_gb300.engine import gen_puzzle as E_gen_puzzle
    ensure_pdb(eng)
    tiles = WL.mixed_1024()[127].tiles()
    out = []
    for log2 in (20, 22, 24):
        r = eng.puzzle_solve_bounded(4, tiles, log2)
        out.append({"max_table_slots": 1 << log2, "table_mb": (1 << log2) * 32 >> 20, "status": r["status"],
                    "steps": r["steps"], "lower_bound": r["lower_bound"], "segments": r["segments"],
                    "expanded": r["expanded"], "solve_ms": round(r["solve_ms"], 1)})
    opt = eng.puzzle_solve(4, tiles)
    for row in out:
        row["optimal_steps"] = opt.steps
    # a 5x5 board 400 random moves from the goal (beyond exact A* in memory)
    eng.pdb_build(5)
    t5 = E_gen_puzzle(77, 5, 400)
    for log2 in (22, 24):
        r = eng.puzzle_solve_bounded(5, t5, log2)
        out.append({"puzzle": "5x5, 400-move walk", "max_table_slots": 1 << log2, "table_mb": (1 << log2) * 32 >> 20,
                    "status": r["status"], "steps": r["steps"], "lower_bound": r["lower_bound"],
                    "segments": r["segments"], "expanded": r["expanded"], "solve_ms": round(r["solve_ms"], 1)})
    return out


def section_dedup(eng, args):
    """The two ways of removing a round's duplicate grid successors on the
    1000^2 and 20000^2 queries: the dedup table's atomic minimum (default)
    and the reference's order, a device radix sort of the round's successors
    by cell + one relax per cell (dedup = 1)."""
    from uastar_gb300 import Engine, workloads as WL
    out = []
    for name, sp, log2 in (("grid_1000", WL.GRID_1000, 22), ("grid_20000", WL.GRID_20000, 28)):
        words = sp.words()
        for mode in (0, 1):
            with Engine(0, heaps=8192, block_threads=256, threads_per_heap=4, hash_log2_slots=log2,
                        dedup=mode) as e:
                e.grid_load(words, sp.H, sp.W)
                e.grid_solve_loaded(sp.start, sp.goal)  # warm-up
                r = e.grid_solve_loaded(sp.start, sp.goal)
            out.append({"workload": name, "dedup": ["table_min", "sort_unique"][mode], "ok": r.ok,
                        "straight": r.straight, "diagonal": r.diagonal, "kernel_ms": round(r.kernel_ms, 2),
                        "rounds": r.rounds, "us_per_round": round(1e3 * r.kernel_ms / max(1, r.rounds), 2),
                        "expanded": r.expanded, "generated": r.generated,
                        "expanded_per_s": round(r.expanded / (r.kernel_ms / 1e3), 1)})
    return out


# ------------------------------------------------------------ reference arm
def run_reference(args, rank, world):
    if rank != 0:
        return None
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    from concurrent.futures import ThreadPoolExecutor
    from uastar_gb300 import workloads as WL
    sp = WL.GRID_20000
    words = sp.words()
    cores = os.cpu_count() or 1
    cap = args.ref_cap

    def one(_):
        r, _p = O.grid_astar(words, sp.H, sp.W, sp.start, sp.goal, max_expansions=cap, want_path=False)
        return r.expanded

    with ThreadPoolExecutor(cores) as ex:
        for _ in range(args.warmup):
            list(ex.map(one, range(cores)))
        t0 = time.perf_counter()
        total = 0
        for _ in range(args.steps):
            total += sum(ex.map(one, range(cores)))
        dt = time.perf_counter() - t0
    value = total / dt
    sample = (f"{cores} threads, each the same 20000^2 query stopped after {cap} expansions "
              f"(reference-semantics CPU A*, oracle restatement of src/pathway/CPU-solver.cpp)")
    return {"impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * dt / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator)", "config": {"workload": WORKLOAD, "grid": "20000x20000",
                                                               "block_rate": 0.30, "seed": sp.seed},
            "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--headline-only", action="store_true")
    ap.add_argument("--sections", default="c3,c4,c5,mb,dedup")
    ap.add_argument("--cpu-cap", type=int, default=12_000_000)
    ap.add_argument("--ref-cap", type=int, default=3_000_000)
    ap.add_argument("--c3-count", type=int, default=100)
    ap.add_argument("--plain-sample", type=int, default=64)
    ap.add_argument("--serve-count", type=int, default=1000)
    ap.add_argument("--serve-rates", type=lambda s: [float(x) for x in s.split(",")], default=[50.0, 200.0, 1000.0])
    ap.add_argument("--serve-timeout", type=float, default=120.0)
    ap.add_argument("--autotune", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    from uastar_gb300 import replicas
    rank, world, local_rank = replicas.dist_env()
    if world > 1:
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        if backend == "nccl":
            import torch
            torch.cuda.set_device(local_rank)
        dist.init_process_group(backend)

    if args.impl == "reference":
        line = run_reference(args, rank, world)
        if rank == 0:
            print(json.dumps(line), flush=True)
        return

    eng, line = run_ours(args, rank, world, local_rank)
    if rank == 0:
        line["cpu_baseline"] = cpu_baseline(args)
        # The single-GPU sections run at N = 1 only: a replica run measures
        # the headline, without holding N GPUs for minutes more.
        if not args.headline_only and world == 1:
            # The other workloads run on an engine with the default (automatic)
            # configuration, which is what a caller of the plain, batched and
            # serving entry points gets; the headline engine's fixed 2^28-slot
            # table and 8192 heaps belong to the 20000^2 query only.
            from uastar_gb300 import Engine
            with Engine(local_rank) as deng:
                secs = [s for s in args.sections.split(",") if s]
                for name, fn in [("c3", section_c3), ("c4", section_c4), ("c5", section_c5), ("mb", section_mb),
                                 ("dedup", section_dedup)]:
                    if name in secs:
                        t0 = time.perf_counter()
                        try:
                            key = {"c3": "puzzle15_x100", "c4": "mixed_1024_batched", "c5": "serving",
                                   "mb": "memory_bounded_puzzle", "dedup": "dedup_modes"}[name]
                            line[key] = fn(deng, args)
                        except Exception as exc:  # report, keep the headline
                            line[f"{name}_error"] = repr(exc)
                        log(f"section {name}: {time.perf_counter() - t0:.1f} s")
        print(json.dumps(line), flush=True)
    eng.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

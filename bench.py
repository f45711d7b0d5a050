"""Benchmark of the GA* engine on one GB300 (or N replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--sections c3,c4,c5,mb,dedup | --headline-only]
    python bench.py --case NAME [--repeat R]      (one workload, for profilers)

Headline (one JSON line on rank 0): expanded nodes/s of the plain engine on
the 20000 x 20000 grid (4e8 cells, 30 % blocked, corner to corner, k = 8192
heaps, 2^28-slot dedup table).  A step = one complete solve of that query
with the bitmap resident in HBM (search + path extraction + host
re-validation), so `s_per_solve` is the step time.  `e2e` is the same metric
through the C-ABI call that takes a pinned host bitmap (H2D copy, search,
path D2H inside the timed region).  `latency_model` splits the search into
rounds x microseconds per round next to the bare cost of a team barrier.

The line also carries, each with its own CPU baseline (the oracle, a CPU
restatement of the reference's A*, timed on this host's cores in this run):
  puzzle15_x100       15-puzzle x 100 (200-move walks), plain engine, solves/s
  mixed_1024_batched  768 puzzles + 256 grids, batched persistent engine with
                      the configuration the autotuner picks, against the plain
                      engine on the same mix
  serving             the Poisson stream of 20000 requests at the top rate
                      (and shorter streams at lower rates), p50/p99 latency,
                      every served result compared with the plain engine (as
                      far as the time guard allows) and a 512-request sample
                      with the reference's own results
  memory_bounded_puzzle, dedup_modes
All inputs are seeded synthetic instances (uastar_gb300.workloads).

--impl reference times the reference's CPU A* (the oracle restatement of
src/pathway/CPU-solver.cpp, built from oracle/) on this host's cores: every
core runs the same 20000^2 query, each stopped after a fixed number of
expansions, and the line reports their aggregate expanded nodes/s; one full
solve on one core gives its seconds per solve.  That arm loads no engine code.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"

METRIC = "expanded nodes/s (GA* on the 20000x20000 grid, 30% blocked)"
UNIT = "nodes/s"
WORKLOAD = "grid_20000"
# The 20000^2 query (the seed was screened by the reference's CPU solver; the
# fixture records it).  The reference arm builds it with the oracle's own
# generator, the engine arm with the engine's: the same bits.
C2_H = C2_W = 20000
C2_RATE, C2_SEED = 0.30, 7
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


def golden(name: str):
    p = GOLDEN / name
    return json.loads(p.read_text()) if p.exists() else None


def cpu_info() -> dict:
    """Host core count and CPU model (lscpu, else /proc/cpuinfo)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        try:
            for line in open("/proc/cpuinfo"):
                if line.lower().startswith(("model name", "cpu part")):
                    model = line.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    return {"nproc": os.cpu_count() or 1, "model": model or "unknown", "machine": platform.machine()}


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


# --------------------------------------------------------- CPU baselines
def oracle_module():
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    return O


def cpu_stream_sample(jobs, cores: int, budget_s: float) -> dict:
    """Independent oracle solves on `cores` threads (the oracle's C calls
    release the GIL, so each thread is one core's solver).  `jobs` are
    callables returning (solved, expansions); they are started in order
    until `budget_s` has passed, and every started one runs to its end (each
    is bounded by its own expansion cap)."""
    from concurrent.futures import FIRST_COMPLETED, ThreadPoolExecutor, wait
    jobs = list(jobs)
    t0 = time.perf_counter()
    started = solved = capped = 0
    nodes = 0
    with ThreadPoolExecutor(cores) as ex:
        live = set()
        while started < len(jobs) and len(live) < cores:
            live.add(ex.submit(jobs[started]))
            started += 1
        while live:
            done, live = wait(live, return_when=FIRST_COMPLETED)
            for f in done:
                ok, n = f.result()
                solved += int(ok)
                capped += int(not ok)
                nodes += n
            while started < len(jobs) and len(live) < cores and time.perf_counter() - t0 < budget_s:
                live.add(ex.submit(jobs[started]))
                started += 1
    wall = time.perf_counter() - t0
    return {"started": started, "solved": solved, "capped": capped, "wall_s": round(wall, 2),
            "solves_per_s": round(solved / wall, 3), "nodes_per_s": round(nodes / wall, 1)}


def oracle_job(O, spec, tables, cap: int):
    """One oracle solve of a workload spec: (solved, expansions)."""
    from uastar_gb300 import workloads as WL
    if isinstance(spec, WL.PuzzleSpec):
        def run():
            r, _ = O.puzzle_astar(4, spec.tiles(), tables, max_expansions=cap)
            return bool(r.solved), int(r.expanded)
    else:
        def run():
            r, _ = O.grid_astar(spec.words(), spec.H, spec.W, spec.start, spec.goal, max_expansions=cap,
                                want_path=False)
            return bool(r.solved), int(r.expanded)
    return run


def pdb_tables_for_oracle(eng):
    """The 15-puzzle tables as the oracle takes them (one array per pattern),
    copied back from the GPU (byte-equal to the reference's files, checked by
    the tests); the oracle's own generator would take ~20 minutes."""
    if getattr(eng, "_bench_tables", None) is None:
        ensure_pdb(eng)
        t = eng.pdb_fetch(4)
        eng._bench_tables = [t[:518918400], t[518918400:]]
    return eng._bench_tables


def cpu_baseline_stream(eng, specs, cores: int, budget_s: float, cap: int, what: str) -> dict:
    O = oracle_module()
    tables = pdb_tables_for_oracle(eng)
    res = cpu_stream_sample([oracle_job(O, s, tables, cap) for s in specs], cores, budget_s)
    info = cpu_info()
    return {"value": res["solves_per_s"], "unit": "solves/s", "cores": cores, "kind": "port",
            "cpu": info["model"], "nproc": info["nproc"], **res,
            "sample": f"{what}: instances started in order on {cores} threads (one independent oracle solve "
                      f"each, reference-semantics CPU A*) until {budget_s:.0f} s had passed, each stopped "
                      f"after {cap} expansions (stopped = not solved)"}


# ----------------------------------------------------------------- our arm
def run_ours(args, rank, world, local_rank):
    import numpy as np
    import torch
    from uastar_gb300 import Engine, replicas, workloads as WL

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
    c2 = golden("grid_c2.json")
    ref_pair = (c2["ref"]["straight"], c2["ref"]["diagonal"]) if c2 else None

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

    # latency model: rounds x us per round, next to a bare team barrier on the
    # same launch geometry
    rounds = sum(r.rounds for r in results) / len(results)
    barrier_us, cas_barrier_us = eng.round_floor(2000)
    latency = {"rounds": int(rounds), "path_cells": int(r0.path_len),
               "rounds_per_path_cell": round(rounds / max(1, r0.path_len), 3),
               "us_per_round": round(1e3 * mean_kernel_ms / max(1.0, rounds), 3),
               "floor_barrier_us": round(barrier_us, 3), "floor_cas_barrier_us": round(cas_barrier_us, 3),
               "note": "a round is at least one team barrier plus its chain of dependent memory accesses "
                       "(floor_cas_barrier_us: one dependent table CAS per thread and the barrier, "
                       "uastar_round_floor); rounds are bounded below by the path length"}

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
        "s_per_solve": round(elapsed_ms / args.steps / 1e3, 4),
        "config": {"workload": WORKLOAD, "grid": "20000x20000", "block_rate": 0.30, "seed": sp.seed,
                   "heaps": 8192, "block_threads": 256, "threads_per_heap": 4, "hash_slots": 2 ** 28,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2: each solve rewrites its 8.6 GB dedup table first",
                   "step": "one full solve (search + path walk + host validation), bitmap resident"},
        "result": {"straight": r0.straight, "diagonal": r0.diagonal, "cost": r0.cost,
                   "expanded": r0.expanded, "generated": r0.generated, "pushed": r0.pushed,
                   "rounds": r0.rounds, "path_len": r0.path_len, "matches_reference": parity,
                   "reference_astar": ({"generated": c2["ref"].get("generated"),
                                        "expanded": c2["ref"].get("expanded"),
                                        "note": "sequential A* of the reference's CPU solver on the same "
                                                "query (fixture)"} if c2 else None)},
        "latency_model": latency,
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
    O = oracle_module()
    from uastar_gb300 import workloads as WL
    sp = WL.GRID_20000
    words = sp.words()
    cap = args.cpu_cap
    t0 = time.perf_counter()
    r, _ = O.grid_astar(words, sp.H, sp.W, sp.start, sp.goal, max_expansions=cap, want_path=False)
    dt = time.perf_counter() - t0
    return {"value": round(r.expanded / r.solve_seconds, 1), "unit": UNIT, "cores": 1, "kind": "port",
            "cpu": cpu_info()["model"],
            "sample": f"reference-semantics CPU A* on the same 20000^2 query, stopped after {r.expanded} "
                      f"expansions ({r.solve_seconds:.1f} s of search, {dt:.1f} s wall incl. setup)"}


# ----------------------------------------------------------- extra sections
def ensure_pdb(eng):
    """The 15-puzzle tables, built once per engine (any section may run first)."""
    if not getattr(eng, "_bench_pdb_ms", None):
        eng._bench_pdb_ms = eng.pdb_build(4)
    return eng._bench_pdb_ms


def section_c3(eng, args):
    """15-puzzle x 100 (200-move walks), plain engine one at a time."""
    from uastar_gb300 import workloads as WL
    t_pdb = ensure_pdb(eng)
    specs = WL.puzzle15_x100(count=args.c3_count)
    rows = golden("puzzle_c3.json") or []
    gold = {r["seed"]: r["ref"]["steps"] for r in rows}
    boards = [s.tiles() for s in specs]
    for b in boards[:3]:
        eng.puzzle_solve(4, b)
    t0 = time.perf_counter()
    res = [eng.puzzle_solve(4, b) for b in boards]
    dt = time.perf_counter() - t0
    agree = [gold[s.seed] == r.steps for s, r in zip(specs, res) if s.seed in gold]
    out = {"instances": len(specs), "solves_per_s": round(len(specs) / dt, 2),
           "expanded_per_s": round(sum(r.expanded for r in res) / dt, 1),
           "mean_solve_ms": round(1e3 * dt / len(specs), 3), "pdb_build_ms": round(t_pdb, 1),
           "all_ok": all(r.ok for r in res),
           "optimal_agreement": (f"{sum(agree)}/{len(agree)}" if agree else None)}
    if args.cpu_sections:
        out["cpu_baseline"] = cpu_baseline_stream(eng, specs, 1, args.cpu_budget, args.cpu_solve_cap,
                                                  "the 100 boards of this section in order")
        out["speedup_vs_cpu"] = round(out["solves_per_s"] / max(1e-9, out["cpu_baseline"]["value"]), 1)
    return out


def section_c4(eng, args):
    """Mixed 1024 (768 puzzles + 256 grids): batched engine, with the
    configuration the autotuner picks on a sample of the mix, vs the plain
    engine on the same mix."""
    from uastar_gb300 import workloads as WL
    ensure_pdb(eng)
    specs = WL.mixed_1024()
    insts = [s.instance() for s in specs]
    cfg, tune = {}, None
    if not args.no_autotune:
        t0 = time.perf_counter()
        cfg = eng.autotune(insts[::args.tune_stride])
        tune = {"sample": f"every {args.tune_stride}th instance ({len(insts[::args.tune_stride])})",
                "seconds": round(time.perf_counter() - t0, 2), "configs_timed": cfg.get("tried"),
                "chosen": {k: cfg[k] for k in ("threads_per_instance", "threads_per_heap", "heap_capacity",
                                               "load_factor", "cluster_size", "tier1_rounds",
                                               "tier2_puzzle_rounds")}}
    kw = {k: cfg.get(k, 0) for k in ("threads_per_instance", "threads_per_heap", "heap_capacity", "load_factor",
                                     "cluster_size", "tier1_rounds", "tier2_puzzle_rounds")}
    res, st = eng.batch_solve(insts, **kw)  # warm-up (allocations, graph)
    t0 = time.perf_counter()
    res, st = eng.batch_solve(insts, **kw)
    dt = time.perf_counter() - t0
    batched = len(insts) / dt
    # plain engine on a sample of the same mix, one instance at a time
    sample = list(range(0, len(specs), max(1, len(specs) // args.plain_sample)))
    t0 = time.perf_counter()
    plain_ok = plain_exp = 0
    for i in sample:
        s, inst = specs[i], insts[i]
        if isinstance(s, WL.PuzzleSpec):
            r = eng.puzzle_solve(4, inst.tiles)
            plain_ok += int(r.ok and r.steps == res[i]["steps"])
        else:
            r = eng.grid_solve(inst.words, s.H, s.W, s.start, s.goal)
            plain_ok += int(r.ok and (r.straight, r.diagonal) == (res[i]["straight"], res[i]["diagonal"]))
        plain_exp += r.expanded
    plain_s = time.perf_counter() - t0
    plain = len(sample) / plain_s
    agree = None
    rows = golden("mixed_c4.json")
    if rows:
        ok = 0
        for row, r in zip(rows, res):
            if row["kind"] == "puzzle":
                ok += int(r["status"] == 0 and r["steps"] == row["ref"]["steps"])
            else:
                ok += int(r["status"] == 0 and (r["straight"], r["diagonal"]) ==
                          (row["ref"]["straight"], row["ref"]["diagonal"]))
        agree = f"{ok}/{len(rows)}"
    out = {"instances": len(insts), "batched_solves_per_s": round(batched, 1), "s_per_batch": round(dt, 3),
           "plain_solves_per_s": round(plain, 2), "speedup_vs_plain": round(batched / plain, 2),
           "expanded_per_s": round(st["expanded"] / dt, 1), "waves": st["waves"], "escalated": st["escalated"],
           "threads_per_instance": st["threads_per_instance"], "heap_capacity": st["heap_capacity"],
           "load_factor": st["load_factor"], "autotune": tune, "all_ok": all(r["status"] == 0 for r in res),
           "plain_sample": f"{len(sample)} instances (every {len(specs) // len(sample)}th)",
           "plain_agrees": f"{plain_ok}/{len(sample)}", "optimal_agreement": agree,
           # the ratio = (aggregate expansion rate ratio) x (expansions per solve, plain / batched)
           "plain_expanded_per_s": round(plain_exp / plain_s, 1),
           "expansions_per_solve": {"batched": round(st["expanded"] / len(insts)),
                                    "batched_on_plain_sample": round(sum(res[i]["expanded"] for i in sample)
                                                                     / len(sample)),
                                    "plain_on_plain_sample": round(plain_exp / len(sample))}}
    if args.cpu_sections:
        order = seeded_order(len(specs), 0xC4)
        out["cpu_baseline"] = cpu_baseline_stream(eng, [specs[i] for i in order], os.cpu_count() or 1,
                                                  args.cpu_budget, args.cpu_solve_cap,
                                                  "the 1024-instance mix in a seeded random order")
        out["speedup_vs_cpu"] = round(batched / max(1e-9, out["cpu_baseline"]["value"]), 1)
    return out


def seeded_order(n: int, seed: int) -> list[int]:
    from uastar_gb300 import workloads as WL
    return sorted(range(n), key=lambda i: WL.splitmix64(seed, i))


def serve_golden():
    """Reference results of the serving stream's sample: {stream index: row}."""
    rows = golden("serve_c5_sample.json")
    return {r["index"]: r for r in rows if r["ref"].get("solved")} if rows else {}


def same_result(spec, r, ref) -> bool:
    from uastar_gb300 import workloads as WL
    if r is None or r.get("status") != 0:
        return False
    if isinstance(spec, WL.PuzzleSpec):
        return r["steps"] == ref["steps"]
    return (r["straight"], r["diagonal"]) == (ref["straight"], ref["diagonal"])


def serve_run(eng, stream, rate: float, args) -> tuple[dict, dict]:
    """Serve `stream` ((offset at rate 1, spec) pairs) with arrivals at `rate`:
    requests are generated on a thread pool and submitted ahead of their
    arrival times; returns (row, {index: result})."""
    from concurrent.futures import ThreadPoolExecutor
    from uastar_gb300 import workloads as WL
    eng.serve_start(hbm_budget_gb=120.0)
    t0 = WL.E.now_s() + 0.5
    ids = {}
    with ThreadPoolExecutor(max(1, (os.cpu_count() or 2) - 1)) as ex:
        for i, inst in enumerate(ex.map(lambda x: x[1].instance(), stream)):
            ids[eng.serve_submit(inst, t0 + stream[i][0] / rate)] = i
    got = {}
    deadline = time.time() + args.serve_timeout
    while len(got) < len(ids) and time.time() < deadline:
        for rid, r in eng.serve_poll():
            got[ids[rid]] = r
        time.sleep(0.002)
    st = eng.serve_stop(10.0)
    for rid, r in eng.serve_poll():
        got[ids[rid]] = r
    lat = sorted(r["latency_ms"] for r in got.values() if r["status"] == 0)
    done_t = max((r["latency_ms"] / 1e3 + stream[i][0] / rate for i, r in got.items()), default=1e-9)
    row = {"rate_per_s": rate, "requests": len(ids), "completed_ok": len(lat),
           "solves_per_s": round(len(lat) / max(done_t, 1e-9), 1), "s_to_last": round(done_t, 2),
           "p50_ms": round(lat[len(lat) // 2], 3) if lat else None,
           "p99_ms": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 3) if lat else None,
           "quanta": st["quanta"], "peak_resident": st["peak_resident"],
           "peak_budget_gb": round(st["peak_budget_gb"], 2),
           "migrations": sum(r.get("migrations", 0) for r in got.values()),
           "expanded_per_s": round(sum(r["expanded"] for r in got.values() if r["status"] == 0)
                                   / max(done_t, 1e-9), 1)}
    return row, got


def section_c5(eng, args):
    """Serving: Poisson stream, admission against a 120 GB budget.  The
    20000-request stream runs at the top rate; lower rates run the first
    `serve_extra_count` requests of the same stream."""
    from uastar_gb300 import workloads as WL
    ensure_pdb(eng)
    t_gen = time.perf_counter()
    stream = WL.serve_stream(args.serve_count, 1.0)
    t_gen = time.perf_counter() - t_gen
    out = {"stream": f"{len(stream)} requests, 50 % 15-puzzle (walk 60..300), 50 % grid (side 256..8192, "
                     f"block rate 10..40 %); 120 GB admission budget", "generate_s": round(t_gen, 1), "rates": []}
    served = None
    for rate in sorted(args.serve_rates, reverse=True):
        part = stream if rate == max(args.serve_rates) else stream[:args.serve_extra_count]
        row, got = serve_run(eng, part, rate, args)
        out["rates"].append(row)
        if served is None:
            served = got
    # the reference's own results on the seeded sample (reference CPU A*)
    gold = serve_golden()
    if gold:
        ok = sum(int(same_result(stream[i][1], served.get(i), g["ref"])) for i, g in gold.items()
                 if i < len(stream))
        out["optimal_agreement"] = f"{ok}/{sum(1 for i in gold if i < len(stream))}"
        out["optimal_sample"] = "seeded sample of the stream with its 64 largest grids and 64 longest walks"
    # every served result against the batched engine on the same requests
    # (another scheduling of the same search kernels), in chunks
    t0 = time.perf_counter()
    agree_b = 0
    for c0 in range(0, len(stream), args.check_chunk):
        part = stream[c0:c0 + args.check_chunk]
        insts = WL.parallel_map(lambda x: x[1].instance(), part)
        res, _ = eng.batch_solve(insts)
        agree_b += sum(int(same_result(spec, served.get(c0 + k), r)) for k, ((_, spec), r) in enumerate(zip(part, res))
                       if r["status"] == 0)
        del insts
    out["batched_compared"] = f"{agree_b}/{len(stream)} served results equal the batched engine's " \
                              f"({time.perf_counter() - t0:.0f} s)"
    # the plain engine, one request at a time, in stream order, under a time guard
    t0 = time.perf_counter()
    n = agree = exp = 0
    for i, (_, spec) in enumerate(stream):
        if time.perf_counter() - t0 > args.plain_budget:
            break
        if isinstance(spec, WL.PuzzleSpec):
            r = eng.puzzle_solve(4, spec.tiles())
            ref = {"steps": r.steps}
        else:
            r = eng.grid_solve(spec.words(), spec.H, spec.W, spec.start, spec.goal)
            ref = {"straight": r.straight, "diagonal": r.diagonal}
        n += 1
        exp += r.expanded
        agree += int(r.ok and same_result(spec, served.get(i), ref))
    plain_s = time.perf_counter() - t0
    plain = n / plain_s
    out["plain_solves_per_s"] = round(plain, 2)
    # the ratio = (aggregate expansion rate ratio) x (expansions per solve, plain / served)
    out["plain_expanded_per_s"] = round(exp / plain_s, 1)
    out["expansions_per_solve"] = {
        "plain": round(exp / max(n, 1)),
        "served_same_requests": round(sum(served[i]["expanded"] for i in range(n) if i in served) / max(n, 1))}
    out["plain_compared"] = f"{agree}/{n} of {len(stream)} served results equal the plain engine's " \
                            f"(stream order, {plain_s:.0f} s time guard {args.plain_budget:.0f} s)"
    for row in out["rates"]:
        row["speedup_vs_plain"] = round(row["solves_per_s"] / plain, 2)
    if args.cpu_sections:
        order = seeded_order(len(stream), 0xC5)
        out["cpu_baseline"] = cpu_baseline_stream(eng, [stream[i][1] for i in order], os.cpu_count() or 1,
                                                  args.cpu_budget, args.cpu_solve_cap,
                                                  "the serving stream's requests in a seeded random order")
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
    exact = lambda r: {"exact_passes": r["exact_passes"], "exact_optimal": bool(r["exact_optimal"]),
                       "exact_nodes": r["exact_nodes"], "exact_ms": round(r["exact_ms"], 1)}
    for log2 in (20, 22, 24):
        r = eng.puzzle_solve_bounded(4, tiles, log2)
        out.append({"max_table_slots": 1 << log2, "table_mb": (1 << log2) * 32 >> 20, "status": r["status"],
                    "steps": r["steps"], "lower_bound": r["lower_bound"], "segments": r["segments"],
                    "expanded": r["expanded"], "solve_ms": round(r["solve_ms"], 1), **exact(r)})
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
                    "segments": r["segments"], "expanded": r["expanded"], "solve_ms": round(r["solve_ms"], 1),
                    **exact(r)})
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
    """The reference's CPU A* (oracle restatement) on every host core; loads
    only the oracle library."""
    if rank != 0:
        return None
    import numpy as np
    O = oracle_module()
    from concurrent.futures import ThreadPoolExecutor
    words = O.gen_grid(C2_SEED, C2_H, C2_W, C2_RATE, (0, 0), (C2_H - 1, C2_W - 1))
    start, goal = (0, 0), (C2_H - 1, C2_W - 1)
    c2 = golden("grid_c2.json")
    if c2:
        import hashlib
        assert hashlib.sha256(np.asarray(words, dtype="<u8").tobytes()).hexdigest() == c2["words_sha256"]
    cores = os.cpu_count() or 1
    cap = args.ref_cap

    def one(_):
        r, _p = O.grid_astar(words, C2_H, C2_W, start, goal, max_expansions=cap, want_path=False)
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
    # one full solve on one core: the reference's seconds per solve
    full = None
    if args.ref_full_solve:
        r, _p = O.grid_astar(words, C2_H, C2_W, start, goal, want_path=False)
        full = {"s_per_solve": round(r.solve_seconds, 2), "expanded": int(r.expanded),
                "generated": int(r.generated), "straight": int(r.straight), "diagonal": int(r.diagonal),
                "cost": r.cost, "cores": 1}
    info = cpu_info()
    sample = (f"{cores} threads, each the same 20000^2 query stopped after {cap} expansions "
              f"(reference-semantics CPU A*, oracle restatement of src/pathway/CPU-solver.cpp)")
    return {"impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * dt / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator)",
            "s_per_solve": full["s_per_solve"] if full else None, "full_solve": full,
            "config": {"workload": WORKLOAD, "grid": "20000x20000", "block_rate": C2_RATE, "seed": C2_SEED},
            "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": cores, "kind": "port",
                             "cpu": info["model"], "sample": sample},
            "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# -------------------------------------------------------------------- cases
CASES = ["grid_1000", "grid_20000", "grid_4096", "puzzle15", "mixed_small", "cluster_small", "pdb4", "sort",
         "grow", "migrate", "bounded", "walk", "noalloc"]


def run_case(args) -> None:
    """One named workload, for profilers: each repeat solves it once and
    prints a line; captures take the second launch of the kernel of interest
    (`-s 1 -c 1`).  Every case holds a few GB on the device at most, except
    grid_20000 (the headline query, 8.6 GB table: launch lists only)."""
    import numpy as np
    from uastar_gb300 import Engine, workloads as WL
    c = args.case
    if c in ("grid_1000", "grid_20000", "grid_4096"):
        sp = {"grid_1000": WL.GRID_1000, "grid_20000": WL.GRID_20000,
              "grid_4096": WL.screened_grid(4096, 4096, 0.30, 7)}[c]
        log2 = {"grid_1000": 22, "grid_20000": 28, "grid_4096": 25}[c]
        words = sp.words()
        # fixed tables: one search launch per solve (no in-place growth)
        with Engine(0, heaps=8192, block_threads=256, threads_per_heap=4, hash_log2_slots=log2,
                    dedup=args.dedup) as eng:
            for _ in range(args.repeat):
                r = eng.grid_solve(words, sp.H, sp.W, sp.start, sp.goal)
                print(f"{c}: {r.straight}+{r.diagonal}*sqrt2 cost {r.cost:.4f} expanded {r.expanded} "
                      f"generated {r.generated} rounds {r.rounds} kernel {r.kernel_ms:.1f} ms", flush=True)
    elif c == "puzzle15":
        with Engine(0, hash_log2_slots=25) as eng:  # fixed table: one launch per solve
            eng.pdb_build(4)
            for _ in range(args.repeat):
                t0 = time.perf_counter()
                steps = [eng.puzzle_solve(4, s.tiles()).steps for s in WL.puzzle15_x100(count=args.count)]
                print(f"puzzle15: {len(steps)} solves in {time.perf_counter() - t0:.3f} s, steps {steps}", flush=True)
    elif c == "sort":
        # the sorted dedup mode's team sort on its own: the largest launch
        # (2048 keys per SM) of 29-bit keys, the 20000^2 grid's cell width
        import torch
        n = 2048 * torch.cuda.get_device_properties(0).multi_processor_count
        keys = np.random.default_rng(1).integers(0, 1 << 29, n, dtype=np.uint64).astype(np.uint32)
        with Engine(0) as eng:
            for _ in range(args.repeat):
                t0 = time.perf_counter()
                perm = eng.sort_keys(keys, 29)
                ok = bool((keys[perm][1:] >= keys[perm][:-1]).all())
                print(f"sort: {n} keys, sorted {ok}, {1e3 * (time.perf_counter() - t0):.2f} ms with copies", flush=True)
    elif c == "pdb4":
        with Engine(0) as eng:
            for _ in range(args.repeat):
                print(f"pdb4: built in {eng.pdb_build(4):.1f} ms", flush=True)
    elif c == "grow":
        # an auto-sized dedup table that starts at 2^22 slots and grows in
        # place (k_grow_move / k_grow_links / k_grow_heaps) when half full:
        # a 15-puzzle whose search stores ~4 M states (200-move walk, seed 1039)
        with Engine(0) as eng:
            eng.pdb_build(4)
            tiles = WL.PuzzleSpec(4, 200, 1039).tiles()
            for _ in range(args.repeat):
                r = eng.puzzle_solve(4, tiles)
                print(f"grow: {r.steps} moves, {r.table_grows} table growths, {r.table_used} slots in use, "
                      f"kernel {r.kernel_ms:.1f} ms", flush=True)
    elif c == "migrate":
        # serving requests whose frontier outgrows one CTA move to cluster
        # slots with their search state (k_migrate_heaps)
        specs = [WL.screened_grid(3000, 3000, 0.15, 40 + i, exact=True) for i in range(6)]
        specs += [WL.PuzzleSpec(4, 90, 9100 + i) for i in range(24)]
        with Engine(0) as eng:
            eng.pdb_build(4)
            for _ in range(args.repeat):
                eng.serve_start(hbm_budget_gb=4.0)
                for s in specs:
                    eng.serve_submit(s.instance())
                res, t0 = [], time.time()
                while len(res) < len(specs) and time.time() - t0 < 120:
                    res += eng.serve_poll()
                    time.sleep(0.002)
                st = eng.serve_stop(10.0)
                print(f"migrate: {sum(r['status'] == 0 for _, r in res)}/{len(res)} ok, "
                      f"{sum(r['migrations'] for _, r in res)} migrations, {st['quanta']} quanta", flush=True)
    elif c == "bounded":
        # memory-bounded mode (k_best_open between segments)
        with Engine(0) as eng:
            eng.pdb_build(4)
            tiles = WL.mixed_1024()[127].tiles()
            for _ in range(args.repeat):
                r = eng.puzzle_solve_bounded(4, tiles, 20)
                print(f"bounded: {r['steps']} moves, bound {r['lower_bound']}, {r['segments']} segments", flush=True)
    elif c == "walk":
        # path walks after solves: k_walk on a 4096^2 grid, the in-kernel
        # walk of a batch
        sp = WL.screened_grid(4096, 4096, 0.30, 7)
        words = sp.words()
        grids = [WL.screened_grid(1024, 1024, 0.25, 60 + i, exact=True).instance() for i in range(16)]
        with Engine(0, heaps=8192, block_threads=256, threads_per_heap=4, hash_log2_slots=25) as eng:
            for _ in range(args.repeat):
                r = eng.grid_solve(words, sp.H, sp.W, sp.start, sp.goal)
                res, _st = eng.batch_solve(grids)
                print(f"walk: path {r.path_len} cells; batch {sum(x['status'] == 0 for x in res)}/{len(res)} ok",
                      flush=True)
    elif c == "noalloc":
        # the allocation-free entry point on a 1024^2 grid
        import torch
        from uastar_gb300 import _lib as L
        import ctypes as C
        sp = WL.screened_grid(1024, 1024, 0.30, 3, exact=True)
        words = torch.from_numpy(sp.words().view(np.int64)).cuda()
        path = torch.zeros(1 << 20, dtype=torch.int32, device="cuda")
        res = torch.zeros(64, dtype=torch.uint8, device="cuda")
        lib = L.load()
        for _ in range(args.repeat):
            rc = lib.uastar_grid_solve_noalloc(C.c_void_p(words.data_ptr()), sp.H, sp.W, 0, 0, sp.H - 1,
                                               sp.W - 1, C.c_void_p(path.data_ptr()), path.numel(),
                                               C.c_void_p(res.data_ptr()), None)
            torch.cuda.synchronize()
            out = L.NoallocGridResult.from_buffer_copy(bytes(res.cpu().numpy()[:C.sizeof(L.NoallocGridResult)]))
            print(f"noalloc: rc {rc} status {out.status} {out.straight}+{out.diagonal}*sqrt2 "
                  f"path {out.path_len}", flush=True)
    else:
        tag = c
        if c == "cluster_small":
            # 36 15-puzzles of 120-move walks and 4 grids of 2200^2: a 64-round
            # budget on the single-CTA tier sends most of them to 8-CTA clusters
            specs = [WL.PuzzleSpec(4, 120, 8000 + i) for i in range(36)]
            specs += [WL.screened_grid(2200, 2200, 0.25, 21 + i, exact=True) for i in range(4)]
            kw = {"tier1_rounds": 64}
        else:
            specs = [WL.PuzzleSpec(4, 60 + i, 7000 + i) for i in range(48)]
            specs += [WL.screened_grid(256 + 32 * i, 256 + 32 * i, 0.25, 11 + i, exact=True) for i in range(8)]
            kw = {}
        insts = [s.instance() for s in specs]
        with Engine(0) as eng:
            eng.pdb_build(4)
            for _ in range(args.repeat):
                res, st = eng.batch_solve(insts, **kw)
                print(f"{tag}: {sum(r['status'] == 0 for r in res)}/{len(res)} ok, "
                      f"{st['wall_ms']:.1f} ms, waves {st['waves']}", flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--case", choices=CASES, help="run one workload for a profiler and exit")
    ap.add_argument("--repeat", type=int, default=2, help="--case: solves")
    ap.add_argument("--count", type=int, default=10, help="--case puzzle15: boards")
    ap.add_argument("--dedup", type=int, default=0, help="--case grids: 0 table minimum, 1 per-round sort + unique")
    ap.add_argument("--headline-only", action="store_true")
    ap.add_argument("--sections", default="c3,c4,c5,mb,dedup")
    ap.add_argument("--cpu-cap", type=int, default=12_000_000)
    ap.add_argument("--ref-cap", type=int, default=3_000_000)
    ap.add_argument("--ref-full-solve", type=int, default=1, help="reference arm: time one full solve on one core")
    ap.add_argument("--c3-count", type=int, default=100)
    ap.add_argument("--plain-sample", type=int, default=64)
    ap.add_argument("--serve-count", type=int, default=20000)
    ap.add_argument("--serve-extra-count", type=int, default=2000, help="requests at the lower rates")
    ap.add_argument("--serve-rates", type=lambda s: [float(x) for x in s.split(",")], default=[50.0, 200.0, 1000.0])
    ap.add_argument("--serve-timeout", type=float, default=600.0)
    ap.add_argument("--plain-budget", type=float, default=180.0,
                    help="seconds of plain-engine solves over the serving stream")
    ap.add_argument("--check-chunk", type=int, default=2500, help="serving: requests per batched check call")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--tune-stride", type=int, default=2)
    ap.add_argument("--cpu-sections", type=int, default=1, help="CPU baselines of the c3/c4/c5 sections")
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds per section CPU baseline")
    ap.add_argument("--cpu-solve-cap", type=int, default=4_000_000, help="expansions per CPU baseline solve")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    if args.case:
        run_case(args)
        return

    rank, world = int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        # rank 0 alone times the CPU path; the other ranks have nothing to do
        line = run_reference(args, rank, world)
        if rank == 0:
            print(json.dumps(line), flush=True)
        return

    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")

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
            eng.close()
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

"""Benchmark: Focused-ACO ant-tours+LS per second on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload throughput|uneven|large|gp-population|time-to-gap]
                    [--no-cpu-baseline] [--no-time-to-gap] [--window-only]

A step is one replay of the engine's per-evaluation CUDA graph: 16 ACO
iterations of the whole panel, in each of which every ant of every colony
constructs a tour from its colony's parent and runs its local search, then
each colony reduces, selects and updates its trails (the colonies run as
independent chains inside the graph, so one chain's slowest ants overlap
the other chains' iterations).  The W warm-up steps run in an evaluation of
their own; the K timed steps are iterations 0 .. 16K of a fresh evaluation
from the initial tours -- the same iterations the end-to-end call, the CPU
baseline and the reference arm run.  Default workload (throughput): 16
instances of N=1000 integer coordinates uniform in [0,10^6]^2 x 16 seeds =
256 colonies, 32 ants each, k=16, backup 64, LS width 20, MNE 8, 2-opt,
retention 0.98; its line also carries the converged window (iteration 400
on), the learned prior's time to a 1% gap against plain FACO (the
learned-prior workload: 64 instances, N in {1000, 2000}, 32 ants, k=20), and
`other_workloads`: the uneven, large and GP-population lines of the same run
(device and end-to-end values, each from a child run without its CPU
baseline).
Other workloads:
  uneven         256 clustered instances, N ~ U[200,1000], 16 ants, k=16
                 (one colony each; size-class launches in one CUDA graph);
                 the end-to-end call runs 500 iterations;
  large          16 clustered instances, N ~ U[5000,10000] in [0,10^7]^2,
                 5 seeds, 64 ants, k=32, 2-opt window 32 + Or-opt (<= 3);
  gp-population  one N=500 instance, 128 random GP controller programs, one
                 colony each, 32 ants, k=16, 1000 iterations per call (a step
                 is one population evaluation);
  time-to-gap    learned-prior vs plain FACO wall-clock to a 1% mean gap alone;
  large-prior    the large clustered panel (80 colonies, 1000 iterations)
                 plain against the learned prior with its per-instance plain
                 fallback: both arms' final gaps and every fallback decision.
The data are synthetic (seeded), standing in for the reference's uniform
TSP1000 rows and its batch workloads.  With N>1 each rank runs its own
panel (independent colonies, weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time
from dataclasses import dataclass
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

L2_BYTES = 129 * 2**20
CPU_COLONIES_PER_THREAD = 16
STEADY_ITERATION = 400   # the converged-colony window of the throughput workload
ITERATIONS_PER_STEP = 16  # a step: one replay of the engine's per-evaluation CUDA graph
# DRAM traffic and issue figures of the default panel from one ncu capture at
# iteration 160, the middle of the timed window (gplsaco_gb300.profile_ant:
# one unchained launch of the ant kernel and of the colony update over every
# colony): dram__bytes_read.sum + dram__bytes_write.sum of the two kernels,
# 21.48 MB + 34.20 MB per iteration, x 16 iterations per step; the ant
# kernel's smsp__issue_active and smsp__inst_executed (341.6 M over 8,192
# ant-tours).  Reported for the default workload only.
THROUGHPUT_CAPTURE = {
    "traffic_bytes_per_step": 16 * (21_403_136 + 30_208 + 34_198_528 + 22_528),
    "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of ant_kernel and colony_update_kernel, "
                       "one unchained launch each over every colony at iteration 160 of this panel, x 16 "
                       "iterations per step"),
    "ant_issue_active_pct": 61.36,
    "ant_warp_instructions_per_ant_tour": 335_252_667 / 8192,
    "issue_source": ("ncu smsp__issue_active.avg.pct_of_peak_sustained_active and smsp__inst_executed.sum of "
                     "the whole-panel ant launch at iteration 160 of this panel"),
}


@dataclass
class Workload:
    """One benchmark panel: instances, the colony -> (instance, seed) map and
    the FACO settings every colony runs with."""
    name: str
    metric: str
    description: str
    xys: list
    colony_instance: np.ndarray
    seeds: np.ndarray
    ants: int
    k: int
    b: int
    w: int
    ls_mode: int = 0
    mne: int = 8
    retention: float = 0.98
    e2e_iterations: int | None = None  # iterations of the end-to-end call (None: the timed window's)
    cpu_colonies_per_thread: int = CPU_COLONIES_PER_THREAD

    def run_iterations(self, steps: int) -> int:
        """Iterations of the end-to-end call; the CPU sample spans the same:
        the timed window (steps x 16 iterations from the initial tours)
        unless the workload names its own call length."""
        return self.e2e_iterations or ITERATIONS_PER_STEP * steps

    @property
    def colonies(self) -> int:
        return int(self.colony_instance.size)

    def sizes(self) -> np.ndarray:
        return np.array([len(self.xys[i]) for i in self.colony_instance], np.int64)


def instance_xy(i: int, n: int = 1000) -> np.ndarray:
    rng = np.random.default_rng(1000 + i)
    return rng.integers(0, 10**6 + 1, size=(n, 2)).astype(np.int32)


def make_workload(name: str, rank: int = 0) -> Workload:
    from gplsaco_gb300 import instances
    if name == "throughput":
        return Workload(
            "throughput", "ant-tours+LS/sec (plain FACO, N=1000)",
            "plain FACO, N=1000 uniform int coords, 16 instances x 16 seeds = 256 colonies, 32 ants, k=16, "
            "backup 64, LS width 20, MNE 8, 2-opt, retention 0.98",
            [instance_xy(i) for i in range(16)], np.repeat(np.arange(16), 16),
            np.tile(np.arange(16, dtype=np.uint64), 16) + np.uint64(1000 * rank), 32, 16, 64, 20)
    if name == "uneven":
        return Workload(
            "uneven", "ant-tours+LS/sec (uneven batch, N~U[200,1000])",
            "plain FACO, 256 clustered instances (4-16 Gaussian clusters, sigma 2-8% of [0,10^6], 20% uniform "
            "noise), N ~ U[200,1000], one colony each, 16 ants, k=16, backup 64, LS width 20, MNE 8, 2-opt, "
            "retention 0.98; colony chains of one size class each as parallel graph branches, warps per block "
            "autotuned",
            instances.uneven_batch(256, (200, 1000)), np.arange(256),
            np.full(256, 1 + 1000 * rank, np.uint64), 16, 16, 64, 20, e2e_iterations=500)
    if name == "large":
        return Workload(
            "large", "ant-tours+LS/sec (large clustered, N~U[5000,10000])",
            "plain FACO, 16 clustered instances (32-64 clusters, [0,10^7]^2), N ~ U[5000,10000], 5 seeds each "
            "= 80 colonies, 64 ants, k=32, backup 64, 2-opt window 32 + Or-opt (segments <= 3), MNE 8, "
            "retention 0.98",
            instances.large_clustered(16), np.repeat(np.arange(16), 5),
            np.tile(np.arange(5, dtype=np.uint64), 16) + np.uint64(1000 * rank), 64, 32, 64, 32, ls_mode=1,
            cpu_colonies_per_thread=2)
    raise ValueError(f"unknown workload {name}")


def max_over_ranks(value: float, world: int, device=None) -> float:
    """The job's time is the slowest rank's: MAX all-reduce of one float
    (NCCL on the GPU ranks; any initialised process group works)."""
    if world <= 1:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def size_classes(sizes) -> int:
    """Ant-kernel launches per iteration: one per instance size class
    (n rounded up to a power of two, at least 256)."""
    def class_of(n):
        c = 0
        while (256 << c) < n:
            c += 1
        return c
    return len({class_of(int(n)) for n in sizes})


def step_bytes(wl: Workload, work: np.ndarray, steps: int) -> dict:
    """Algorithmic bytes of one step (ITERATIONS_PER_STEP iterations of every
    colony) of a window of `steps` steps, from that window's own counters:
    per ant and iteration the parent read + tour write (8 B per node); per
    colony and iteration the trail update (16 B per candidate entry: trail
    read and write, product write, heuristic read); and the counted work --
    candidate id + weight per construction step (8 B x k), 20 B per LS move
    evaluation, 16 B per moved tour element."""
    n = wl.sizes().astype(np.float64)
    ants = ITERATIONS_PER_STEP * float(np.sum(8.0 * wl.ants * n))
    counted = 8.0 * wl.k * float(work[:, 0].sum()) + 20.0 * float(work[:, 1].sum()) + 16.0 * float(work[:, 2].sum())
    ants += counted / steps
    update = ITERATIONS_PER_STEP * float(np.sum(16.0 * n * wl.k))
    return {"ant_kernel": ants, "colony_update": update, "total": ants + update}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [line for line in out.splitlines() if line.strip()]

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in getattr(self, "lines", []):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_colonies(wl: Workload, threads: int, colonies: int, iterations: int, program=None) -> float:
    """Runs `colonies` colonies of the workload (its colonies in order,
    cycling) for `iterations` iterations each with the oracle port (C), one
    colony per host thread; returns elapsed seconds (preparation excluded)."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle
    oracle.lib()
    picks = [c % wl.colonies for c in range(colonies)]
    needed = sorted({int(wl.colony_instance[c]) for c in picks})
    with ThreadPoolExecutor(max_workers=threads) as pool:
        preps = dict(zip(needed, pool.map(lambda i: oracle.prepare(wl.xys[i], wl.k, wl.b, wl.w), needed)))

    def one(c):
        i = int(wl.colony_instance[c])
        oracle.run_colony(wl.xys[i], preps[i], ants=wl.ants, k=wl.k, b=wl.b, w=wl.w, mne=wl.mne,
                          iterations=iterations, key=oracle.lib().orc_colony_key(int(wl.seeds[c]), 1 + i),
                          retention=wl.retention, threads=1, want_trace=False, ls_mode=wl.ls_mode,
                          program=program, total_iterations=iterations if program else None)

    start = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as pool:
        list(pool.map(one, picks))
    return time.perf_counter() - start


def cpu_baseline(wl: Workload, iterations: int) -> dict:
    """The oracle port on a bounded sample of the same workload: one colony
    per host thread at a time, `iterations` iterations from the prepared
    initial tour."""
    threads = os.cpu_count() or 1
    colonies = min(wl.cpu_colonies_per_thread * threads, wl.colonies)
    elapsed = cpu_colonies(wl, threads, colonies, iterations)
    fe = colonies * wl.ants * iterations
    return {"value": fe / elapsed, "unit": "ant-tours+LS/s", "cores": threads, "kind": "port",
            "sample": f"{colonies} colonies of the {wl.name} panel x {wl.ants} ants x {iterations} iterations "
                      f"({fe} ant-tours+LS) from the prepared initial tour, one colony per host thread, "
                      f"{elapsed:.1f} s"}


def measured_peak():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        return json.loads(path.read_text())["hbm_gbs"], "measured"
    return 6800.0, "fallback"


def run_reference(args, rank: int) -> None:
    """The CPU implementation of the path (the oracle port; the reference's own
    C++ core is built only where its sources are) on all host threads: one
    colony per thread at a time, the workload's CPU sample length."""
    if rank != 0:
        return
    if args.workload == "gp-population":
        run_population_reference(args)
        return
    if args.workload in ("time-to-gap", "large-prior"):
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned edge prior: the "
                          "learned-prior comparisons have no reference arm"}), flush=True)
        return
    wl = make_workload(args.workload)
    threads = os.cpu_count() or 1
    iterations = wl.run_iterations(args.steps)
    colonies = min(wl.cpu_colonies_per_thread * threads, wl.colonies)
    cpu_colonies(wl, threads, threads, max(1, min(args.warmup, 3)))
    elapsed = cpu_colonies(wl, threads, colonies, iterations)
    fe = colonies * wl.ants * iterations
    value = fe / elapsed
    line = {"impl": "reference", "metric": wl.metric, "value": value, "unit": "ant-tours+LS/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * elapsed * ITERATIONS_PER_STEP / iterations,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64", "data": "synthetic",
            "config": {"workload": f"{wl.description}; CPU: {colonies} colonies ({threads} host threads, one "
                                   f"colony each at a time), {iterations} iterations from the initial tour",
                       "colonies": colonies, "ants": wl.ants, "timed_iterations": [0, iterations]},
            "cpu_baseline": {"value": value, "unit": "ant-tours+LS/s", "cores": threads, "kind": "port",
                             "sample": f"{colonies} colonies x {iterations} iterations"},
            "e2e": {"value": value, "unit": "ant-tours+LS/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _engine(wl: Workload, device: int, follow: int = 0):
    import gplsaco_gb300 as g
    settings = g.FixedFacoSettings(ants=wl.ants, primary_width=wl.k, backup_width=wl.b, ls_width=wl.w,
                                   retention=wl.retention, ls_mode=wl.ls_mode, follow=follow)
    engine = g.FacoBatchEngine(int(max(len(x) for x in wl.xys)), wl.colonies, settings, device=device)
    t0 = time.perf_counter()
    for i, xy in enumerate(wl.xys):
        engine.register_problem(1 + i, xy.astype(np.float64))
    return engine, time.perf_counter() - t0


def run_gb300(args, rank: int, world: int) -> None:
    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    wl = make_workload(args.workload, rank)
    engine, registration_s = _engine(wl, local, args.follow)
    keys = (wl.colony_instance + 1).astype(np.uint64)
    seeds = wl.seeds
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.ExternalStream(engine.stream_ptr)
    classes = size_classes(wl.sizes())

    def timed_steps() -> list:
        """K graph replays, L2 flushed before each, CUDA events on the engine's stream."""
        out = []
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            engine.step(per_step)
            b.record(stream)
            b.synchronize()
            out.append(a.elapsed_time(b))
        return out

    # ---- warm-up: W steps of an evaluation of their own ----
    engine.begin(keys, seeds, wl.mne)
    plan = engine.launch_plan()
    per_step = plan["graph_iterations"]
    assert per_step == ITERATIONS_PER_STEP, plan
    for _ in range(args.warmup):
        engine.step(per_step)
    engine.finish()
    torch.cuda.synchronize()

    # ---- device throughput: inputs resident, a fresh evaluation from the
    # initial tours, the K timed steps = iterations 0 .. 16K ----
    window = per_step * args.steps
    engine.begin(keys, seeds, wl.mne)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        step_ms = timed_steps()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
    totals = engine.finish()
    assert totals["completed_batches"] == window
    work = totals["colony_work"].astype(np.float64)        # the window's own counters
    elapsed_ms = max_over_ranks(float(np.sum(step_ms)), world, "cuda")
    fe_window = window * wl.colonies * wl.ants
    value = world * fe_window / (elapsed_ms / 1e3)
    if args.window_only:
        engine.close()
        if rank == 0:
            print(json.dumps({"metric": wl.metric, "value": value, "unit": "ant-tours+LS/s", "n_gpus": world,
                              "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps,
                              "window_only": True, "timed_iterations": [0, window],
                              "colony_work": work.sum(axis=0).tolist()}), flush=True)
        return

    # the same iterations again with every kernel launched alone (unchained)
    # and timed with events: the ant kernel's and the colony update's shares
    engine.begin(keys, seeds, wl.mne)
    ant_ms, upd_ms = engine.step_timed(window)
    engine.finish()

    steady = None
    if wl.name == "throughput":
        # converged colonies (construction walks the parent tour: more steps
        # and LS evaluations per tour), in an evaluation with per-iteration traces
        engine.begin(keys, seeds, wl.mne, trace_iterations=STEADY_ITERATION + window)
        engine.step(STEADY_ITERATION)
        torch.cuda.synchronize()
        steady_ms = timed_steps()
        trace = engine.finish()["trace"]
        late, early = trace[STEADY_ITERATION:], trace[:window]
        per_tour = float(fe_window)
        steady = {"value": world * per_tour / (max_over_ranks(float(np.sum(steady_ms)), world, "cuda") / 1e3),
                  "ms_per_step": float(np.mean(steady_ms)),
                  "timed_iterations": [STEADY_ITERATION, STEADY_ITERATION + window],
                  "per_tour": {"construction_steps": float(late["construction_steps"].sum()) / per_tour,
                               "ls_evaluations": float(late["ls_evaluations"].sum()) / per_tour},
                  "per_tour_in_the_value_window": {
                      "construction_steps": float(early["construction_steps"].sum()) / per_tour,
                      "ls_evaluations": float(early["ls_evaluations"].sum()) / per_tour}}

    # ---- end to end through the public API: host keys/seeds in, tours and
    # lengths out; one solve call over the window's iterations ----
    e2e_iters = wl.run_iterations(args.steps)
    engine.evaluate_faco_evaluations(keys, seeds, wl.ants * max(1, args.warmup), wl.mne)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = engine.evaluate_faco_evaluations(keys, seeds, wl.ants * e2e_iters, wl.mne)
    e2e_s = time.perf_counter() - t0
    e2e_value = e2e_iters * wl.colonies * wl.ants / e2e_s
    h2d = keys.nbytes + seeds.nbytes
    d2h = wl.colonies * engine.dimension * 4 + wl.colonies * 8
    assert all(len(it["tour"]) == n for it, n in zip(res["items"], wl.sizes()))
    engine.close()

    # ---- roofline of one step (the graph of ant launches and colony updates) ----
    sb = step_bytes(wl, work, args.steps)
    ms_per_step = elapsed_ms / args.steps
    achieved = sb["total"] / (ms_per_step / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    if rank != 0:
        return
    capture = THROUGHPUT_CAPTURE if wl.name == "throughput" else {}
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
        "traffic": capture.get("traffic_bytes_per_step"),
        "traffic_source": capture.get("traffic_source"),
        "kernel": "ant_kernel + colony_update_kernel: one graph replay (16 iterations, every colony chain)",
        "peak_source": peak_kind,
        "bytes_per_step": sb["total"], "bytes_per_fe": sb["total"] / (per_step * wl.colonies * wl.ants),
        "per_fe": {"construction_steps": float(work[:, 0].sum()) / fe_window,
                   "ls_evaluations": float(work[:, 1].sum()) / fe_window,
                   "moved_elements": float(work[:, 2].sum()) / fe_window},
        "ant_kernel": {"bytes_per_step": sb["ant_kernel"], "ms_per_step_unchained": ant_ms / args.steps,
                       "share_of_unchained_time": ant_ms / (ant_ms + upd_ms),
                       "achieved_unchained_gbs": sb["ant_kernel"] / (ant_ms / args.steps / 1e3) / 1e9},
        "colony_update_kernel": {"bytes_per_step": sb["colony_update"], "ms_per_step_unchained": upd_ms / args.steps},
        "issue": ({"ant_kernel_issue_active_pct": capture.get("ant_issue_active_pct"),
                   "ant_kernel_warp_instructions_per_ant_tour": capture.get("ant_warp_instructions_per_ant_tour"),
                   "source": capture.get("issue_source")}
                  if capture.get("ant_issue_active_pct") else None),
    }
    base = cpu_baseline(wl, e2e_iters) if args.cpu_baseline else None
    line = {
        "metric": wl.metric, "value": value, "unit": "ant-tours+LS/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int64", "data": "synthetic",
        "config": {"workload": wl.description, "colonies": wl.colonies, "ants": wl.ants,
                   "n_range": [int(wl.sizes().min()), int(wl.sizes().max())],
                   "l2": "flushed before every timed step (258 MB write)",
                   "iterations_per_step": per_step,
                   "timed_iterations": [0, window],
                   "warmup": "W steps of a separate evaluation; the timed one starts from the initial tours",
                   "colony_chains": plan["chains"], "follow_batches": {0: "off", 1: "on", 2: "every 32 iterations from the walk length"}[plan["follow"]],
                   "registration_seconds": registration_s, "size_classes": classes},
        "e2e": {"value": e2e_value, "unit": "ant-tours+LS/s", "h2d_bytes_per_step": h2d * per_step / e2e_iters,
                "d2h_bytes_per_step": d2h * per_step / e2e_iters, "iterations": e2e_iters,
                "bytes_per_call": {"h2d": h2d, "d2h": d2h},
                "call": "FacoBatchEngine.evaluate_faco_evaluations (C ABI faco_evaluate), host keys/seeds in, "
                        "host tours/costs out"},
        "roofline": roofline,
        "cpu_baseline": base,
        "clocks": clocks.summary(),
        "gpu_launches": plan["launches_per_iteration"] * window,
    }
    if steady is not None:
        line["steady_state"] = steady
    if wl.name == "throughput" and args.time_to_gap and world == 1:
        line["time_to_gap"] = time_to_gap_block(local, args.follow)
    if wl.name == "throughput" and args.other_workloads and world == 1 and not args.window_only:
        line["other_workloads"] = other_workloads_block(args)
    print(json.dumps(line), flush=True)


OTHER_WORKLOADS = (("uneven", []), ("large", []), ("gp-population", []), ("gp-population", ["--controller", "2"]))


def other_workloads_block(args) -> dict:
    """The other throughput workloads in the same run, each as a child bench
    process (its own device context and memory) without its CPU baseline:
    device and end-to-end value, the workload, its kernel choice and the
    clocks seen while it ran."""
    out = {}
    for name, extra in OTHER_WORKLOADS:
        label = name + ("-controller-2" if extra else "")
        cmd = [sys.executable, str(Path(__file__).resolve()), "--workload", name, "--no-cpu-baseline",
               "--steps", str(args.steps), "--warmup", str(args.warmup), "--follow", str(args.follow), *extra]
        try:
            proc = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
            lines = [ln for ln in proc.stdout.splitlines() if ln.startswith("{")]
            if proc.returncode != 0 or not lines:
                out[label] = {"error": (proc.stderr or proc.stdout)[-300:]}
                continue
            d = json.loads(lines[-1])
        except subprocess.TimeoutExpired:
            out[label] = {"error": "timed out"}
            continue
        cfg = d.get("config", {})
        out[label] = {"metric": d.get("metric"), "value": d.get("value"), "unit": d.get("unit"),
                      "ms_per_step": d.get("ms_per_step"), "e2e": (d.get("e2e") or {}).get("value"),
                      "workload": cfg.get("workload"), "timed_iterations": cfg.get("timed_iterations"),
                      "follow_batches": cfg.get("follow_batches"), "clocks": d.get("clocks")}
    return out


def time_to_gap_block(device: int = 0, follow: int = 0) -> dict:
    """The learned prior's wall-clock to a 1% mean gap against plain GPU FACO
    (the learned-prior workload; both arms tuned on validation instances)."""
    from gplsaco_gb300 import experiments
    res = experiments.time_to_gap(experiments.GapConfig(follow=follow), device=device,
                                  log=lambda m: print(m, file=sys.stderr, flush=True))
    out = experiments.summary(res)
    out["workload"] = ("64 instances (seeds 100-163; N=1000 for 100-131, 2000 for 132-163; uniform for even "
                       "seeds, clustered for odd), 32 ants, k=20, LS width 20, retention 0.98, 2-opt; budget "
                       f"{res['budget_iterations']} iterations per method; reference length = best of 2 plain "
                       "runs of 3000 iterations; prior trained on the engine's own runs of 32 training instances")
    out["follow"] = {0: "auto", 1: "off", 2: "on"}[follow]
    out["ratio_definition"] = ("prior/plain wall-clock to the target, equal resources: two colonies per instance "
                               "in both arms (plain: seeds 1, 2; prior: seed 1 plain as the per-instance fallback + "
                               "seed 2 with the prior), best of the two; ratio_one_colony_per_instance charges the "
                               "prior for the plain warm-up run that decides its fallback")
    return out


# ---- GP evaluation batch: 128 controller programs on one N=500 instance ----
POP_N, POP_SEED, POP_PROGRAMS, POP_ITERATIONS = 500, 2, 128, 1000
POP_METRIC = "GP individuals evaluated/sec (N=500, 32 ants, 1000 iterations each)"


def population_programs(spec: int = 3) -> list:
    """128 random controller programs: feature spec 3 (the colony features of
    the GP evaluation batch) or 2 (the reference's 12-feature controller)."""
    from gplsaco_gb300.programs import random_program
    rng = np.random.default_rng(POP_SEED)
    return [random_program(rng, extended=True, features=10 if spec == 3 else 12, feature_spec_id=spec)
            for _ in range(POP_PROGRAMS)]


def population_workload() -> Workload:
    from gplsaco_gb300 import instances
    return Workload("gp-population", POP_METRIC, "", [instances.uniform(POP_N, POP_SEED)], np.zeros(1, np.int64),
                    np.ones(1, np.uint64), 32, 16, 64, 20)


def population_cpu(threads: int, colonies: int, iterations: int, spec: int = 3) -> float:
    """Elapsed seconds of `colonies` controller-driven colonies (programs in
    order) of `iterations` iterations on the oracle port, one per thread."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle
    oracle.lib()
    wl = population_workload()
    programs = population_programs(spec)
    prep = oracle.prepare(wl.xys[0], wl.k, wl.b, wl.w)

    def one(c):
        oracle.run_colony(wl.xys[0], prep, ants=wl.ants, k=wl.k, b=wl.b, w=wl.w, mne=wl.mne, iterations=iterations,
                          key=oracle.lib().orc_colony_key(1, 1), retention=wl.retention, threads=1,
                          want_trace=False, program=programs[c % len(programs)], total_iterations=POP_ITERATIONS,
                          instance_key=1)

    start = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as pool:
        list(pool.map(one, range(colonies)))
    return time.perf_counter() - start


def population_cpu_line(colonies_per_thread: int = 2, spec: int = 3) -> dict:
    """Whole 1000-iteration controller-driven runs of the first programs on
    the oracle port, one colony per host thread at a time."""
    threads = os.cpu_count() or 1
    colonies = min(POP_PROGRAMS, colonies_per_thread * threads)
    elapsed = population_cpu(threads, colonies, POP_ITERATIONS, spec)
    value = colonies / elapsed
    return {"value": value, "unit": "individuals/s", "cores": threads, "kind": "port",
            "sample": f"{colonies} of the {POP_PROGRAMS} programs, whole {POP_ITERATIONS}-iteration colony runs, "
                      f"one per host thread at a time, {elapsed:.1f} s"}


def run_population_reference(args) -> None:
    base = population_cpu_line(spec=args.controller)
    line = {"impl": "reference", "metric": POP_METRIC, "value": base["value"], "unit": "individuals/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64", "data": "synthetic",
            "config": {"workload": "GP evaluation batch on the oracle port (CPU sample)"},
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": "individuals/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_population(args, rank: int, world: int) -> None:
    import torch

    import gplsaco_gb300 as g

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    wl = population_workload()
    programs = population_programs(args.controller)
    settings = g.FixedFacoSettings(ants=wl.ants, primary_width=wl.k, backup_width=wl.b, ls_width=wl.w,
                                   retention=wl.retention, follow=args.follow)
    engine = g.FacoBatchEngine(POP_N, 1, settings, population_size=POP_PROGRAMS, device=local)
    engine.register_problem(1, wl.xys[0].astype(np.float64))
    keys, seeds = np.ones(1, np.uint64), np.array([1 + 1000 * rank], np.uint64)
    stream = torch.cuda.ExternalStream(engine.stream_ptr)
    budget = wl.ants * POP_ITERATIONS
    for _ in range(args.warmup):
        engine.evaluate_population_evaluations(keys, seeds, budget, programs)
    torch.cuda.synchronize()
    dev_ms, wall = [], []
    with ClockSampler(local) as clocks:
        if world > 1:
            torch.distributed.barrier()
        for _ in range(args.steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0 = time.perf_counter()
            a.record(stream)
            res = engine.evaluate_population_evaluations(keys, seeds, budget, programs)
            b.record(stream)
            b.synchronize()
            wall.append(time.perf_counter() - t0)
            dev_ms.append(a.elapsed_time(b))
        if world > 1:
            torch.distributed.barrier()
    assert len(res) == POP_PROGRAMS and all(len(r["items"][0]["tour"]) == POP_N for r in res)
    elapsed_ms = max_over_ranks(float(np.sum(dev_ms)), world, "cuda")
    plan = engine.launch_plan()
    engine.close()
    if rank != 0:
        return
    value = args.steps * POP_PROGRAMS * world / (elapsed_ms / 1e3)
    e2e = args.steps * POP_PROGRAMS / float(np.sum(wall))
    base = population_cpu_line(spec=args.controller) if args.cpu_baseline else None
    controller = ("feature spec 3: 7 colony features + 3 action descriptors" if args.controller == 3 else
                  "feature spec 2: the reference's 12-feature controller with its tour archive")
    line = {
        "metric": POP_METRIC, "value": value, "unit": "individuals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int64", "data": "synthetic",
        "config": {"workload": "GP evaluation batch: 1 uniform N=500 instance (seed 2), 128 random controller "
                               "programs (depth <= 6), one colony each, 32 ants, k=16, 1000 "
                               "iterations; a step is one evaluate_population_evaluations call",
                   "controller": controller, "colony_chains": plan["chains"],
                   "l2": "each step runs 1000 iterations; the panel's working set (~30 MB) is L2-resident by design"},
        "e2e": {"value": e2e, "unit": "individuals/s", "h2d_bytes_per_step": float(keys.nbytes + seeds.nbytes),
                "d2h_bytes_per_step": float(POP_PROGRAMS * (POP_N * 4 + 8)),
                "call": "FacoBatchEngine.evaluate_population_evaluations (C ABI faco_evaluate_programs)"},
        "roofline": None,
        "cpu_baseline": base,
        "clocks": clocks.summary(),
        "gpu_launches": (1 + plan["launches_per_iteration"] * POP_ITERATIONS) * args.steps,
    }
    print(json.dumps(line), flush=True)


def run_time_to_gap(args) -> None:
    import torch

    torch.cuda.set_device(0)
    block = time_to_gap_block(0, args.follow)
    line = {"metric": "time to 1% mean gap, learned-prior vs plain GPU FACO (ratio)", "value": block["ratio"],
            "unit": "prior/plain wall-clock", "higher_is_better": False, "n_gpus": 1, "data": "synthetic",
            "config": {"workload": block["workload"]}, "time_to_gap": block}
    print(json.dumps(line), flush=True)


def run_large_prior(args) -> None:
    import torch

    torch.cuda.set_device(0)
    from gplsaco_gb300 import experiments
    res = experiments.large_prior(experiments.LargeConfig(follow=args.follow),
                                  log=lambda m: print(m, file=sys.stderr, flush=True))
    line = {"metric": "final mean gap after 1000 iterations, plain vs learned prior with per-instance fallback "
                      "(large clustered panel)",
            "value": res["final_gap_prior"], "plain_value": res["final_gap_plain"], "unit": "mean gap",
            "higher_is_better": False, "n_gpus": 1, "data": "synthetic",
            "config": {"workload": "16 clustered instances, N ~ U[5000,10000], 32-64 clusters in [0,10^7]^2, 5 seeds "
                                   "each (80 colonies), 64 ants, k=32, 2-opt window 32 + Or-opt (<= 3), MNE 8, "
                                   "retention 0.98, 1000 iterations; prior trained on 16 smaller instances of the "
                                   "same generator (N 1000-2000); fallback at iteration 96; gaps against the best "
                                   "length either arm reaches"},
            "large_prior": res}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-time-to-gap", dest="time_to_gap", action="store_false",
                    help="leave the learned prior's time-to-gap block out of the throughput line")
    ap.add_argument("--follow", type=int, default=0, choices=[0, 1, 2],
                    help="parent-following construction steps in batches: 0 auto (always when every ant warp "
                         "fits in one wave of the GPU, else chosen every 32 iterations from the walk length), "
                         "1 off, 2 on")
    ap.add_argument("--no-other-workloads", dest="other_workloads", action="store_false",
                    help="leave the uneven, large and GP-population blocks out of the throughput line")
    ap.add_argument("--window-only", action="store_true",
                    help="registration, warm-up and the timed window only (for kernel profiles): no unchained "
                         "replay, converged window, end-to-end call, CPU baseline or time-to-gap")
    ap.add_argument("--workload", default="throughput",
                    choices=["throughput", "uneven", "large", "gp-population", "time-to-gap", "large-prior"],
                    help="time-to-gap: learned-prior vs plain FACO wall-clock to a 1%% mean gap (N=1000/2000)")
    ap.add_argument("--controller", type=int, default=3, choices=[2, 3],
                    help="gp-population: feature spec of the programs (3: the batch's colony features; "
                         "2: the reference's 12-feature controller)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.workload == "time-to-gap":
        run_time_to_gap(args)
        return
    if args.workload == "large-prior":
        run_large_prior(args)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    if args.workload == "gp-population":
        run_population(args, rank, world)
    else:
        run_gb300(args, rank, world)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

"""Benchmark: plain Focused-ACO ant-tours+LS per second at N=1000 on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

A step is one ACO iteration of the whole panel: every ant of every colony
constructs a tour from its colony's parent and runs its local search, then
each colony reduces, selects and updates its trails.  Workload: 16 instances
of N=1000 integer coordinates uniform in [0,10^6]^2 x 16 seeds = 256 colonies,
32 ants each, k=16, backup 64, LS width 20, MNE 8, 2-opt, retention 0.98.
The data are synthetic (seeded), standing in for the reference's uniform
TSP1000 rows.  With N>1 each rank runs its own panel (independent colonies,
weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N = 1000
INSTANCES = 16
SEEDS_PER_INSTANCE = 16
ANTS, K_PRIMARY, BACKUP, LS_WIDTH, MNE, RETENTION = 32, 16, 64, 20, 8, 0.98
PRECONDITION = 100   # untimed iterations before the timed steps (steady-state trails)
CPU_COLONIES_PER_THREAD = 6
METRIC = "ant-tours+LS/sec (plain FACO, N=1000)"
L2_BYTES = 129 * 2**20


def instance_xy(i: int) -> np.ndarray:
    rng = np.random.default_rng(1000 + i)
    return rng.integers(0, 10**6 + 1, size=(N, 2)).astype(np.int32)


def bytes_per_fe(n, k, ants, steps_per_fe, evals_per_fe, moved_per_fe) -> float:
    """Algorithmic bytes per ant-tour+LS: parent read + tour write (8N),
    candidate id + weight per construction step (8k each), 20 B per LS move
    evaluation, 16 B per moved tour element, trail update amortised per ant."""
    return 8 * n + 8 * k * steps_per_fe + 20 * evals_per_fe + 16 * moved_per_fe + 16 * n * k / ants


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
                                          "--format=csv,noheader,nounits", "-lms", "200"],
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


def cpu_colonies(threads: int, colonies: int, iterations: int) -> float:
    """Runs `colonies` N=1000 colonies of `iterations` iterations each with the
    oracle port (C), one colony per host thread; returns elapsed seconds."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle
    oracle.lib()
    xy = instance_xy(0)
    prep = oracle.prepare(xy, K_PRIMARY, BACKUP, LS_WIDTH)

    def one(i):
        oracle.run_colony(xy, prep, ants=ANTS, k=K_PRIMARY, b=BACKUP, w=LS_WIDTH, mne=MNE, iterations=iterations,
                          key=oracle.lib().orc_colony_key(i, 1), retention=RETENTION, threads=1, want_trace=False)

    start = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as pool:
        list(pool.map(one, range(colonies)))
    return time.perf_counter() - start


def cpu_baseline(iterations: int) -> dict:
    """The oracle port on a bounded sample of the same workload: one N=1000
    colony of 32 ants per host thread, `iterations` iterations from the
    prepared initial tour (the span of the e2e measurement)."""
    threads = os.cpu_count() or 1
    colonies = CPU_COLONIES_PER_THREAD * threads
    elapsed = cpu_colonies(threads, colonies, iterations)
    fe = colonies * ANTS * iterations
    return {"value": fe / elapsed, "unit": "ant-tours+LS/s", "cores": threads, "kind": "port",
            "sample": f"{colonies} N=1000 colonies x 32 ants x {iterations} iterations ({fe} ant-tours+LS) "
                      f"from the prepared initial tour, one colony per host thread, {elapsed:.1f} s"}


def measured_peak():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        return json.loads(path.read_text())["hbm_gbs"], "measured"
    return 6800.0, "fallback"


def run_reference(args, rank: int) -> None:
    """The CPU implementation of the path (the oracle port; the reference's own
    C++ core cannot be built on this host) on all host threads: one colony per
    thread, PRECONDITION + steps iterations each, like the e2e measurement."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    iterations = PRECONDITION + args.steps
    colonies = CPU_COLONIES_PER_THREAD * threads
    cpu_colonies(threads, threads, max(1, args.warmup))
    elapsed = cpu_colonies(threads, colonies, iterations)
    fe = colonies * ANTS * iterations
    value = fe / elapsed
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "ant-tours+LS/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / iterations,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
            "data": "synthetic",
            "config": {"workload": f"plain FACO N=1000 uniform, {colonies} colonies x 32 ants ({threads} host "
                                   f"threads, one colony each at a time), k=16, backup 64, LS width 20, MNE 8, "
                                   f"2-opt, retention 0.98, {iterations} iterations from the initial tour",
                       "colonies": colonies, "ants": ANTS, "n": N},
            "cpu_baseline": {"value": value, "unit": "ant-tours+LS/s", "cores": threads, "kind": "port",
                             "sample": f"{colonies} colonies x {iterations} iterations"},
            "e2e": {"value": value, "unit": "ant-tours+LS/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gb300(args, rank: int, world: int) -> None:
    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    import gplsaco_gb300 as g

    colonies = INSTANCES * SEEDS_PER_INSTANCE
    settings = g.FixedFacoSettings(ants=ANTS, primary_width=K_PRIMARY, backup_width=BACKUP, ls_width=LS_WIDTH,
                                   retention=RETENTION)
    engine = g.FacoBatchEngine(N, colonies, settings, device=local)
    t0 = time.perf_counter()
    for i in range(INSTANCES):
        engine.register_problem(1 + i, instance_xy(i).astype(np.float64))
    registration_s = time.perf_counter() - t0
    keys = np.repeat(np.arange(1, INSTANCES + 1, dtype=np.uint64), SEEDS_PER_INSTANCE)
    seeds = (np.tile(np.arange(SEEDS_PER_INSTANCE, dtype=np.uint64), INSTANCES)
             + np.uint64(1000 * rank))
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.ExternalStream(engine.stream_ptr)

    # ---- device throughput: inputs resident, L2 flushed before every step ----
    # the panel first runs PRECONDITION iterations so that the timed steps see
    # converged trails (construction steps per tour grow as they converge)
    engine.begin(keys, seeds, MNE)
    engine.step(PRECONDITION + args.warmup)
    torch.cuda.synchronize()
    step_ms = []
    with ClockSampler(local) as clocks:
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            engine.step(1)
            b.record(stream)
            b.synchronize()
            step_ms.append(a.elapsed_time(b))
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
    # per-kernel split of a few more steps (ant kernel = the dominant kernel)
    kernel_steps = 3
    ant_ms, upd_ms = engine.step_timed(kernel_steps)
    totals = engine.finish()
    iters = totals["completed_batches"]
    fe_total = iters * colonies * ANTS
    s_fe = totals["construction_steps"] / fe_total
    e_fe = totals["ls_evaluations"] / fe_total
    r_fe = totals["reversed_elements"] / fe_total
    elapsed_ms = float(np.sum(step_ms))
    if world > 1:
        t = torch.tensor([elapsed_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    fe_timed = args.steps * colonies * ANTS * world
    value = fe_timed / (elapsed_ms / 1e3)

    # ---- end to end through the public API: host keys/seeds in, tours out;
    # one solve call of PRECONDITION + steps iterations from the initial tours ----
    e2e_iters = PRECONDITION + args.steps
    engine.evaluate_faco_evaluations(keys, seeds, ANTS * args.warmup, MNE)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = engine.evaluate_faco_evaluations(keys, seeds, ANTS * e2e_iters, MNE)
    e2e_s = time.perf_counter() - t0
    e2e_value = e2e_iters * colonies * ANTS / e2e_s
    h2d = keys.nbytes + seeds.nbytes
    d2h = colonies * N * 4 + colonies * 8
    assert all(len(it["tour"]) == N for it in res["items"])

    # ---- roofline of the ant kernel (per launch = one step of all ants) ----
    bfe = bytes_per_fe(N, K_PRIMARY, ANTS, s_fe, e_fe, r_fe)
    ants_per_launch = colonies * ANTS
    achieved = bfe * ants_per_launch / (ant_ms / kernel_steps / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    engine.close()
    if rank != 0:
        return
    base = cpu_baseline(PRECONDITION + 4) if args.cpu_baseline else None
    line = {
        "metric": METRIC, "value": value, "unit": "ant-tours+LS/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int64", "data": "synthetic",
        "config": {"workload": "plain FACO, N=1000 uniform int coords, 16 instances x 16 seeds = 256 colonies, "
                               "32 ants, k=16, backup 64, LS width 20, MNE 8, 2-opt, retention 0.98",
                   "colonies": colonies, "ants": ANTS, "n": N, "l2": "flushed before every timed step "
                   "(258 MB write)", "timed_iterations_start_at": PRECONDITION + args.warmup,
                   "registration_seconds": registration_s},
        "e2e": {"value": e2e_value, "unit": "ant-tours+LS/s", "h2d_bytes_per_step": h2d / e2e_iters,
                "d2h_bytes_per_step": d2h / e2e_iters, "iterations": e2e_iters,
                "call": "FacoBatchEngine.evaluate_faco_evaluations (C ABI faco_evaluate), host keys/seeds in, "
                        "host tours/costs out"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "kernel": "ant_kernel<engine>", "peak_source": peak_kind,
                     "bytes_per_fe": bfe, "per_fe": {"construction_steps": s_fe, "ls_evaluations": e_fe,
                                                      "moved_elements": r_fe},
                     "ant_kernel_ms": ant_ms / kernel_steps, "update_kernel_ms": upd_ms / kernel_steps},
        "cpu_baseline": base,
        "clocks": clocks.summary(),
        "gpu_launches": 2 * args.steps,
    }
    print(json.dumps(line), flush=True)


def run_time_to_gap(args) -> None:
    import torch

    torch.cuda.set_device(0)
    from gplsaco_gb300 import experiments
    res = experiments.time_to_gap(log=lambda m: print(m, file=sys.stderr, flush=True))
    line = {"metric": "time to 1% mean gap, learned-prior vs plain GPU FACO (ratio)", "value": res["ratio"],
            "unit": "prior/plain wall-clock", "higher_is_better": False, "n_gpus": 1, "data": "synthetic",
            "config": {"workload": "16 instances (N=1000/2000, uniform/clustered, seeds 100-115), 32 ants, "
                                   "k=20, MNE 8, 2-opt; reference = best of 2 plain runs of 1500 iterations"},
            "time_to_gap": res}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--workload", default="throughput", choices=["throughput", "time-to-gap"],
                    help="time-to-gap: learned-prior vs plain FACO wall-clock to a 1%% mean gap (N=1000/2000)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.workload == "time-to-gap":
        run_time_to_gap(args)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    run_gb300(args, rank, world)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

"""Where the time of an uneven batch goes, and how much a persistent kernel
could take off it.

    python -m gplsaco_gb300.uneven_study [--iterations 512]

The uneven batch: 256 clustered instances with N ~ U[200, 1000], one colony
each, 16 ants, k=16, backup 64, LS width 20, MNE 8, retention 0.98.  Every
run below is timed with CUDA events on the engine's stream over the first
`iterations` iterations from the initial tours, after a warm-up evaluation
on the same engine:

  full            all 256 colonies, the default launch plan (one ant launch
                  per size class as parallel graph branches, colonies dealt
                  into independent chains)
  full, steps one at a time
                  the same without batched parent-following steps
  one-chain       all 256 colonies in one chain: every iteration waits for
                  the slowest colony of the batch (and chains=2, 4)
  class c         only the colonies of size class c (n in (128 * 2^c, 256 * 2^c]),
                  default plan
  unchained       the largest class again, every ant launch and colony
                  update launched alone with events around each: the device
                  milliseconds of the ant kernel and of the colony update;
                  the chained run of the class less these is the time
                  between kernels (launch gaps, branch joins)
  largest colony alone
                  the N = 992 colony by itself: the latency of one colony's
                  iterations on an otherwise idle GPU

A persistent kernel that keeps every colony's iterations inside one launch
still runs the iterations of one colony one after another, each waiting for
that colony's slowest ant; so the largest class run alone is a lower bound
on its time, and the unchained split shows the most it could remove there
(the launch gaps, and the update if it were free).  One JSON line per run.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import instances
from .engine import FacoBatchEngine, FixedFacoSettings


def class_of(n: int) -> int:
    c = 0
    while (256 << c) < n:
        c += 1
    return c


def _engine(xys, chains: int = 0, follow: int = 0) -> FacoBatchEngine:
    settings = FixedFacoSettings(ants=16, primary_width=16, backup_width=64, ls_width=20, retention=0.98,
                                 chains=chains, follow=follow)
    engine = FacoBatchEngine(max(len(x) for x in xys), len(xys), settings)
    for i, xy in enumerate(xys):
        engine.register_problem(1 + i, xy.astype(np.float64))
    return engine


WARMUP_ITERATIONS = 64


def _run(name: str, xys, iterations: int, chains: int = 0, unchained: bool = False, follow: int = 0) -> dict:
    import torch
    engine = _engine(xys, chains, follow)
    keys = np.arange(1, len(xys) + 1, dtype=np.uint64)
    seeds = np.ones(len(xys), np.uint64)
    stream = torch.cuda.ExternalStream(engine.stream_ptr)
    engine.begin(keys, seeds, 8)
    engine.step(WARMUP_ITERATIONS)
    engine.finish()
    engine.begin(keys, seeds, 8)
    plan = engine.launch_plan()
    torch.cuda.synchronize()
    out = {"run": name, "colonies": len(xys), "n_min": min(len(x) for x in xys),
           "n_max": max(len(x) for x in xys), "iterations": iterations, "plan": plan}
    if unchained:
        ant_ms, update_ms = engine.step_timed(iterations)
        res = engine.finish()
        out.update({"ant_ms": ant_ms, "update_ms": update_ms})
    else:
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        engine.step(iterations)
        b.record(stream)
        b.synchronize()
        res = engine.finish()
        out["ms"] = a.elapsed_time(b)
        out["ant_tours_per_s"] = len(xys) * 16 * iterations / (out["ms"] * 1e-3)
    out["mean_cost"] = float(np.mean(res["costs"]))
    out["construction_steps"] = res["construction_steps"]
    out["ls_evaluations"] = res["ls_evaluations"]
    engine.close()
    return out


def main(argv=None) -> None:
    global WARMUP_ITERATIONS
    ap = argparse.ArgumentParser()
    ap.add_argument("--iterations", type=int, default=512)
    ap.add_argument("--warmup-iterations", type=int, default=WARMUP_ITERATIONS)
    ap.add_argument("--only", help="run only this one (full, one-chain, chains=G, class C)")
    args = ap.parse_args(argv)
    WARMUP_ITERATIONS = args.warmup_iterations
    xys = instances.uneven_batch(256, (200, 1000))
    classes = sorted({class_of(len(x)) for x in xys})
    if args.only:
        if args.only.startswith("class "):
            part = [x for x in xys if class_of(len(x)) == int(args.only.split()[1])]
            print(json.dumps(_run(args.only, part, args.iterations)), flush=True)
        else:
            chains = {"full": 0, "one-chain": 1}.get(args.only)
            if chains is None:
                chains = int(args.only.split("=")[1])
            print(json.dumps(_run(args.only, xys, args.iterations, chains=chains)), flush=True)
        return
    print(json.dumps(_run("full", xys, args.iterations)), flush=True)
    print(json.dumps(_run("full, steps one at a time", xys, args.iterations, follow=1)), flush=True)
    for chains in (1, 2, 4):
        name = "one-chain" if chains == 1 else f"chains={chains}"
        print(json.dumps(_run(name, xys, args.iterations, chains=chains)), flush=True)
    runs = []
    for c in classes:
        part = [x for x in xys if class_of(len(x)) == c]
        runs.append(_run(f"class {c}", part, args.iterations))
        print(json.dumps(runs[-1]), flush=True)
    largest = [x for x in xys if class_of(len(x)) == classes[-1]]
    line = _run(f"class {classes[-1]} unchained", largest, args.iterations, unchained=True)
    # launch gaps of the chained run of the same colonies: its time less the
    # device time of its kernels
    line["chained_ms"] = runs[-1]["ms"]
    line["gap_ms"] = line["chained_ms"] - line["ant_ms"] - line["update_ms"]
    print(json.dumps(line), flush=True)
    one = [x for x in xys if len(x) == max(len(y) for y in xys)]
    print(json.dumps(_run("largest colony alone", one, args.iterations)), flush=True)

if __name__ == "__main__":
    main()

"""One ant-kernel launch of the throughput panel at a chosen iteration, for
kernel profiles.

    python -m gplsaco_gb300.profile_ant --save PATH [--iterations I]
    python -m gplsaco_gb300.profile_ant --load PATH [--follow F] [--launches L]

The first form runs the throughput panel (16 instances of N=1000 uniform
integer coordinates x 16 seeds = 256 colonies, 32 ants, k=16, backup 64, LS
width 20, MNE 8, retention 0.98) for I iterations and writes a colony
snapshot.  The second form registers the same panel with the launch-shape
tuner off (so that no tuning launches precede it), restores the snapshot and
runs L iterations with every kernel launched alone (unchained), printing the
device milliseconds of the ant kernel and of the colony update.  Under a
profiler the L ant launches of the second form are the only ant-kernel
launches of their variant after registration: `ant_kernel<0>` (steps one at
a time, F=1) or `ant_kernel<7>` (parent-following steps in batches, F=2: the
batched build for panels beyond one wave, which this panel is).
"""
from __future__ import annotations

import argparse
import json
from pathlib import Path

import numpy as np

from . import instances
from .engine import CountedState, FacoBatchEngine, FixedFacoSettings


def panel(follow: int = 0, autotune: int = 1):
    settings = FixedFacoSettings(ants=32, primary_width=16, backup_width=64, ls_width=20, retention=0.98,
                                 follow=follow, autotune=autotune)
    engine = FacoBatchEngine(1000, 256, settings)
    for i in range(16):
        engine.register_problem(1 + i, instances.uniform(1000, 1000 + i).astype(np.float64))
    keys = np.repeat(np.arange(1, 17, dtype=np.uint64), 16)
    seeds = np.tile(np.arange(16, dtype=np.uint64), 16)
    return engine, keys, seeds


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--save")
    ap.add_argument("--load")
    ap.add_argument("--iterations", type=int, default=400)
    ap.add_argument("--follow", type=int, default=1, choices=[1, 2])
    ap.add_argument("--launches", type=int, default=1)
    args = ap.parse_args(argv)
    if args.save:
        engine, keys, seeds = panel(follow=1)
        engine.begin(keys, seeds, 8)
        engine.step(args.iterations)
        Path(args.save).write_bytes(engine.capture_state().to_bytes())
        engine.finish()
        engine.close()
        print(json.dumps({"saved": args.save, "iterations": args.iterations}))
        return
    if not args.load:
        ap.error("--save or --load is required")
    engine, _, _ = panel(follow=args.follow, autotune=0)
    engine.restore_state(CountedState(Path(args.load).read_bytes()))
    ant_ms, update_ms = engine.step_timed(args.launches)
    res = engine.finish()
    print(json.dumps({"follow": args.follow, "launches": args.launches, "ant_ms": ant_ms, "update_ms": update_ms,
                      "iterations_done": res["completed_batches"], "mean_cost": float(np.mean(res["costs"]))}))
    engine.close()


if __name__ == "__main__":
    main()

"""Generates tests/golden/ref_colony_lengths.json: final tour lengths of
whole plain-FACO colony runs by the reference's own CPU core (oracle/_ref,
compiled from the reference sources), 100 seeds per case, on seeded uniform
instances with the EUC_2D integer metric.  The engine's distributions over
the same seed count are compared with these (mean and Mann-Whitney), since the
reference draws its randomness from std::mt19937_64 and the engine from
Philox: only the distributions, not the tours, can agree.

    python tests/golden/make_ref_distribution.py   (needs oracle/build_ref.sh)
"""
from __future__ import annotations

import json
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from gplsaco_gb300 import instances  # noqa: E402
from oracle import oracle  # noqa: E402

# (n, instance seed, iterations): config 1's instance and uniform N=500/1000
CASES = [(100, 1, 100), (500, 2, 100), (1000, 3, 100), (500, 2, 300), (1000, 3, 300)]
SEEDS = list(range(1, 101))
PARAMS = dict(ants=32, k=16, b=64, w=20, mne=8, retention=0.98, p_best=0.1, epoch_source_probability=0.01)


def main() -> None:
    if oracle.ref() is None:
        raise SystemExit("oracle/_ref is not built (oracle/build_ref.sh)")
    out = {"generator": "gplsaco_gb300.instances.uniform(n, seed), coordinates in [0, 10^6]^2",
           "metric": "EUC_2D integer", "params": PARAMS, "seeds": SEEDS, "cases": []}
    for n, seed, iterations in CASES:
        xy = instances.uniform(n, seed)
        prep = oracle.prepare(xy, PARAMS["k"], PARAMS["b"], PARAMS["w"])
        kw = {k: v for k, v in PARAMS.items()}
        with ThreadPoolExecutor(8) as pool:
            lengths = list(pool.map(lambda s: oracle.ref_colony(xy, prep, iterations=iterations, seed=s, **kw)[1],
                                    SEEDS))
        out["cases"].append({"n": n, "instance_seed": seed, "iterations": iterations,
                             "initial_cost": int(prep["cost"]), "lengths": [int(v) for v in lengths]})
        print(n, seed, iterations, sum(lengths) / len(lengths), flush=True)
    (Path(__file__).parent / "ref_colony_lengths.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()

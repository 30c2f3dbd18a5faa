"""One launch each of the engine's auxiliary kernels on a realistic size, for
kernel profiles.

    python -m gplsaco_gb300.profile_kernels knn
        registration of one large clustered instance (N = 9,647 of the large
        workload, k=32 + backup 64 + LS 32): one knn_kernel launch (radix
        select + bitonic sort of every node's nearest 96 nodes);
    python -m gplsaco_gb300.profile_kernels score
        GP scoring of 128 random controller programs x 32 colonies each
        (4,096 colonies, 12 features x 32 actions): one score_kernel launch;
    python -m gplsaco_gb300.profile_kernels fingerprint
        one iteration of the GP evaluation batch's shape with the reference's
        12-feature controller (one N=500 instance, 128 programs, 32 ants):
        fingerprint_kernel launches (tour fingerprints, one warp per ant).
Each prints what it ran as one JSON line.
"""
from __future__ import annotations

import json
import sys
import time

import numpy as np

from . import instances
from .engine import FacoBatchEngine, FixedFacoSettings, score_cuda
from .programs import random_program


def knn() -> dict:
    xy = instances.large_clustered(1)[0]
    engine = FacoBatchEngine(len(xy), 1, FixedFacoSettings(ants=64, primary_width=32, backup_width=64, ls_width=32))
    t = time.perf_counter()
    info = engine.register_problem(1, xy.astype(np.float64))
    engine.close()
    return {"kernel": "knn_kernel", "n": len(xy), "rows": 32 + 64, "registration_s": time.perf_counter() - t,
            "initial_cost": int(info["initial_cost"])}


def score() -> dict:
    rng = np.random.default_rng(2)
    programs = [random_program(rng, extended=True) for _ in range(128)]
    colonies = 128 * 32
    features = rng.random((12, colonies, 32), dtype=np.float32)
    masks = np.full(colonies, 0xFFFFFFFF, np.uint32)
    res = score_cuda(programs, features, masks)
    return {"kernel": "score_kernel", "programs": 128, "colonies": colonies,
            "mean_action": float(np.mean(res["actions"]))}


def fingerprint() -> dict:
    rng = np.random.default_rng(2)
    programs = [random_program(rng, extended=True, features=12, feature_spec_id=2) for _ in range(128)]
    engine = FacoBatchEngine(500, 1, FixedFacoSettings(ants=32, retention=0.98), population_size=128)
    engine.register_problem(1, instances.uniform(500, 2).astype(np.float64))
    res = engine.evaluate_population_evaluations(np.ones(1, np.uint64), np.ones(1, np.uint64), 32 * 2, programs)
    engine.close()
    return {"kernel": "fingerprint_kernel", "colonies": 128, "ants": 32, "n": 500, "iterations": 2,
            "individuals": len(res)}


def main(argv=None) -> None:
    argv = sys.argv[1:] if argv is None else argv
    which = {"knn": knn, "score": score, "fingerprint": fingerprint}
    if len(argv) != 1 or argv[0] not in which:
        raise SystemExit("usage: python -m gplsaco_gb300.profile_kernels knn|score|fingerprint")
    print(json.dumps(which[argv[0]]()))


if __name__ == "__main__":
    main()

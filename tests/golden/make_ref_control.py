"""Generates tests/golden/ref_control.json: outputs of the reference's own
12-feature controller code (cpp/src/control_cpu.cpp and
cpp/include/gp_faco/control_ops.hpp, compiled unmodified into oracle/_ref by
oracle/build_ref.sh) on small seeded inputs -- tour fingerprints, sample
nodes, start regions, archive updates and whole action snapshots.

    python tests/golden/make_ref_control.py

Needs oracle/_ref (built where the reference sources are present).  The
inputs are stored beside the outputs, so the tests need only this file.
"""
from __future__ import annotations

import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import oracle  # noqa: E402

OUT = Path(__file__).with_name("ref_control.json")


def _tour_cost(m, t):
    return int(np.sum(m[t, np.roll(t, -1)].astype(np.int64)))


def variants(rng, tour, count, moves):
    """Tours a few random segment reversals away from `tour`, plus a rotated
    and a reversed copy of it (the same cycle written differently)."""
    out = [np.roll(tour, 7), tour[::-1].copy()]
    for _ in range(count):
        t = tour.copy()
        for _ in range(rng.integers(1, moves + 1)):
            i = int(rng.integers(0, t.size - 4))
            j = i + int(rng.integers(1, 4))
            t[i:j + 1] = t[i:j + 1][::-1]
        out.append(t)
    return out


def instance(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "grid":
        return rng.integers(0, 12, (n, 2)).astype(np.int32)
    return rng.integers(0, 10**4, (n, 2)).astype(np.int32)


def main() -> None:
    R = oracle.ref()
    if R is None:
        raise SystemExit("oracle/_ref is not built")
    rng = np.random.default_rng(2026)
    data = {"fingerprints": [], "samples": [], "regions": [], "archives": [], "snapshots": []}
    for n in (3, 4, 7, 50, 200):
        for _ in range(2):
            t = rng.permutation(n).astype(np.uint32)
            out = np.zeros(2, np.uint64)
            R.ref_fingerprint(t, n, out)
            data["fingerprints"].append({"tour": t.tolist(), "fp": [str(int(x)) for x in out]})
    for n, key in ((3, 1), (10, 2), (64, 3), (65, 4), (1000, 2**63 + 5)):
        out = np.zeros(min(n, 64), np.uint32)
        R.ref_sample_nodes(n, key, out)
        data["samples"].append({"n": n, "key": str(key), "nodes": out.tolist()})
    for n, k in ((5, 4), (16, 15), (17, 16), (60, 16)):
        xy = instance("uniform", n, n)
        prep = oracle.prepare(xy, k, 0, min(20, n - 1))
        t = prep["initial"]
        for mode in (0, 1):
            for region in range(4):
                key = int(rng.integers(0, 2**63))
                batch = int(rng.integers(0, 1000))
                out = np.zeros(16, np.uint32)
                R.ref_build_region(t, n, prep["primary"], k, key, batch, mode, region, out)
                data["regions"].append({"tour": t.tolist(), "primary": prep["primary"].tolist(), "key": str(key),
                                        "batch": batch, "mode": mode, "region": region,
                                        "nodes": out[:min(n, 16)].tolist()})
    for kind, n, seed in (("grid", 40, 1), ("uniform", 200, 2), ("grid", 25, 3), ("uniform", 400, 4)):
        xy = instance(kind, n, seed)
        m = oracle.euc2d_matrix(xy).astype(np.float64)
        prep = oracle.prepare(xy, min(16, n - 1), 0, min(20, n - 1))
        base = prep["initial"]
        entries = [base] + variants(rng, base, 4, 2)
        batch = variants(rng, base, 10, 3)
        costs = [_tour_cost(m.astype(np.int64), t) for t in batch]
        best = batch[int(np.argmin(costs))] if min(costs) < _tour_cost(m.astype(np.int64), base) else base
        ent = np.ascontiguousarray(np.stack(entries), dtype=np.uint32)
        bat = np.ascontiguousarray(np.stack(batch), dtype=np.uint32)
        out_t = np.zeros((4, n), np.uint32); out_c = np.zeros(4); out_i = np.zeros(8, np.uint64)
        count = C.c_uint32()
        rc = R.ref_archive_update(n, m, ent.reshape(-1), ent.shape[0], np.ascontiguousarray(best, np.uint32),
                                  bat.reshape(-1), bat.shape[0], out_t.reshape(-1), out_c, out_i, C.byref(count))
        assert rc == 0, rc
        c = count.value
        data["archives"].append({"xy": xy.tolist(), "entries": ent.tolist(), "global": best.tolist(),
                                 "batch": bat.tolist(), "tours": out_t[:c].tolist(),
                                 "costs": [int(x) for x in out_c[:c]], "ids": [str(int(x)) for x in out_i[:2 * c]]})
    for kind, n, seed, rounds in (("uniform", 17, 11, 3), ("grid", 40, 12, 5), ("uniform", 120, 13, 8),
                                  ("uniform", 9, 14, 0), ("uniform", 300, 15, 4), ("grid", 64, 16, 2),
                                  ("uniform", 300, 17, 6)):
        xy = instance(kind, n, seed)
        m = oracle.euc2d_matrix(xy).astype(np.float64)
        k = min(16, n - 1)
        prep = oracle.prepare(xy, k, 0, min(20, n - 1))
        base = prep["initial"]
        entries = [base] + variants(rng, base, 3, 1)
        active = variants(rng, base, 1, 2)[-1] if seed % 2 else entries[-1]
        parent = variants(rng, base, 1, 2)[-1]
        samples = np.zeros(min(n, 64), np.uint32)
        key = int(rng.integers(0, 2**63))
        R.ref_sample_nodes(n, key, samples)
        scale, eps = oracle.local_scale(xy)
        cost = _tour_cost(m.astype(np.int64), base)
        tmax = 1.0 / (cost * (1 - 0.98))
        tmin = tmax * 0.01
        feedback = [float(np.float32(rng.random())), float(np.float32(rng.random())), int(rng.integers(0, 40)),
                    int(rng.integers(0, 40)), int(rng.integers(0, 5))]
        solve_key = int(rng.integers(0, 2**63))
        batch_no = int(rng.integers(0, 500))
        elapsed = float(rng.random())
        mask = int(rng.integers(1, 2**32)) | 1
        ent = np.ascontiguousarray(np.stack(entries), dtype=np.uint32)
        features = np.zeros((12, 32), np.float32)
        regions = np.zeros((2, 4, 16), np.uint32)
        alt, legal = C.c_uint32(), C.c_uint32()
        trails = np.zeros((n, k)); dflt = C.c_double()
        rc = R.ref_action_snapshot(n, m, np.ascontiguousarray(prep["primary"], np.uint32), k, samples, samples.size,
                                   scale, eps, np.ascontiguousarray(active, np.uint32), ent.reshape(-1),
                                   ent.shape[0], np.asarray(feedback, np.float64),
                                   np.ascontiguousarray(parent, np.uint32), tmax, 0.98, tmin, tmax, 1.0 / cost,
                                   rounds, elapsed, solve_key, batch_no, mask, features.reshape(-1),
                                   regions.reshape(-1), C.byref(alt), C.byref(legal), trails.reshape(-1),
                                   C.byref(dflt))
        assert rc == 0, rc
        data["snapshots"].append({
            "xy": xy.tolist(), "primary": prep["primary"].tolist(), "samples": samples.tolist(),
            "entries": ent.tolist(), "active": np.asarray(active).tolist(), "feedback": feedback,
            "trails": trails.tolist(), "default_trail": dflt.value, "tau_min": tmin, "tau_max": tmax,
            "elapsed": elapsed, "solve_key": str(solve_key), "batch": batch_no, "mask": mask,
            "features": features.view(np.uint32).tolist(), "regions": regions.tolist(),
            "alternative": alt.value, "legal": legal.value})
    OUT.write_text(json.dumps(data, separators=(",", ":")))
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    main()

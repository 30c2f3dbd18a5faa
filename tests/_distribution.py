"""Final-length distributions against the reference's CPU core
(tests/golden/ref_colony_lengths.json, made by
tests/golden/make_ref_distribution.py): 100 seeds per case on each side, so
that a mean difference of 0.1% is resolved (the reference's own spread is
0.09-0.21% of the mean per run, a standard error of the difference of about
0.03% at 100 seeds)."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

FIXTURE = Path(__file__).parent / "golden" / "ref_colony_lengths.json"
MEAN_TOLERANCE = 1e-3      # mean within 0.1%
P_MIN = 0.05               # two-sided Mann-Whitney


def load() -> dict:
    return json.loads(FIXTURE.read_text())


def compare(reference, ours) -> dict:
    from scipy.stats import mannwhitneyu
    r, o = np.asarray(reference, np.float64), np.asarray(ours, np.float64)
    diff = (o.mean() - r.mean()) / r.mean()
    se = np.sqrt(r.var(ddof=1) / r.size + o.var(ddof=1) / o.size) / r.mean()
    p = float(mannwhitneyu(r, o, alternative="two-sided").pvalue) if np.any(r != o) else 1.0
    return {"mean_diff": float(diff), "se": float(se), "p": p,
            "ok": abs(diff) <= MEAN_TOLERANCE and p > P_MIN}

"""The oracle's whole colony runs (Philox draws) against the reference's own
CPU core (std::mt19937_64 draws): final-length distributions over 100 seeds
agree (mean within 0.1% and two-sided Mann-Whitney p > 0.05)."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from gplsaco_gb300 import instances
from tests import _distribution

pytest.importorskip("scipy")


@pytest.mark.parametrize("case", range(len(_distribution.load()["cases"])))
def test_oracle_lengths_match_reference_distribution(oracle, case):
    fx = _distribution.load()
    c, p = fx["cases"][case], fx["params"]
    xy = instances.uniform(c["n"], c["instance_seed"])
    prep = oracle.prepare(xy, p["k"], p["b"], p["w"])
    assert int(prep["cost"]) == c["initial_cost"]

    def run(seed):
        return oracle.run_colony(xy, prep, ants=p["ants"], k=p["k"], b=p["b"], w=p["w"], mne=p["mne"],
                                 iterations=c["iterations"], key=oracle.lib().orc_colony_key(seed, 1),
                                 retention=p["retention"], p_best=p["p_best"],
                                 epoch_source_probability=p["epoch_source_probability"], want_trace=False)["cost"]

    with ThreadPoolExecutor(8) as pool:
        ours = list(pool.map(run, fx["seeds"]))
    res = _distribution.compare(c["lengths"], ours)
    assert res["ok"], res

"""End to end against the reference's own CPU core: the engine's
final-length distributions on uniform N=100/500/1000 instances agree with
the reference's (tests/golden/ref_colony_lengths.json, 100 seeds per case):
mean within 0.1% and two-sided Mann-Whitney p > 0.05.  Runs through the C
ABI (faco_evaluate)."""
import numpy as np
import pytest

from gplsaco_gb300 import instances
from tests import _distribution

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api(engine_lib):
    pytest.importorskip("scipy")
    import gplsaco_gb300 as g
    return g


@pytest.mark.parametrize("case", range(len(_distribution.load()["cases"])))
def test_engine_lengths_match_reference_distribution(api, case):
    fx = _distribution.load()
    c, p = fx["cases"][case], fx["params"]
    settings = api.FixedFacoSettings(ants=p["ants"], primary_width=p["k"], backup_width=p["b"], ls_width=p["w"],
                                     retention=p["retention"], p_best=p["p_best"],
                                     epoch_source_probability=p["epoch_source_probability"])
    seeds = np.asarray(fx["seeds"], np.uint64)
    engine = api.FacoBatchEngine(c["n"], seeds.size, settings)
    reg = engine.register_problem(1, instances.uniform(c["n"], c["instance_seed"]).astype(np.float64))
    assert reg["initial_cost"] == c["initial_cost"]
    res = engine.evaluate_faco_evaluations(np.ones(seeds.size, np.uint64), seeds, p["ants"] * c["iterations"],
                                           p["mne"])
    engine.close()
    ours = [it["cost"] for it in res["items"]]
    out = _distribution.compare(c["lengths"], ours)
    assert out["ok"], out

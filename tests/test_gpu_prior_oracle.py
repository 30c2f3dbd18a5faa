"""The learned prior's application on the GPU, bit for bit against the CPU
restatement (oracle/faco_oracle.c: orc_prior_eta, orc_departure_rows,
orc_run_colony_prior), and what a trained prior gains over plain FACO.

The network's probabilities come from the engine's own tensor-core forward
(faco_mlp_forward) over the engine's own candidate-edge features
(faco_edge_data) of the same colony state -- the forward and the features are
checked against their oracles in test_gpu_prior.py.  Everything after the
probability is exact FP32 arithmetic, so the heuristic rows, the products and
whole prior-enabled colony runs (tours, lengths, every trace row) must equal
the oracle's.  The reference has no learned prior; the rule it changes is
initialize_products (cuda/colony_state.cuh:91-110) and
SparsePheromone::product_cache (cpp/src/faco_cpu.cpp:351-363)."""
import numpy as np
import pytest

from tests import _cases

pytestmark = pytest.mark.gpu

TRACE_FIELDS = ("iteration_best_cost", "global_cost", "parent_cost", "iteration_best", "source_is_epoch",
                "construction_steps", "ls_evaluations")


@pytest.fixture(scope="module")
def api(engine_lib):
    import gplsaco_gb300 as g
    from gplsaco_gb300 import prior
    return g, prior


def _probabilities(prior, engine, params, sizes, k):
    """The network's probability of every candidate entry of every colony
    at the engine's current state, split per colony ([n, k] each)."""
    x, _ = engine.edge_data(features=True, labels=False)
    p = prior.forward(params, x)
    out, o = [], 0
    for n in sizes:
        out.append(p[o:o + n * k].reshape(n, k))
        o += n * k
    assert o == p.size
    return out


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("gamma,floor,departures", [(1, 0.2, False), (2, 0.05, False), (2, 0.05, True)])
def test_prior_rows_match_oracle(api, oracle, gamma, floor, departures):
    """eta' = eta (floor + p)^gamma on enabled colonies, the instance's eta on
    the others; products = trail * eta' (or the departure rule); the same
    after a refresh mid-run and after the fallback disables a colony."""
    g, prior = api
    n, k, ants = 300, 16, 8
    xy = _cases.uniform_instance(n, seed=31)
    engine = g.FacoBatchEngine(n, 3, g.FixedFacoSettings(ants=ants, retention=0.9))
    engine.register_problem(5, xy.astype(np.float64))
    rows = engine.problem_rows(5)
    primary = rows["primary"]
    eta = oracle.heuristic(xy, primary)
    params = prior.init_params(seed=11)
    enabled = np.array([1, 0, 1], np.uint8)
    engine.begin(np.full(3, 5, np.uint64), np.array([1, 2, 3], np.uint64), 8)

    def check(probs, enabled):
        for c in range(3):
            got = engine.colony_rows(c)
            want_eta = oracle.prior_eta(eta, probs[c], floor, gamma) if enabled[c] else eta
            assert np.array_equal(_bits(got["eta"]), _bits(want_eta)), c
            if enabled[c] and departures:
                # before the first batch every colony's parent is the initial tour
                want = oracle.departure_rows(primary, rows["initial_tour"], got["trails"], eta, want_eta)
            else:
                want = (got["trails"] * want_eta).astype(np.float32)
            assert np.array_equal(_bits(got["products"]), _bits(want)), c

    probs = _probabilities(prior, engine, params, [n] * 3, k)
    engine.prior_set(params, enabled, floor, gamma, departures)
    check(probs, enabled)
    # trails and best tours move; the refresh recomputes from the new state
    # (the departure rule then follows the new parent tours, so only the
    # plain-total rows are compared after steps)
    if not departures:
        engine.step(4)
        probs = _probabilities(prior, engine, params, [n] * 3, k)
        engine.prior_refresh()
        check(probs, enabled)
        # fallback: colony 2 back to plain FACO, the others re-applied
        enabled = np.array([1, 0, 0], np.uint8)
        probs = _probabilities(prior, engine, params, [n] * 3, k)
        engine.prior_set(None, enabled, floor, gamma, departures)
        check(probs, enabled)
    engine.finish()
    engine.close()


@pytest.mark.parametrize("n,gamma,floor,departures,ls_mode", [(200, 2, 0.05, False, 0), (200, 1, 0.5, True, 0),
                                                               (537, 2, 0.05, False, 1), (1000, 2, 0.2, True, 0),
                                                               (2300, 2, 0.05, True, 0)])
def test_prior_colony_runs_match_oracle(api, oracle, n, gamma, floor, departures, ls_mode):
    """Whole prior-enabled colony runs: the colonies with the prior (and the
    one without, in the same evaluation) give the oracle's tours, lengths
    and every iteration's trace row bit for bit; so does a run whose prior
    is refreshed mid-run and then disabled by the per-instance fallback.
    At N=2300 the trail update and departure rows run in several blocks
    per colony."""
    g, prior = api
    k, ants, iterations = 16, 8, 14
    xy = _cases.uniform_instance(n, seed=40 + n)
    settings = g.FixedFacoSettings(ants=ants, retention=0.98, ls_mode=ls_mode)
    engine = g.FacoBatchEngine(n, 3, settings)
    key = 77
    engine.register_problem(key, xy.astype(np.float64))
    prep = oracle.prepare(xy, k, 64, 20)
    assert np.array_equal(engine.problem_rows(key)["primary"], prep["primary"])
    eta = oracle.heuristic(xy, prep["primary"])
    params = prior.init_params(seed=n)
    seeds = np.array([3, 4, 5], np.uint64)
    enabled = np.array([1, 0, 1], np.uint8)
    refresh_at, fallback_at = 5, 9
    engine.begin(np.full(3, key, np.uint64), seeds, 8, trace_iterations=iterations)
    schedules = [[] for _ in range(3)]

    def record(at, probs, enabled):
        for c in range(3):
            e = oracle.prior_eta(eta, probs[c], floor, gamma) if enabled[c] else eta
            schedules[c].append((at, e, bool(enabled[c]) and departures))

    probs = _probabilities(prior, engine, params, [n] * 3, k)
    engine.prior_set(params, enabled, floor, gamma, departures)
    record(0, probs, enabled)
    engine.step(refresh_at)
    probs = _probabilities(prior, engine, params, [n] * 3, k)
    engine.prior_refresh()
    record(refresh_at, probs, enabled)
    engine.step(fallback_at - refresh_at)
    enabled = np.array([1, 0, 0], np.uint8)
    probs = _probabilities(prior, engine, params, [n] * 3, k)
    engine.prior_set(None, enabled, floor, gamma, departures)
    record(fallback_at, probs, enabled)
    engine.step(iterations - fallback_at)
    res = engine.finish()
    m = oracle.euc2d_matrix(xy)
    for c in range(3):
        ref = oracle.run_colony(xy, prep, ants=ants, k=k, b=64, w=20, mne=8, iterations=iterations,
                                key=oracle.lib().orc_colony_key(int(seeds[c]), key), retention=0.98,
                                ls_mode=ls_mode, prior=schedules[c])
        tour = np.asarray(res["tours"][c], np.int64)
        assert int(res["costs"][c]) == ref["cost"], c
        assert np.array_equal(tour, ref["tour"]), c
        assert int(np.sum(m[tour, np.roll(tour, -1)])) == ref["cost"]
        for it in range(iterations):
            row, want = res["trace"][it, c], ref["trace"][it]
            for field in TRACE_FIELDS:
                assert int(row[field]) == int(want[field]), (c, it, field)
            assert row["tau_min"] == np.float32(want["tau_min"]) and row["tau_max"] == np.float32(want["tau_max"])
    engine.close()

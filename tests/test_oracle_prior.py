"""The learned prior's application, restated on the CPU (oracle/faco_oracle.c:
orc_prior_eta, orc_departure_rows, orc_run_colony_prior).

The reference has no learned prior: it reweights the heuristic of
initialize_products (cuda/colony_state.cuh:91-110) and of
SparsePheromone::product_cache (cpp/src/faco_cpu.cpp:351-363).  So the C
restatement is pinned here by an independent numpy restatement of the same
FP32 arithmetic and by properties: a schedule that hands back the instance's
own heuristic is plain FACO bit for bit (with and without the departure
rule), the departure rule keeps the parent-tour entries and the plain total
weight per node, and a reweighted colony still yields valid tours with exact
lengths."""
import numpy as np
import pytest

from tests import _cases


def _numpy_prior_eta(eta, prob, floor, gamma):
    f = (np.float32(floor) + prob.astype(np.float32)).astype(np.float32)
    factor = (f * f).astype(np.float32) if gamma == 2 else f
    return (eta.astype(np.float32) * factor).astype(np.float32)


def _numpy_departure_rows(primary, parent, trails, eta, prior):
    n, k = primary.shape
    pos = np.empty(n, np.int64)
    pos[parent] = np.arange(n)
    succ = parent[(pos + 1) % n]
    pred = parent[(pos - 1) % n]
    out = np.zeros((n, k), np.float32)
    for i in range(n):
        on = (primary[i] == succ[i]) | (primary[i] == pred[i])
        plain = np.float32(0.0)
        total = np.float32(0.0)
        for j in range(k):             # sequential FP32 sums in candidate order
            if on[j]:
                continue
            plain = np.float32(plain + np.float32(trails[i, j] * eta[i, j]))
            total = np.float32(total + np.float32(trails[i, j] * prior[i, j]))
        scale = np.float32(plain / total) if total > 0 else np.float32(1.0)
        for j in range(k):
            t = trails[i, j]
            out[i, j] = np.float32(t * eta[i, j]) if on[j] else np.float32(np.float32(t * prior[i, j]) * scale)
    return out


@pytest.mark.parametrize("gamma", [1, 2])
@pytest.mark.parametrize("floor", [0.05, 0.5])
def test_prior_eta_matches_numpy(oracle, gamma, floor):
    rng = np.random.default_rng(gamma * 10 + int(floor * 100))
    eta = rng.uniform(1e-7, 1e-3, (300, 16)).astype(np.float32)
    prob = rng.random((300, 16), dtype=np.float32)
    prob[0, :4] = [0.0, 1.0, 0.5, np.float32(1e-30)]
    got = oracle.prior_eta(eta, prob, floor, gamma)
    want = _numpy_prior_eta(eta, prob, floor, gamma)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.all(got > 0)        # never removes a candidate


def test_departure_rows_match_numpy_and_keep_totals(oracle):
    n, k = 120, 12
    xy = _cases.uniform_instance(n, seed=3)
    prep = oracle.prepare(xy, k, 0, min(20, n - 1))
    primary = prep["primary"]
    rng = np.random.default_rng(4)
    parent = rng.permutation(n).astype(np.uint32)
    trails = rng.uniform(1e-7, 1e-5, (n, k)).astype(np.float32)
    eta = oracle.heuristic(xy, primary)
    prior = oracle.prior_eta(eta, rng.random((n, k), dtype=np.float32), 0.05, 2)
    got = oracle.departure_rows(primary, parent, trails, eta, prior)
    want = _numpy_departure_rows(primary, parent, trails, eta, prior)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    pos = np.empty(n, np.int64)
    pos[parent] = np.arange(n)
    succ, pred = parent[(pos + 1) % n], parent[(pos - 1) % n]
    on = (primary == succ[:, None]) | (primary == pred[:, None])
    plain = (trails * eta).astype(np.float32)
    assert np.array_equal(got[on], plain[on])
    off_total = np.where(on, 0.0, got.astype(np.float64)).sum(axis=1)
    plain_total = np.where(on, 0.0, plain.astype(np.float64)).sum(axis=1)
    assert np.allclose(off_total, plain_total, rtol=1e-5)
    # the prior only re-ranks: with the plain heuristic as the prior it is the plain product
    same = oracle.departure_rows(primary, parent, trails, eta, eta)
    assert np.array_equal(same, plain)


@pytest.mark.parametrize("departures", [False, True])
def test_plain_heuristic_schedule_is_plain_faco(oracle, departures):
    """A schedule that applies the instance's own heuristic (at the start and
    again mid-run) leaves the colony run unchanged bit for bit."""
    n, k, ants, iterations = 150, 16, 8, 12
    xy = _cases.uniform_instance(n, seed=8)
    prep = oracle.prepare(xy, k, 64, 20)
    key = oracle.lib().orc_colony_key(3, 1)
    plain = oracle.run_colony(xy, prep, ants=ants, k=k, b=64, w=20, mne=8, iterations=iterations, key=key)
    eta = oracle.heuristic(xy, prep["primary"])
    sched = [(0, eta, departures), (5, eta, departures)]
    got = oracle.run_colony(xy, prep, ants=ants, k=k, b=64, w=20, mne=8, iterations=iterations, key=key,
                            prior=sched)
    assert got["cost"] == plain["cost"] and np.array_equal(got["tour"], plain["tour"])
    assert got["trace"] == plain["trace"]
    assert np.array_equal(got["products"], plain["products"])


@pytest.mark.parametrize("departures", [False, True])
def test_reweighted_colony_is_valid_and_changes_the_walk(oracle, departures):
    n, k, ants, iterations = 200, 16, 8, 15
    xy = _cases.uniform_instance(n, seed=9)
    prep = oracle.prepare(xy, k, 64, 20)
    key = oracle.lib().orc_colony_key(5, 2)
    eta = oracle.heuristic(xy, prep["primary"])
    rng = np.random.default_rng(10)
    prob = rng.random((n, k), dtype=np.float32)
    sched = [(0, oracle.prior_eta(eta, prob, 0.05, 2), departures), (7, eta, False)]
    plain = oracle.run_colony(xy, prep, ants=ants, k=k, b=64, w=20, mne=8, iterations=iterations, key=key)
    got = oracle.run_colony(xy, prep, ants=ants, k=k, b=64, w=20, mne=8, iterations=iterations, key=key,
                            prior=sched)
    again = oracle.run_colony(xy, prep, ants=ants, k=k, b=64, w=20, mne=8, iterations=iterations, key=key,
                              prior=sched)
    t = got["tour"].astype(np.int64)
    assert np.array_equal(np.sort(t), np.arange(n))
    m = oracle.euc2d_matrix(xy)
    assert int(np.sum(m[t, np.roll(t, -1)])) == got["cost"]
    assert got["trace"] == again["trace"] and got["cost"] == again["cost"]
    assert got["trace"][:7] != plain["trace"][:7]     # a random prior changes the first batches' walks
    # from batch 7 on the heuristic is plain again: the products are trail * eta
    assert np.array_equal(got["products"], (got["trails"] * eta).astype(np.float32))


def test_schedule_order_is_checked(oracle):
    n = 50
    xy = _cases.uniform_instance(n, seed=1)
    prep = oracle.prepare(xy, 16, 16, 20)
    eta = oracle.heuristic(xy, prep["primary"])
    with pytest.raises(ValueError):
        oracle.run_colony(xy, prep, ants=4, k=16, b=16, w=20, mne=8, iterations=3, key=1,
                          prior=[(2, eta, False), (1, eta, False)])

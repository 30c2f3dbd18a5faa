"""CUDA engine vs the CPU oracle, through the C ABI.  Integer/index work is
compared bit-for-bit; FP32 trails against the FP64 reference arithmetic
within 1e-6 relative."""
import ctypes as C

import numpy as np
import pytest

from tests import _cases, _programs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api(engine_lib):
    import gplsaco_gb300 as g
    return g


def _oracle_ant_case(oracle, xy, ordered, tour, target, cap, **kw):
    return oracle.ant(tour, ordered, int(target), cap, xy=xy, **kw)


def _compare_ant(gpu, t, ref, ctx):
    assert np.array_equal(gpu["construction_tours"][t], ref["construction_tour"]), ctx
    assert gpu["construction_costs"][t] == ref["construction_cost"], ctx
    assert np.array_equal(gpu["tours"][t], ref["tour"]), ctx
    assert np.array_equal(gpu["positions"][t], ref["positions"]), ctx
    c = gpu["counters"][t]
    got = tuple(int(x) for x in c)
    want = (ref["mne"], ref["steps"], ref["nonidentity"], ref["processed"], ref["checks"], ref["evaluations"],
            ref["accepted"], ref["reactivations"], ref["limit_reached"], len(ref["checklist"]))
    assert got == want, ctx
    assert np.array_equal(gpu["checklists"][t][:len(ref["checklist"])], ref["checklist"]), ctx
    assert gpu["final_costs"][t] == ref["final_cost"], ctx


@pytest.mark.parametrize("n", _cases.N_GRID)
@pytest.mark.parametrize("metric", [0, 1, 2])
@pytest.mark.parametrize("ls_mode", [0, 1])
def test_explicit_choice_construction_and_ls(api, oracle, n, metric, ls_mode):
    """Identical construction tour, LS tour, positions, checklist order and
    work counters for explicit visit orders (tests/cpp/test_cuda_faco.cpp:31-104);
    ls_mode 0 is the reference's best-gain 2-opt, 1 the 2-opt + Or-opt
    first-improvement variant."""
    xy = _cases.coordinates(n, metric, seed=83741 + n + metric * 1117)
    matrix = oracle.euc2d_matrix(xy)
    width = min(20, n - 1)
    rows = _cases.ls_rows(matrix, width, reverse=metric == 0)
    ordered = oracle.distance_ordered(rows, matrix)
    ants = 16
    tours, visits, targets = _cases.ant_tasks(n, ants, seed=n * 31 + metric)
    for cap in _cases.CAPS:
        gpu = api.ant_diagnostic(xy, rows, tours, targets, cap, visits=visits, ls_mode=ls_mode)
        for t in range(ants):
            ref = _oracle_ant_case(oracle, xy, ordered, tours[t], targets[t], cap, visit=visits[t],
                                   ls_mode=ls_mode)
            _compare_ant(gpu, t, ref, f"n={n} metric={metric} cap={cap} ant={t} ls_mode={ls_mode}")


def test_identity_two_opt_golden(api):
    """A 3-node cycle has no real 2-opt move (tests/cpp/test_cuda_faco.cpp:106-125)."""
    xy = np.array([[0, 0], [25, 0], [10, 27]], np.int32)
    rows = np.array([[1, 2], [2, 0], [1, 0]], np.uint32)
    ident = np.arange(3, dtype=np.uint32)
    gpu = api.ant_diagnostic(xy, rows, ident[None], [2], 1000, visits=ident[None])
    assert int(gpu["counters"][0][6]) == 0
    assert np.array_equal(gpu["tours"][0], ident)


@pytest.mark.parametrize("n,k,b", [(7, 2, 1), (17, 16, 0), (100, 16, 64), (100, 2, 1), (500, 16, 64),
                                   (1000, 16, 64), (1000, 2, 1)])
def test_injected_uniform_roulette(api, oracle, n, k, b):
    """Given a stream of uniforms, construction picks bit-identical nodes,
    including zero-weight, backup and global fallbacks (tests/cpp/test_fixed_faco.cpp:236-249)."""
    rng = np.random.default_rng(4703 + n + k)
    xy = _cases.uniform_instance(n, seed=n + 8999)
    b = min(b, n - 1 - k)
    prep = oracle.prepare(xy, k, b, min(20, n - 1))
    products = rng.random((n, k), dtype=np.float32) * np.float32(1e-3)
    products[rng.random((n, k)) < 0.1] = 0.0
    products[rng.random(n) < 0.05] = 0.0          # whole rows of zero weight
    ants = 16
    tours = np.stack([rng.permutation(n) for _ in range(ants)]).astype(np.uint32)
    uniforms = rng.random((ants, n))
    starts = rng.integers(0, n, ants).astype(np.uint32)
    targets = np.full(ants, 16, np.uint32)
    gpu = api.ant_diagnostic(xy, prep["ls"], tours, targets, 5000, uniforms=uniforms, starts=starts,
                             primary=prep["primary"], products=products, backup=prep["backup"] if b else None)
    for t in range(ants):
        ref = oracle.ant(tours[t], prep["ls"], 16, 5000, xy=xy, uniforms=uniforms[t], start=int(starts[t]),
                         primary=prep["primary"], products32=products, backup=prep["backup"] if b else None)
        steps = ref["steps"]
        assert np.array_equal(gpu["selected"][t][:steps + 1], ref["selected"]), f"n={n} ant={t}"
        _compare_ant(gpu, t, ref, f"n={n} k={k} b={b} ant={t}")


def test_pheromone_step(api, oracle):
    rng = np.random.default_rng(11)
    n, k = 1000, 16
    xy = _cases.uniform_instance(n, seed=3)
    prep = oracle.prepare(xy, k, 0, 20)
    primary = prep["primary"]
    eta = (1.0 / np.maximum(1, oracle.euc2d_matrix(xy)[np.arange(n)[:, None], primary])).astype(np.float32)
    for retention in (0.25, 0.5, 0.98):
        tmin, tmax = np.float32(1e-7), np.float32(2e-6)
        trails = rng.uniform(float(tmin), float(tmax), (n, k)).astype(np.float32)
        parent = rng.permutation(n).astype(np.uint32)
        inc = np.float32(1.0 / 7.3e7)
        got_t, got_p = api.pheromone_step(primary, parent, trails, eta, retention=float(np.float32(retention)),
                                          minimum=float(tmin), maximum=float(tmax), increment=float(inc))
        ref_t = trails.reshape(-1).copy(); ref_p = np.zeros(n * k, np.float32); d = C.c_float(tmax)
        oracle.lib().orc_pheromone32(n, k, primary, parent, np.float32(retention), tmin, tmax, inc,
                                     eta.reshape(-1), ref_t, ref_p, C.byref(d))
        assert np.array_equal(got_t.reshape(-1), ref_t) and np.array_equal(got_p.reshape(-1), ref_p)
        # FP32 engine trails vs FP64 reference arithmetic: 1e-6 relative
        t64 = trails.astype(np.float64).reshape(-1); d64 = C.c_double(float(tmax))
        oracle.lib().orc_pheromone64(n, k, primary, parent, retention, float(tmin), float(tmax), float(inc), t64,
                                     C.byref(d64))
        assert np.max(np.abs(got_t.reshape(-1) - t64) / t64) <= 1e-6


def test_scores_reference_and_extended(api, oracle):
    rng = np.random.default_rng(6677)
    features = rng.random((12, 7, 32), dtype=np.float32)
    masks = rng.integers(1, 0xFFFFFFFF, size=7, dtype=np.uint32)
    masks[:3] = [1, 1 << 31, 0xFFFFFFFF]
    for extended in (False, True):
        for _ in range(128):
            program = _programs.random_program(rng, extended=extended)
            got = api.score_cuda(program, features, masks)
            ref_scores, ref_actions = oracle.score(program, features, masks)
            assert np.array_equal(got["scores"], ref_scores)
            assert np.array_equal(got["actions"], ref_actions)
    zeros = np.zeros((12, 3, 32), np.float32)
    program = dict(ir_version=1, numeric_spec_id=1, feature_spec_id=1, opcode=[0], operand=[4], constant_bits=[])
    got = api.score_cuda(program, zeros, np.array([0xFFFFFFFF, 1 << 31, 1 << 7], np.uint32))
    assert got["actions"].tolist() == [0, 31, 7]


def _settings(api, ants, k=16, b=64, w=20, retention=0.98, epoch=0.01, ls_limit=100000, ls_mode=0, workspace=0,
              follow=0):
    return api.FixedFacoSettings(ants=ants, primary_width=k, backup_width=b, ls_width=w, retention=retention,
                                 epoch_source_probability=epoch, ls_evaluation_limit=ls_limit, ls_mode=ls_mode,
                                 workspace=workspace, follow=follow)


@pytest.mark.parametrize("n,ants,iterations,variant,ls_mode,workspace", [
    (7, 4, 8, 0, 0, 0), (17, 8, 8, 1, 0, 0), (100, 32, 20, 2, 0, 0), (500, 16, 6, 3, 0, 0), (1000, 32, 4, 0, 0, 0),
    (17, 8, 8, 1, 1, 0), (100, 32, 20, 2, 1, 0), (1000, 32, 4, 0, 1, 0),
    (7, 4, 8, 0, 0, 2), (100, 32, 20, 2, 0, 2), (500, 16, 6, 3, 1, 2), (1000, 32, 4, 0, 0, 2),
    (1000, 16, 40, 3, 0, 0), (2600, 8, 3, 3, 0, 0), (2600, 8, 3, 1, 1, 2), (2600, 8, 4, 0, 0, 0),
    (2600, 8, 4, 2, 1, 2)])
@pytest.mark.parametrize("follow", [1, 2])
def test_engine_run_matches_oracle(api, oracle, n, ants, iterations, variant, ls_mode, workspace, follow):
    """Whole plain-FACO runs: registration rows and initial tour, every
    iteration's best/global/parent costs and trail bounds, the final global
    tour and the FP32 trails agree bit-for-bit with the oracle -- with the
    ants' tours in shared memory and in the global-memory workspace, and
    with the relocations deferred into runs (long walks once trails
    converge; every relocation above 2048 nodes), with the steps along
    the parent tour taken one at a time and in batches (follow 1 / 2), and
    with the trail update of a large matrix (N=2600, k=16) spread over
    several blocks per colony."""
    k = 2 if variant % 2 else 16
    b = 1 if variant % 2 else 64
    retention = (0.25, 0.5, 0.75, 0.98)[variant]
    epoch = (0.0, 0.01, 1.0, 0.3)[variant]
    xy = _cases.uniform_instance(n, seed=4703 + n)
    settings = _settings(api, ants, k, b, 20, retention, epoch, 5000, ls_mode, workspace, follow)
    engine = api.FacoBatchEngine(n, 3, settings)
    info = engine.register_problem(n + 8999, xy.astype(np.float64))
    kk, bb, ww = min(k, n - 1), min(b, n - 1 - min(k, n - 1)), min(20, n - 1)
    prep = oracle.prepare(xy, kk, bb, ww)
    rows = engine.problem_rows(n + 8999)
    assert np.array_equal(rows["primary"], prep["primary"]) and np.array_equal(rows["backup"], prep["backup"])
    assert np.array_equal(rows["ls"], prep["ls"]) and np.array_equal(rows["initial_tour"], prep["initial"])
    assert info["initial_cost"] == prep["cost"]
    seeds = np.array([17, 29, 17], np.uint64)
    keys = np.full(3, n + 8999, np.uint64)
    res = engine.evaluate_faco_evaluations(keys, seeds, ants * iterations, 8, trace=True)
    assert res["completed_tour_evaluations_per_colony"] == ants * iterations
    for c in range(3):
        key = oracle.lib().orc_colony_key(int(seeds[c]), n + 8999)
        ref = oracle.run_colony(xy, prep, ants=ants, k=kk, b=bb, w=ww, mne=8, iterations=iterations, key=key,
                                retention=retention, epoch_source_probability=epoch, ls_limit=5000,
                                ls_mode=ls_mode)
        assert res["items"][c]["cost"] == ref["cost"]
        assert res["items"][c]["tour"] == ref["tour"].tolist()
        for it in range(iterations):
            row, want = res["trace"][it, c], ref["trace"][it]
            for field in ("iteration_best_cost", "global_cost", "parent_cost", "iteration_best", "source_is_epoch",
                          "construction_steps", "ls_evaluations"):
                assert int(row[field]) == int(want[field]), (c, it, field)
            assert row["tau_min"] == np.float32(want["tau_min"]) and row["tau_max"] == np.float32(want["tau_max"])
    # same seed, same instance -> same result (colonies 0 and 2)
    assert res["items"][0]["tour"] == res["items"][2]["tour"]
    engine.close()


@pytest.mark.parametrize("workspace", [0, 2])
def test_uneven_batch_matches_independent_runs(api, oracle, workspace):
    """Instances of different sizes share one evaluation; each colony equals
    its own oracle run (tests/cpp/test_batch_engine.cpp:39-88)."""
    sizes = [200, 537, 1000, 311]
    ants, iterations = 16, 5
    settings = _settings(api, ants, workspace=workspace)
    engine = api.FacoBatchEngine(1000, 8, settings)
    preps = {}
    for i, n in enumerate(sizes):
        xy = _cases.uniform_instance(n, seed=100 + i)
        engine.register_problem(1000 + i, xy.astype(np.float64))
        preps[1000 + i] = (xy, oracle.prepare(xy, 16, 64, 20))
    keys = np.array([1003, 1000, 1002, 1001, 1002], np.uint64)
    seeds = np.array([5, 6, 7, 8, 9], np.uint64)
    res = engine.evaluate_faco_evaluations(keys, seeds, ants * iterations, 8)
    for c in range(keys.size):
        xy, prep = preps[int(keys[c])]
        key = oracle.lib().orc_colony_key(int(seeds[c]), int(keys[c]))
        ref = oracle.run_colony(xy, prep, ants=ants, k=16, b=64, w=20, mne=8, iterations=iterations, key=key)
        assert res["items"][c]["cost"] == ref["cost"], c
        assert res["items"][c]["tour"] == ref["tour"].tolist(), c
    engine.close()


def test_full_size_invariants(api, oracle):
    """N=1000, 64 colonies x 32 ants: every global tour is a permutation whose
    recomputed EUC_2D length equals the reported one; global costs never
    increase; FE accounting is ants x iterations; checkpoints are prefixes."""
    n, colonies, ants, iterations = 1000, 64, 32, 12
    engine = api.FacoBatchEngine(n, colonies, _settings(api, ants))
    xys = []
    for i in range(4):
        xy = _cases.uniform_instance(n, seed=1 + i)
        xys.append(xy)
        engine.register_problem(i + 1, xy.astype(np.float64))
    keys = np.array([1 + (c % 4) for c in range(colonies)], np.uint64)
    seeds = np.arange(colonies, dtype=np.uint64)
    res = engine.evaluate_faco_evaluations(keys, seeds, ants * iterations, 8, checkpoint_iterations=[0, 5, 12],
                                           trace=True)
    assert res["total_tour_evaluations"] == colonies * ants * iterations
    for c in range(colonies):
        tour = np.array(res["items"][c]["tour"], np.uint32)
        assert np.array_equal(np.sort(tour), np.arange(n))
        m = xys[c % 4]
        length = int(np.sum(oracle.euc2d_matrix(m)[tour, np.roll(tour, -1)]))
        assert length == res["items"][c]["cost"]
        g = res["trace"]["global_cost"][:, c]
        assert np.all(np.diff(g) <= 0)
    assert res["checkpoints"][-1]["tours"] == [item["tour"] for item in res["items"]]
    engine.close()


@pytest.mark.parametrize("limit", [1, 2, 19, 20, 21, 39, 40, 41, 1000])
def test_ls_evaluation_limit_boundaries_with_ties(api, oracle, limit):
    """The warp 2-opt stops at exactly the LS evaluation budget, with equal
    lengths and coincident points (zero gains, ties by node order) on a 12x12
    grid -- plain and GP-controlled colonies equal the oracle's serial scan
    (tests/python/test_parallel_ls_cuda.py:15-38); checkpoint lists that
    repeat, decrease or pass the budget are refused (test_v2_cuda.py:34-36)."""
    n, ants, iterations = 67, 8, 12
    xy = np.random.default_rng(420).integers(0, 12, (n, 2)).astype(np.int32)
    settings = _settings(api, ants, ls_limit=limit, retention=0.9)
    program = _programs.random_program(np.random.default_rng(limit), features=10, feature_spec_id=3)
    engine = api.FacoBatchEngine(n, 2, settings, population_size=2)
    engine.register_problem(312, xy.astype(np.float64))
    prep = oracle.prepare(xy, 16, 50, 20)
    keys = np.full(2, 312, np.uint64)
    seeds = np.array([17, 29], np.uint64)
    plain = engine.evaluate_faco_evaluations(keys, seeds, ants * iterations, 8, trace=True)
    controlled = engine.evaluate_population_evaluations(keys, seeds, ants * iterations, [program, program])
    for c in range(2):
        key = oracle.lib().orc_colony_key(int(seeds[c]), 312)
        ref = oracle.run_colony(xy, prep, ants=ants, k=16, b=50, w=20, mne=8, iterations=iterations, key=key,
                                retention=0.9, ls_limit=limit)
        assert plain["items"][c]["tour"] == ref["tour"].tolist() and plain["items"][c]["cost"] == ref["cost"]
        assert [int(x) for x in plain["trace"]["ls_evaluations"][:, c]] == \
            [int(row["ls_evaluations"]) for row in ref["trace"]]
        ref = oracle.run_colony(xy, prep, ants=ants, k=16, b=50, w=20, mne=8, iterations=iterations, key=key,
                                retention=0.9, ls_limit=limit, program=program, total_iterations=iterations)
        for part in controlled:
            assert part["items"][c]["tour"] == ref["tour"].tolist() and part["items"][c]["cost"] == ref["cost"]
    if limit == 1:
        for points in ([1, 1], [3, 1], [iterations + 1]):
            with pytest.raises(ValueError):
                engine.evaluate_faco_evaluations(keys, seeds, ants * iterations, 8, checkpoint_iterations=points)
    engine.close()


def test_invalid_inputs_raise_before_search(api):
    """Strict inputs (tests/python/test_fixed_faco_gpu.py:39-68, test_batch_engine.py:62-79)."""
    engine = api.FacoBatchEngine(50, 2, _settings(api, 8))
    xy = _cases.uniform_instance(50, seed=1).astype(np.float64)
    with pytest.raises(ValueError):
        engine.register_problem(1, xy.astype(np.float32))
    with pytest.raises(ValueError):
        engine.register_problem(True, xy)
    bad = xy.copy(); bad[0, 0] = np.nan
    with pytest.raises(ValueError):
        engine.register_problem(1, bad)
    bad = xy.copy(); bad[0, 0] = -2.0**23; bad[1, 0] = 2.0**23      # span 2^24: EUC_2D no longer exact in double
    with pytest.raises(ValueError):
        engine.register_problem(1, bad)
    bad = xy.copy(); bad[0, 0] = 0.5
    with pytest.raises(ValueError):
        engine.register_problem(1, bad)
    engine.register_problem(1, xy)
    keys = np.array([1, 1], np.uint64); seeds = np.array([1, 2], np.uint64)
    with pytest.raises(ValueError):
        engine.evaluate_faco_evaluations(keys, seeds, 7, 8)          # not whole ant batches
    with pytest.raises(ValueError):
        engine.evaluate_faco_evaluations(keys.astype(np.int64), seeds, 8, 8)
    with pytest.raises(ValueError):
        engine.evaluate_faco_evaluations(np.array([1, 9], np.uint64), seeds, 8, 8)  # unregistered
    zero = engine.evaluate_faco_evaluations(keys, seeds, 0, 8)
    rows = engine.problem_rows(1)
    assert zero["items"][0]["tour"] == rows["initial_tour"].tolist()
    engine.close()


def _control_state(trace, initial_cost):
    """Controller feedback after the last batch, from an oracle trace:
    restarts (actions >= 16), batches since the last global improvement, and
    the start region / MNE target the last action set."""
    best, last = initial_cost, 0
    for it, row in enumerate(trace):
        if row["global_cost"] < best:
            best, last = row["global_cost"], it + 1
    a = int(trace[-1]["action"])
    return {"restarts": sum(int(row["action"]) >= 16 for row in trace), "stagnant_batches": len(trace) - last,
            "start_region": (a >> 2) & 3, "mne_target": 2 << (a & 3)}


@pytest.mark.parametrize("n,ants,iterations", [(60, 8, 10), (250, 16, 12), (1000, 32, 6)])
def test_gp_controlled_population_matches_oracle(api, oracle, n, ants, iterations):
    """GP-controlled colonies (feature spec 3: features, warp scoring of 32
    actions, MNE / start region / restart actions) agree bit-for-bit with the
    oracle: final tours and costs, and per iteration the best/global/parent
    costs, trail bounds, MNE target used and action chosen."""
    rng = np.random.default_rng(2024 + n)
    programs = [_programs.random_program(rng, extended=bool(i % 2), features=10, feature_spec_id=3)
                for i in range(5)]
    programs.append(dict(ir_version=1, numeric_spec_id=2, feature_spec_id=3, opcode=[0], operand=[9],
                         constant_bits=[]))                              # always restart
    replicas = 2
    xy = _cases.uniform_instance(n, seed=n + 5)
    settings = _settings(api, ants, retention=0.9)
    engine = api.FacoBatchEngine(n, replicas, settings, population_size=len(programs))
    engine.register_problem(42, xy.astype(np.float64))
    prep = oracle.prepare(xy, 16, 64, 20)
    keys = np.full(replicas, 42, np.uint64)
    seeds = np.arange(replicas, dtype=np.uint64) + 3
    mask = 0xFFFFFFFF if n != 250 else 0x00FF00FF
    res = engine.evaluate_population_evaluations(keys, seeds, ants * iterations, programs, mask, trace=True)
    assert len(res) == len(programs)
    for i, program in enumerate(programs):
        part = res[i]
        assert part["population_size"] == len(programs) and len(part["items"]) == replicas
        assert part["completed_construction_steps"] == int(part["colony_work"][:, 0].sum())
        for j in range(replicas):
            key = oracle.lib().orc_colony_key(int(seeds[j]), 42)
            ref = oracle.run_colony(xy, prep, ants=ants, k=16, b=64, w=20, mne=8, iterations=iterations, key=key,
                                    retention=0.9, program=program, mask=mask, total_iterations=iterations)
            assert part["items"][j]["cost"] == ref["cost"], (i, j)
            assert part["items"][j]["tour"] == ref["tour"].tolist(), (i, j)
            for it in range(iterations):
                row, want = part["trace"][it, j], ref["trace"][it]
                for field in ("iteration_best_cost", "global_cost", "parent_cost", "iteration_best", "mne_target",
                              "action", "construction_steps", "ls_evaluations"):
                    assert int(row[field]) == int(want[field]), (i, j, it, field)
                assert row["tau_min"] == np.float32(want["tau_min"]) and row["tau_max"] == np.float32(want["tau_max"])
            assert part["control_states"][j] == _control_state(ref["trace"], prep["cost"]), (i, j)
    # a joint_single controller dict is its one tree; a conditional one whose
    # restart role reads the MNE-level descriptor is refused
    one = engine.evaluate_controller_evaluations(
        np.full(2, 42, np.uint64), seeds, ants * iterations,
        {"controller_version": 1, "representation": "joint_single", "controller_id": 7, "trees": [programs[0]]},
        mask)
    assert [it["cost"] for it in one["items"]] == [it["cost"] for it in res[0]["items"]]
    reads_level = dict(ir_version=1, numeric_spec_id=1, feature_spec_id=3, opcode=[0], operand=[7],
                       constant_bits=[])
    with pytest.raises(ValueError):
        engine.evaluate_controller_evaluations(
            keys, seeds, ants * iterations,
            {"controller_version": 1, "representation": "conditional_three", "controller_id": 7,
             "trees": [reads_level, programs[1], programs[2]]})
    with pytest.raises(ValueError):
        engine.evaluate_population_evaluations(np.full(3, 42, np.uint64), np.arange(3, dtype=np.uint64),
                                               ants * iterations, programs)     # not the whole panel
    engine.close()


def test_fixed_faco_gpu_and_sessions(api, oracle):
    """FixedFacoGpu.run_iterations restarts its colony on every call and
    equals the batch engine's colony for the same (instance, seed);
    GpuSession.solve_population returns one result per program."""
    n, ants, iterations = 120, 8, 6
    xy = _cases.uniform_instance(n, seed=77)
    settings = _settings(api, ants)
    fixed = api.FixedFacoGpu(xy.astype(np.float64), 5, settings)
    first = fixed.run_iterations(3, iterations, 8)
    again = fixed.run_iterations(3, iterations, 8)
    assert first["tour"] == again["tour"] and first["cost"] == again["cost"]
    assert first["batches"] == iterations and first["cost"] <= first["initial_cost"]
    prep = oracle.prepare(xy, 16, 64, 20)
    ref = oracle.run_colony(xy, prep, ants=ants, k=16, b=64, w=20, mne=8, iterations=iterations,
                            key=oracle.lib().orc_colony_key(3, 5), retention=0.98)
    assert first["cost"] == ref["cost"] and first["tour"] == ref["tour"].tolist()
    with pytest.raises(ValueError):
        fixed.run_iterations(True, 1, 8)
    fixed.close()
    from gplsaco_gb300.session import GpuSession, Instance
    session = GpuSession(colonies=2, settings=settings)
    problems = {"a": Instance(5, xy)}
    programs = [dict(ir_version=1, numeric_spec_id=1, feature_spec_id=3, opcode=[0], operand=[4], constant_bits=[]),
                dict(ir_version=1, numeric_spec_id=1, feature_spec_id=3, opcode=[0], operand=[5], constant_bits=[])]
    results, timing = session.solve_population(problems, [("a", 3), ("a", 4)], iterations, programs)
    assert len(results) == 2 and all(len(r["items"]) == 2 for r in results)
    plain, _ = session.solve(problems, [("a", 3), ("a", 4)], iterations)
    assert plain["items"][0]["cost"] == ref["cost"]
    session.close()


@pytest.mark.parametrize("n,k,b,w", [(2500, 32, 64, 32), (600, 16, 250, 20)])
def test_registration_rows_match_oracle(api, oracle, n, k, b, w):
    """Registration on a clustered instance with duplicated points (length
    ties order by node id): candidate rows from the GPU near lists (or the
    host sort when the rows are wider than the kernel's list), the
    nearest-neighbour tour and its initial 2-opt equal the oracle's
    preparation (prepared_problem.cpp:58-120)."""
    from gplsaco_gb300 import instances
    xy = instances.clustered(n, 31).astype(np.int32)
    xy[1::97] = xy[0]                      # duplicates of node 0
    xy[5::101] = xy[3]
    settings = _settings(api, 8, k, b, w)
    engine = api.FacoBatchEngine(n, 1, settings)
    info = engine.register_problem(7, xy.astype(np.float64))
    rows = engine.problem_rows(7)
    prep = oracle.prepare(xy, k, b, w)
    assert np.array_equal(rows["primary"], prep["primary"])
    assert np.array_equal(rows["backup"], prep["backup"])
    assert np.array_equal(rows["ls"], prep["ls"])
    assert np.array_equal(rows["initial_tour"], prep["initial"]) and info["initial_cost"] == prep["cost"]
    # A registered identity is immutable (batch_engine.cu:285-289, test_batch_engine.py:82-86).
    assert engine.register_problem(7, xy.astype(np.float64)) == info
    with pytest.raises(ValueError):
        engine.register_problem(7, xy.astype(np.float64) + 0.1)
    with pytest.raises(ValueError):
        engine.register_problem(7, xy[:-1].astype(np.float64))
    assert np.array_equal(engine.problem_rows(7)["primary"], prep["primary"])
    engine.close()


def test_snapshot_resume_continues_bit_for_bit(api):
    """Colony snapshots (CountedState, counted_state.hpp:23-38): a run
    captured after 5 iterations and continued for 7 on a fresh engine equals
    a straight 12-iteration run -- plain and GP-controlled; corrupted or
    mismatched snapshots are refused."""
    ants, n1, n2 = 8, 150, 230
    xys = {11: _cases.uniform_instance(n1, seed=21), 12: _cases.uniform_instance(n2, seed=22)}
    settings = _settings(api, ants, retention=0.9)

    def engine():
        e = api.FacoBatchEngine(n2, 4, settings)
        for key, xy in xys.items():
            e.register_problem(key, xy.astype(np.float64))
        return e

    keys = np.array([11, 12, 12, 11], np.uint64)
    seeds = np.array([1, 2, 3, 4], np.uint64)
    a = engine()
    full = a.evaluate_faco_evaluations(keys, seeds, ants * 12, 8)
    cap = a.capture_faco_state(keys, seeds, ants * 5)
    state = api.CountedState.from_bytes(cap["state"].to_bytes())
    info = state.describe()
    assert info["completed_batches"] == 5 and info["instance_keys"] == keys.tolist()
    assert info["global_costs"] == [it["cost"] for it in cap["evaluation"]["items"]]
    b = engine()
    rest = b.continue_faco_state(state, ants * 7)
    assert [it["tour"] for it in rest["items"]] == [it["tour"] for it in full["items"]]
    assert [it["cost"] for it in rest["items"]] == [it["cost"] for it in full["items"]]
    assert rest["completed_batches"] == 12
    assert rest["completed_construction_steps"] == full["completed_construction_steps"]
    assert rest["completed_ls_evaluations"] == full["completed_ls_evaluations"]

    program = dict(ir_version=1, numeric_spec_id=2, feature_spec_id=3, opcode=[0, 0, 2], operand=[1, 8, 0],
                   constant_bits=[])
    full_p = a.evaluate_program_evaluations(keys, seeds, ants * 12, program)
    cap_p = a.capture_program_state(keys, seeds, ants * 12, ants * 5, program)
    rest_p = b.continue_program_state(cap_p["state"], ants * 7, program)
    assert [it["tour"] for it in rest_p["items"]] == [it["tour"] for it in full_p["items"]]
    assert [it["cost"] for it in rest_p["items"]] == [it["cost"] for it in full_p["items"]]
    other = dict(program, operand=[2, 8, 0])
    with pytest.raises(ValueError):
        b.continue_program_state(cap_p["state"], ants * 7, other)

    raw = bytearray(state.to_bytes())
    raw[len(raw) // 2] ^= 0x40
    with pytest.raises(ValueError):
        b.restore_state(api.CountedState(bytes(raw)))              # checksum
    c = api.FacoBatchEngine(n2, 4, _settings(api, ants, retention=0.5))
    for key, xy in xys.items():
        c.register_problem(key, xy.astype(np.float64))
    with pytest.raises(ValueError):
        c.restore_state(state)                                     # other settings
    d = api.FacoBatchEngine(n2, 4, settings)
    d.register_problem(11, xys[11].astype(np.float64))
    with pytest.raises(ValueError):
        d.restore_state(state)                                     # instance 12 missing
    for e in (a, b, c, d):
        e.close()


@pytest.mark.parametrize("spec", [3, 2])
def test_gp_evolution_on_the_engine(api, spec):
    """A short evolution (8 programs, 3 generations) evaluated as population
    batches on the engine: every generation's programs run, the elites carry
    the best fitness forward (same panel and seeds, so re-evaluation is exact)
    -- with the engine's controller features and the reference's 12."""
    from gplsaco_gb300 import evolution as ev
    n, ants = 60, 8
    xy = _cases.uniform_instance(n, seed=321)
    settings = _settings(api, ants)
    engine = api.FacoBatchEngine(n, 2, settings, population_size=8)
    info = engine.register_problem(5, xy.astype(np.float64))
    keys, seeds = np.full(2, 5, np.uint64), np.array([1, 2], np.uint64)
    refs = np.full(2, float(info["initial_cost"]))
    evo = ev.evolve(engine, keys, seeds, refs, 6,
                    ev.EvolutionSettings(population=8, generations=3, elites=2, feature_spec_id=spec), 9)
    fitness = [w["fitness"] for w in evo.winners]
    assert len(fitness) == 3 and all(0 < f <= 1.0 for f in fitness)
    assert fitness[1] <= fitness[0] and fitness[2] <= fitness[1]
    assert len(evo.shortlist()) >= 3
    engine.close()


def test_population_matches_every_serial_member(api):
    """A population batch equals each member run on its own: tours, costs,
    work counters and controller feedback, over two panels of three
    instances; a duplicated program gets its own colonies and equal results;
    sub-populations (any slice, fewer than the engine holds) reproduce their
    members' results; population sizes 0 and 129 and an empty population are
    refused (tests/python/test_population_cuda.py:27-103)."""
    from gplsaco_gb300 import evolution as ev
    n, replicas, iterations, ants = 67, 4, 40, 8
    settings = _settings(api, ants)
    evo = ev.Evolution(ev.EvolutionSettings(population=8, elites=2), 1103)
    evo.initialize()
    values = evo.programs()
    values[-1] = values[0]
    serial = api.FacoBatchEngine(n, replicas, settings)
    expanded = api.FacoBatchEngine(n, replicas, settings, population_size=len(values))
    for key in (1, 2, 3):
        xy = np.random.default_rng(107 + key).integers(0, 5000, (n, 2)).astype(np.float64)
        for engine in (serial, expanded):
            engine.register_problem(key, xy)
    fields = ("completed_construction_steps", "completed_ls_evaluations", "completed_tour_evaluations_per_colony",
              "total_tour_evaluations", "control_states")
    for panel, panel_seeds in (([1, 1, 2, 2], [17, 29, 17, 29]), ([3, 2, 3, 1], [41, 29, 53, 17])):
        keys, seeds = np.asarray(panel, np.uint64), np.asarray(panel_seeds, np.uint64)
        results = expanded.evaluate_population_evaluations(keys, seeds, iterations * ants, values)
        assert len(results) == len(values)
        for program, actual in zip(values, results, strict=True):
            expected = serial.evaluate_program_evaluations(keys, seeds, iterations * ants, program)
            assert [(r["tour"], r["cost"]) for r in actual["items"]] == \
                [(r["tour"], r["cost"]) for r in expected["items"]]
            for field in fields:
                assert actual[field] == expected[field], field
            assert actual["actual_seconds"] * len(values) == pytest.approx(actual["population_actual_seconds"])
        assert results[0]["items"] == results[-1]["items"]
        for start, stop in ((3, 8), (0, 1), (0, 3), (0, 8)):
            chunk = expanded.evaluate_population_evaluations(keys, seeds, iterations * ants, values[start:stop])
            assert len(chunk) == stop - start
            for expected, actual in zip(results[start:stop], chunk, strict=True):
                assert [(r["tour"], r["cost"]) for r in actual["items"]] == \
                    [(r["tour"], r["cost"]) for r in expected["items"]]
                for field in fields:
                    assert actual[field] == expected[field], field
    for count in (0, 129):
        with pytest.raises(ValueError):
            api.FacoBatchEngine(n, replicas, settings, population_size=count)
    with pytest.raises(ValueError):
        expanded.evaluate_population_evaluations(keys, seeds, ants, [])
    single = serial.evaluate_population_evaluations(keys, seeds, ants, [values[1]])[0]
    expected = serial.evaluate_program_evaluations(keys, seeds, ants, values[1])
    assert single["control_states"] == expected["control_states"]
    assert [r["tour"] for r in single["items"]] == [r["tour"] for r in expected["items"]]
    serial.close()
    expanded.close()


@pytest.mark.parametrize("case", ["n3", "single_ant", "all_identical", "mostly_duplicates"])
def test_degenerate_instances_match_oracle(api, oracle, case):
    """Edge cases: the smallest instance, one colony of one ant, every point
    identical (all lengths 0: zero-weight roulette and no improving move),
    and an instance that is mostly duplicates -- each equal to the oracle
    bit for bit, every returned tour a permutation of its length."""
    rng = np.random.default_rng(77)
    ants, iterations, k, b, w = 4, 6, 16, 64, 20
    if case == "n3":
        xy = np.array([[0, 0], [3, 4], [6, 0]], np.int32)
    elif case == "single_ant":
        xy = _cases.uniform_instance(40, seed=3)
        ants = 1
    elif case == "all_identical":
        xy = np.full((25, 2), 123456, np.int32)
    else:
        xy = np.repeat(_cases.uniform_instance(6, seed=9), 8, axis=0)[rng.permutation(48)]
    n = xy.shape[0]
    settings = _settings(api, ants, k, b, w)
    engine = api.FacoBatchEngine(n, 2, settings)
    engine.register_problem(3, xy.astype(np.float64))
    kk, bb, ww = min(k, n - 1), min(b, n - 1 - min(k, n - 1)), min(w, n - 1)
    prep = oracle.prepare(xy, kk, bb, ww)
    seeds = np.array([1, 2], np.uint64)
    res = engine.evaluate_faco_evaluations(np.full(2, 3, np.uint64), seeds, ants * iterations, 8)
    for c in range(2):
        ref = oracle.run_colony(xy, prep, ants=ants, k=kk, b=bb, w=ww, mne=8, iterations=iterations,
                                key=oracle.lib().orc_colony_key(int(seeds[c]), 3), retention=0.98)
        assert res["items"][c]["cost"] == ref["cost"] and res["items"][c]["tour"] == ref["tour"].tolist()
        assert sorted(res["items"][c]["tour"]) == list(range(n))
    engine.close()


def test_score_controllers_match_oracle(api, oracle):
    """faco_score_controllers: conditional_three role scores (slots 0-9) and
    actions bit-identical to the oracle; joint controllers equal score_cuda."""
    rng = np.random.default_rng(4242)
    for extended in (False, True):
        for _ in range(48):
            ctl = _programs.random_conditional(rng, extended=extended)
            features = (np.round(rng.random((12, 7, 32), dtype=np.float32) * 4) / 4).astype(np.float32)
            masks = rng.integers(1, 2**32, size=7, dtype=np.uint64).astype(np.uint32)
            got = api.score_controller_cuda(ctl, features, masks)
            ref_scores, ref_actions = oracle.score_conditional(ctl["trees"], features, masks)
            assert np.array_equal(got["actions"], ref_actions)
            assert np.array_equal(got["scores"], ref_scores)
    program = _programs.random_program(rng, features=10, feature_spec_id=3)
    joint = {"controller_version": 1, "representation": "joint_single", "controller_id": 2, "trees": [program]}
    features = rng.random((12, 5, 32), dtype=np.float32)
    masks = rng.integers(1, 2**32, size=5, dtype=np.uint64).astype(np.uint32)
    got = api.score_controller_cuda(joint, features, masks)
    ref_scores, ref_actions = oracle.score(program, features, masks)
    assert np.array_equal(got["actions"], ref_actions) and np.array_equal(got["scores"], ref_scores)
    bad = _programs.random_conditional(rng)
    bad["trees"][0] = dict(ir_version=1, numeric_spec_id=1, feature_spec_id=3, opcode=[0], operand=[7],
                           constant_bits=[])                       # role 0 reads the MNE level
    with pytest.raises(ValueError):
        api.score_controller_cuda(bad, features, masks)


@pytest.mark.parametrize("n,ants,iterations", [(80, 8, 12), (400, 16, 8)])
def test_conditional_controllers_match_oracle(api, oracle, n, ants, iterations):
    """conditional_three and joint controllers in one population batch: tours,
    costs and every trace field (MNE target used, action chosen) equal the
    oracle's controlled colony runs."""
    rng = np.random.default_rng(808 + n)
    controllers = [_programs.random_conditional(rng), _programs.random_conditional(rng, extended=True),
                   _programs.random_program(rng, features=10, feature_spec_id=3)]
    replicas = 2
    xy = _cases.uniform_instance(n, seed=n + 17)
    settings = _settings(api, ants, retention=0.9)
    engine = api.FacoBatchEngine(n, replicas, settings, population_size=len(controllers))
    engine.register_problem(77, xy.astype(np.float64))
    prep = oracle.prepare(xy, 16, 64, 20)
    keys = np.full(replicas, 77, np.uint64)
    seeds = np.arange(replicas, dtype=np.uint64) + 11
    res = engine.evaluate_population_evaluations(keys, seeds, ants * iterations, controllers, 0xFFFF0FFF)
    assert len(res) == len(controllers)
    for i, ctl in enumerate(controllers):
        for j in range(replicas):
            ref = oracle.run_colony(xy, prep, ants=ants, k=16, b=64, w=20, mne=8, iterations=iterations,
                                    key=oracle.lib().orc_colony_key(int(seeds[j]), 77), retention=0.9,
                                    program=ctl, mask=0xFFFF0FFF, total_iterations=iterations)
            assert res[i]["items"][j]["cost"] == ref["cost"], (i, j)
            assert res[i]["items"][j]["tour"] == ref["tour"].tolist(), (i, j)
    # the single-controller entry point and a trace check on the first one
    one = engine.evaluate_controller_evaluations(np.full(2, 77, np.uint64), seeds, ants * iterations,
                                                 controllers[0], 0xFFFF0FFF)
    assert [it["cost"] for it in one["items"]] == [it["cost"] for it in res[0]["items"]]
    engine.close()


@pytest.mark.parametrize("chains,workspace", [(2, 0), (3, 2), (5, 0)])
def test_colony_chains_change_nothing(api, oracle, chains, workspace):
    """Colonies split into independent chains in the evaluation's graph
    (iterations of different chains overlap) give the results of the
    unchained run bit for bit: tours, costs and every trace row, over two
    graph replays and a remainder; plain FACO on an uneven batch and the
    12-feature controller with decision captures; tours in shared memory and
    in the global workspace (one slot per colony and ant, so concurrent
    chains never share one)."""
    sizes = [200, 537, 1000, 311]
    ants, iterations = 8, 37
    xys = [_cases.uniform_instance(n, seed=200 + i) for i, n in enumerate(sizes)]
    keys = np.array([1003, 1000, 1002, 1001, 1002, 1000, 1003], np.uint64)
    seeds = np.arange(11, 18, dtype=np.uint64)
    program = _programs.random_program(np.random.default_rng(5), features=12, feature_spec_id=2)
    runs = {}
    for ch in (1, chains):
        settings = api.FixedFacoSettings(ants=ants, primary_width=16, backup_width=64, ls_width=20, retention=0.9,
                                         chains=ch, workspace=workspace)
        engine = api.FacoBatchEngine(1000, keys.size, settings)
        for i, xy in enumerate(xys):
            engine.register_problem(1000 + i, xy.astype(np.float64))
        plain = engine.evaluate_faco_evaluations(keys, seeds, ants * iterations, 8, trace=True)
        controlled = engine.evaluate_program_evaluations(keys, seeds, ants * iterations, program, trace=True,
                                                         decision_iterations=[1, 20, iterations])
        runs[ch] = (plain, controlled)
        plan = engine.launch_plan()            # of the last (12-feature controlled) evaluation
        assert plan["size_classes"] == 3 and plan["graph_iterations"] == 16
        if ch == 1:
            assert plan["chains"] == 0 and plan["launches_per_iteration"] == 3 + 2
        else:
            # every class split into at least one chain, at most one chain per colony
            assert 3 <= plan["chains"] <= keys.size and plan["launches_per_iteration"] == 3 * plan["chains"]
        engine.close()
    for a, b in zip(runs[1], runs[chains]):
        assert [it["tour"] for it in a["items"]] == [it["tour"] for it in b["items"]]
        assert [it["cost"] for it in a["items"]] == [it["cost"] for it in b["items"]]
        assert np.array_equal(a["trace"], b["trace"])
    da, db = runs[1][1]["decisions"], runs[chains][1]["decisions"]
    assert len(da) == len(db) == 3 * keys.size
    for x, y in zip(da, db):
        assert x["action"] == y["action"]
        assert np.array_equal(np.asarray(x["features"], np.float32).view(np.uint32),
                              np.asarray(y["features"], np.float32).view(np.uint32))
    xy = xys[2]
    key = oracle.lib().orc_colony_key(int(seeds[2]), int(keys[2]))
    ref = oracle.run_colony(xy, oracle.prepare(xy, 16, 64, 20), ants=ants, k=16, b=64, w=20, mne=8,
                            iterations=iterations, key=key, retention=0.9)
    assert runs[chains][0]["items"][2]["cost"] == ref["cost"]


def test_follow_batches_change_nothing(api):
    """Converged colonies (long walks along the parent tour): the evaluation
    with the parent-following steps taken in batches equals the one that
    takes them one at a time, tours, lengths and every trace row."""
    n, ants, iterations = 1000, 32, 160
    xy = _cases.uniform_instance(n, seed=77)
    out = {}
    for follow in (1, 2):
        engine = api.FacoBatchEngine(n, 4, _settings(api, ants, follow=follow))
        engine.register_problem(3, xy.astype(np.float64))
        keys, seeds = np.full(4, 3, np.uint64), np.array([1, 2, 3, 4], np.uint64)
        engine.begin(keys, seeds, 8, trace_iterations=iterations)
        assert engine.launch_plan()["follow"] == (1 if follow == 2 else 0)
        engine.step(iterations)
        out[follow] = engine.finish()
        engine.close()
    a, b = out[1], out[2]
    assert np.array_equal(a["costs"], b["costs"])
    assert all(np.array_equal(x, y) for x, y in zip(a["tours"], b["tours"]))
    assert np.array_equal(a["trace"], b["trace"])
    assert np.array_equal(a["colony_work"], b["colony_work"])
    late = a["trace"][-16:]
    assert float(late["construction_steps"].sum()) / (16 * 4 * ants) > 30   # walks several times the MNE target


@pytest.mark.parametrize("workspace", [0, 2])
def test_adaptive_batches_change_nothing(api, workspace):
    """A panel beyond one wave of ant warps (160 colonies x 32 ants, N=1000)
    with the automatic setting, the ants' tours in shared memory and in the
    global-memory workspace: the engine reads the walk length every 32
    iterations and switches to the batched-step graph once walks are long.
    The run equals the one that takes every step one at a time -- tours,
    lengths, every trace row -- and by its end the walks are long enough for
    the switch; a run restored from a snapshot in the middle goes on equal
    too, and so does a run stepped in pieces that are not whole graph
    replays (the remainders launched directly, in the variant chosen), or
    timed kernel by kernel."""
    n, ants, colonies, iterations = 1000, 32, 160, 320
    xys = [_cases.uniform_instance(n, seed=500 + i) for i in range(4)]
    keys = np.repeat(np.arange(10, 14, dtype=np.uint64), colonies // 4)
    seeds = np.tile(np.arange(colonies // 4, dtype=np.uint64), 4)

    def engine(follow):
        e = api.FacoBatchEngine(n, colonies, _settings(api, ants, workspace=workspace, follow=follow))
        for i, xy in enumerate(xys):
            e.register_problem(10 + i, xy.astype(np.float64))
        return e

    out = {}
    for follow in (0, 1):
        e = engine(follow)
        e.begin(keys, seeds, 8, trace_iterations=iterations)
        assert e.launch_plan()["follow"] == (2 if follow == 0 else 0)
        e.step(iterations)
        out[follow] = e.finish()
        e.close()
    a, b = out[0], out[1]
    assert np.array_equal(a["costs"], b["costs"])
    assert all(np.array_equal(x, y) for x, y in zip(a["tours"], b["tours"]))
    assert np.array_equal(a["trace"], b["trace"])
    late = a["trace"][-64:]["construction_steps"].astype(np.float64).sum() / (64 * colonies * ants)
    assert late >= (72 if workspace == 0 else 96)   # the last stretches ran with batches
    # snapshot at 160, continued on a fresh engine with the automatic setting
    e = engine(0)
    e.begin(keys, seeds, 8)
    e.step(160)
    state = e.capture_state()
    e.finish()
    e.close()
    e = engine(0)
    e.restore_state(state)
    e.step(iterations - 160)
    res = e.finish()
    e.close()
    assert np.array_equal(res["costs"], a["costs"])
    # stepped in pieces of 5, 27, 11 and 9 iterations (then 8)
    e = engine(0)
    e.begin(keys, seeds, 8, trace_iterations=iterations)
    done = 0
    for piece in [5, 27, 11, 9] * 6 + [8]:
        e.step(piece)
        done += piece
    assert done == iterations
    res = e.finish()
    e.close()
    assert np.array_equal(res["costs"], b["costs"])
    assert all(np.array_equal(x, y) for x, y in zip(res["tours"], b["tours"]))
    assert np.array_equal(res["trace"], b["trace"])
    # the unchained timing path, which runs the variants step() would run
    e = engine(0)
    e.begin(keys, seeds, 8, trace_iterations=iterations)
    ant_ms, update_ms = e.step_timed(iterations)
    res = e.finish()
    e.close()
    assert ant_ms > 0 and update_ms > 0
    assert np.array_equal(res["costs"], b["costs"])
    assert np.array_equal(res["trace"], b["trace"])

"""The reference's 12-feature controller (feature spec 2) on the GPU against
the oracle colony run, through the C ABI: tours, costs, per-batch traces,
the controller feedback and the captured decisions (all 12 x 32 features,
scores, legal masks, actions) bit for bit."""
import numpy as np
import pytest

from tests import _cases, _programs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api(engine_lib):
    import gplsaco_gb300 as g
    return g


def _settings(api, ants, **kw):
    return api.FixedFacoSettings(ants=ants, primary_width=16, backup_width=64, ls_width=20, retention=0.9, **kw)


def _always_restart():
    # the mode feature (4): actions 16-31 score 1 whenever they are legal
    return dict(ir_version=1, numeric_spec_id=1, feature_spec_id=2, opcode=[0], operand=[4], constant_bits=[])


def _check_colony(res, c, ref, iterations, ctx):
    assert res["items"][c]["cost"] == ref["cost"], ctx
    assert res["items"][c]["tour"] == ref["tour"].tolist(), ctx
    for it in range(iterations):
        row, want = res["trace"][it, c], ref["trace"][it]
        for field in ("iteration_best_cost", "global_cost", "parent_cost", "iteration_best", "mne_target", "action",
                      "construction_steps", "ls_evaluations"):
            assert int(row[field]) == int(want[field]), (ctx, it, field)
        assert row["tau_min"] == np.float32(want["tau_min"]) and row["tau_max"] == np.float32(want["tau_max"])
    got, want = res["control_states"][c], ref["control_state"]
    for field in ("archive_size", "stagnant_batches", "epoch_batches", "restarts"):
        assert got[field] == want[field], (ctx, field)
    assert np.float32(got["return_rate"]) == np.float32(want["return_rate"])
    assert np.float32(got["ls_work"]) == np.float32(want["ls_work"])


@pytest.mark.parametrize("n,ants,iterations", [(60, 8, 12), (250, 16, 10), (1000, 32, 6)])
def test_spec2_programs_match_oracle(api, oracle, n, ants, iterations):
    rng = np.random.default_rng(n + 2)
    programs = [_programs.random_program(rng, extended=bool(i % 2), features=12, feature_spec_id=2)
                for i in range(3)] + [_always_restart()]
    xy = _cases.uniform_instance(n, seed=n + 11)
    engine = api.FacoBatchEngine(n, 2, _settings(api, ants))
    engine.register_problem(42, xy.astype(np.float64))
    prep = oracle.prepare(xy, 16, 64, 20)
    keys, seeds = np.full(2, 42, np.uint64), np.array([3, 4], np.uint64)
    points = [1, 2, iterations // 2, iterations]
    mask = 0xFFFFFFFF if n != 250 else 0x0F0F0F0F
    restarts = 0
    for i, program in enumerate(programs):
        res = engine.evaluate_program_evaluations(keys, seeds, ants * iterations, program, "cached", mask, trace=True,
                                                  decision_iterations=points)
        assert len(res["decisions"]) == len(points) * 2
        for c in range(2):
            key = oracle.lib().orc_colony_key(int(seeds[c]), 42)
            ref = oracle.run_colony(xy, prep, ants=ants, k=16, b=64, w=20, mne=8, iterations=iterations, key=key,
                                    retention=0.9, program=program, mask=mask, total_iterations=iterations,
                                    instance_key=42, decision_iterations=points)
            _check_colony(res, c, ref, iterations, (i, c))
            restarts += res["control_states"][c]["restarts"]
            for d, want in enumerate(ref["decisions"]):
                got = res["decisions"][d * 2 + c]
                assert got["iteration"] == want["iteration"] and got["colony"] == c
                assert got["legal_mask"] == want["legal_mask"] and got["action"] == want["action"], (i, c, d)
                assert np.array_equal(np.asarray(got["features"], np.float32).view(np.uint32),
                                      want["features"].view(np.uint32)), (i, c, d)
                assert np.array_equal(np.asarray(got["scores"], np.float32).view(np.uint32),
                                      want["scores"].view(np.uint32)), (i, c, d)
    assert restarts > 0                                   # the restart path ran
    engine.close()


def test_spec2_conditional_controllers_and_population(api, oracle):
    """conditional_three controllers of spec 2 (role features of
    controller.py:9) and joint programs in one population batch."""
    n, ants, iterations, replicas = 120, 8, 10, 2
    rng = np.random.default_rng(5)
    controllers = [_programs.random_conditional_spec2(rng) for _ in range(3)]
    controllers.append({"controller_version": 1, "representation": "joint_single", "controller_id": 9,
                        "trees": [_always_restart()]})
    xy = _cases.uniform_instance(n, seed=77)
    engine = api.FacoBatchEngine(n, replicas, _settings(api, ants), population_size=len(controllers))
    engine.register_problem(7, xy.astype(np.float64))
    prep = oracle.prepare(xy, 16, 64, 20)
    keys, seeds = np.full(replicas, 7, np.uint64), np.array([11, 12], np.uint64)
    parts = engine.evaluate_population_evaluations(keys, seeds, ants * iterations, controllers)
    for i, ctl in enumerate(controllers):
        single = engine.evaluate_controller_evaluations(keys, seeds, ants * iterations, ctl,
                                                        decision_iterations=[1, iterations])
        for c in range(replicas):
            key = oracle.lib().orc_colony_key(int(seeds[c]), 7)
            ref = oracle.run_colony(xy, prep, ants=ants, k=16, b=64, w=20, mne=8, iterations=iterations, key=key,
                                    retention=0.9, program=ctl, total_iterations=iterations, instance_key=7,
                                    decision_iterations=[1, iterations])
            for res in (parts[i], single):
                assert res["items"][c]["tour"] == ref["tour"].tolist(), (i, c)
                assert res["control_states"][c]["restarts"] == ref["control_state"]["restarts"]
            for d, want in enumerate(ref["decisions"]):
                got = single["decisions"][d * replicas + c]
                assert got["action"] == want["action"]
                assert np.array_equal(np.asarray(got["features"], np.float32), want["features"])
                if ctl["representation"] == "conditional_three":
                    stages = got["stages"]
                    assert [s["scores"] for s in stages] == [want["scores"][0:2].tolist(), want["scores"][2:6].tolist(),
                                                             want["scores"][6:10].tolist()]
    engine.close()


def test_spec2_snapshot_resume_and_refusals(api):
    """A spec-2 run captured after 5 batches and continued for 7 equals the
    straight 12-batch run (archive, feedback and start list travel in the
    snapshot); invalid controllers and masks are refused before search."""
    n, ants = 150, 8
    xy = _cases.uniform_instance(n, seed=3)
    program = _programs.random_program(np.random.default_rng(8), features=12, feature_spec_id=2)
    settings = _settings(api, ants)

    def engine():
        e = api.FacoBatchEngine(n, 2, settings)
        e.register_problem(5, xy.astype(np.float64))
        return e

    keys, seeds = np.full(2, 5, np.uint64), np.array([1, 2], np.uint64)
    a = engine()
    straight = a.evaluate_program_evaluations(keys, seeds, ants * 12, program)
    cap = a.capture_program_state(keys, seeds, ants * 12, ants * 5, program)
    b = engine()
    cont = b.continue_program_state(cap["state"], ants * 7, program)
    assert [it["tour"] for it in cont["items"]] == [it["tour"] for it in straight["items"]]
    assert cont["control_states"] == straight["control_states"]
    bad_role = {"controller_version": 1, "representation": "conditional_three", "controller_id": 3,
                "trees": [dict(program, opcode=[0], operand=[5], constant_bits=[]), program, program]}
    with pytest.raises(ValueError):
        a.evaluate_controller_evaluations(keys, seeds, ants * 4, bad_role)
    with pytest.raises(ValueError):
        a.evaluate_program_evaluations(keys, seeds, ants * 4, program, "cached", 0xFFFF0000)
    spec3 = dict(program, feature_spec_id=3, opcode=[0], operand=[1], constant_bits=[])
    pop = api.FacoBatchEngine(n, 2, settings, population_size=2)
    pop.register_problem(5, xy.astype(np.float64))
    with pytest.raises(ValueError):
        pop.evaluate_population_evaluations(keys, seeds, ants * 4, [program, spec3])
    pop.close()
    with pytest.raises(ValueError):
        a.evaluate_program_evaluations(keys, seeds, ants * 4, program, decision_iterations=[2, 2])
    a.close()
    b.close()


@pytest.mark.parametrize("grid", [False, True])
def test_spec2_forced_fingerprint_collisions_match_oracle(api, oracle, grid):
    """With every fingerprint forced to 0 (batch_engine.hpp:66) the archive
    orders and de-duplicates tours by full canonical comparison -- the path
    real runs take only on a fingerprint collision.  On a 12 x 12 grid many
    distinct tours share a length.  Tours, traces, feedback and decisions
    equal the oracle's forced run."""
    n, ants, iterations = 60, 8, 12
    rng = np.random.default_rng(91 + grid)
    xy = (rng.integers(0, 12, (n, 2)) if grid else _cases.uniform_instance(n, seed=5)).astype(np.int32)
    settings = _settings(api, ants, force_fingerprint_collisions=1)
    engine = api.FacoBatchEngine(n, 2, settings)
    engine.register_problem(9, xy.astype(np.float64))
    prep = oracle.prepare(xy, 16, 43, 20)
    keys, seeds = np.full(2, 9, np.uint64), np.array([5, 6], np.uint64)
    points = [1, 4, 8, 12]
    for program in (_programs.random_program(rng, features=12, feature_spec_id=2), _always_restart()):
        res = engine.evaluate_program_evaluations(keys, seeds, ants * iterations, program, trace=True,
                                                  decision_iterations=points)
        for c in range(2):
            key = oracle.lib().orc_colony_key(int(seeds[c]), 9)
            ref = oracle.run_colony(xy, prep, ants=ants, k=16, b=43, w=20, mne=8, iterations=iterations, key=key,
                                    retention=0.9, program=program, total_iterations=iterations, instance_key=9,
                                    decision_iterations=points, force_collisions=True)
            _check_colony(res, c, ref, iterations, ("forced", grid, c))
            for d, want in enumerate(ref["decisions"]):
                got = res["decisions"][d * 2 + c]
                assert got["legal_mask"] == want["legal_mask"] and got["action"] == want["action"]
                assert np.array_equal(np.asarray(got["features"], np.float32).view(np.uint32),
                                      want["features"].view(np.uint32))
    engine.close()


@pytest.mark.parametrize("workspace", [0, 2])
def test_spec2_uneven_batch_and_global_workspace(api, oracle, workspace):
    """The 12-feature controller on an uneven batch (instances of different
    sizes in one evaluation, each colony with its own archive and regions),
    with the ants' tours in shared memory and in the global workspace: every
    colony equals its own oracle run."""
    sizes = [150, 420, 2100]
    ants, iterations = 8, 6
    rng = np.random.default_rng(31)
    program = _programs.random_program(rng, features=12, feature_spec_id=2)
    engine = api.FacoBatchEngine(max(sizes), 3, _settings(api, ants, workspace=workspace))
    preps = {}
    for i, n in enumerate(sizes):
        xy = _cases.uniform_instance(n, seed=40 + i)
        engine.register_problem(70 + i, xy.astype(np.float64))
        preps[70 + i] = (xy, oracle.prepare(xy, 16, 64, 20))
    keys = np.array([72, 70, 71], np.uint64)
    seeds = np.array([3, 4, 5], np.uint64)
    res = engine.evaluate_program_evaluations(keys, seeds, ants * iterations, program, trace=True,
                                              decision_iterations=[2, iterations])
    for c in range(3):
        xy, prep = preps[int(keys[c])]
        key = oracle.lib().orc_colony_key(int(seeds[c]), int(keys[c]))
        ref = oracle.run_colony(xy, prep, ants=ants, k=16, b=64, w=20, mne=8, iterations=iterations, key=key,
                                retention=0.9, program=program, total_iterations=iterations,
                                instance_key=int(keys[c]), decision_iterations=[2, iterations])
        _check_colony(res, c, ref, iterations, ("uneven", workspace, c))
        for d, want in enumerate(ref["decisions"]):
            got = res["decisions"][d * 3 + c]
            assert got["action"] == want["action"]
            assert np.array_equal(np.asarray(got["features"], np.float32).view(np.uint32),
                                  want["features"].view(np.uint32))
    engine.close()

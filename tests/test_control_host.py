"""Host-side logic of the controllers (no GPU): controller validation of both
feature specs through the C ABI, the reference's role-feature rules, the
decision rows and conditional stages in the reference's result shape, and the
evolution loop producing 12-feature programs."""
import numpy as np
import pytest

from tests import _programs


@pytest.fixture(scope="module")
def engine_module():
    from gplsaco_gb300 import build
    build.build()
    from gplsaco_gb300 import engine
    return engine


def _tree(operands, spec=2):
    ops = [0] * len(operands) + [2] * (len(operands) - 1)
    return dict(ir_version=1, numeric_spec_id=1, feature_spec_id=spec, opcode=ops,
                operand=list(operands) + [0] * (len(operands) - 1), constant_bits=[])


def _conditional(trees):
    return {"controller_version": 1, "representation": "conditional_three", "controller_id": 4, "trees": trees}


def test_spec2_role_features_follow_the_reference(engine_module):
    """ROLE_FEATURES (python/gp_faco/controller.py:9): the restart role reads
    features 0-4, 6, 7; the region role all but 5; the MNE role all 12."""
    arrays = engine_module.controller_arrays
    arr, kinds = arrays([_conditional([_tree([0, 4, 6, 7]), _tree([8, 11, 4]), _tree([5, 9])])])
    assert kinds.tolist() == [1] and arr[0].feature_spec_id == 2
    for bad in ([_tree([5]), _tree([1]), _tree([2])], [_tree([8]), _tree([1]), _tree([2])],
                [_tree([1]), _tree([5]), _tree([2])]):
        with pytest.raises(ValueError):
            arrays([_conditional(bad)])
    with pytest.raises(ValueError):                               # one spec per controller
        arrays([_conditional([_tree([1]), _tree([1], spec=3), _tree([2])])])
    rng = np.random.default_rng(3)
    for _ in range(20):
        arrays([_programs.random_conditional_spec2(rng)])


def test_controller_stages_and_decision_rows(engine_module):
    scores = np.arange(32, dtype=np.float32) / 10
    mask = 0xFFFF0F0F
    stages = engine_module.controller_stages(scores, mask, 16 + 8 + 3)
    assert [s["selected"] for s in stages] == [1, 2, 3]
    assert stages[0]["scores"] == [float(np.float32(0.0)), float(np.float32(0.1))]
    assert stages[1]["legal"] == [True, True, True, True] and stages[0]["legal"] == [True, True]
    stages = engine_module.controller_stages(scores, 0x0000000F, 2)
    assert stages[0]["legal"] == [True, False] and [s["selected"] for s in stages] == [0, 0, 2]
    dec = dict(features=np.zeros((1, 2, 12, 32), np.float32), scores=np.zeros((1, 2, 32), np.float32),
               masks=np.array([[0xFFFF, 0xFFFFFFFF]], np.uint32), actions=np.array([[3, 17]], np.int32))
    dec["scores"][0, 1, 5] = np.inf
    rows = engine_module.decision_rows(np.array([4], np.uint32), dec, [0, 1], 2)
    assert [(r["iteration"], r["colony"], r["action"]) for r in rows] == [(4, 0, 3), (4, 1, 17)]
    assert "scores" in rows[0] and len(rows[0]["features"]) == 12 and len(rows[0]["features"][0]) == 32
    assert "stages" in rows[1]


def test_evolution_makes_12_feature_programs(engine_module):
    from gplsaco_gb300 import evolution as ev
    settings = ev.EvolutionSettings(population=16, generations=2, elites=2, feature_spec_id=2)
    evo = ev.Evolution(settings, 1103)
    evo.initialize()
    programs = evo.programs()
    assert all(p["feature_spec_id"] == 2 for p in programs)
    used = {a for p in programs for op, a in zip(p["opcode"], p["operand"]) if op == 0}
    assert max(used) >= 10 and max(used) < 12                     # the reference's 12 terminals
    engine_module.controller_arrays(programs)                     # every program validates
    state = evo.state_dict()
    again = ev.Evolution.from_state_dict(state)
    assert again.settings.feature_spec_id == 2 and again.programs() == programs
    with pytest.raises(ValueError):
        ev.EvolutionSettings(feature_spec_id=1)

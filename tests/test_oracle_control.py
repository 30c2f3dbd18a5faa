"""The engine's GP controller (feature spec 3) in the oracle: invariants.

The reference's 12-feature controller (cuda/control_state.cuh:200-364) is
replaced by the engine's 7 colony features + 3 action descriptors; these
tests pin the restated semantics on the CPU."""
import numpy as np
import pytest

from tests import _cases, _programs


def _program(opcode, operand, consts=()):
    bits = [int(b) for b in np.asarray(consts, np.float32).view(np.uint32)]
    return dict(ir_version=1, numeric_spec_id=2, feature_spec_id=3, opcode=list(opcode), operand=list(operand),
                constant_bits=bits)


def _run(oracle, program, mask=0xFFFFFFFF, n=120, iterations=12, seed=5):
    xy = _cases.uniform_instance(n, seed=seed)
    prep = oracle.prepare(xy, 16, 64, 20)
    key = oracle.lib().orc_colony_key(seed, 77)
    return oracle.run_colony(xy, prep, ants=8, k=16, b=64, w=20, mne=8, iterations=iterations, key=key,
                             retention=0.9, program=program, mask=mask, total_iterations=iterations), prep


def test_constant_programs_pick_their_action(oracle):
    # score = restart flag (feature 9): the best legal action is the first restart action, 16
    res, _ = _run(oracle, _program([0], [9]))
    actions = [r["action"] for r in res["trace"]]
    assert actions == [16] * len(actions)
    # after each restart the next iteration runs with MNE 2 << (16 & 3) = 2
    assert [r["mne_target"] for r in res["trace"]][1:] == [2] * (len(actions) - 1)
    # score = MNE level (feature 7): ties between 3, 7, 11 and 15 resolve to the lowest lane
    res, _ = _run(oracle, _program([0], [7]))
    assert {r["action"] for r in res["trace"]} == {3}
    assert [r["mne_target"] for r in res["trace"]][1:] == [16] * (len(res["trace"]) - 1)


def test_mask_restricts_actions(oracle):
    rng = np.random.default_rng(3)
    mask = (1 << 5) | (1 << 9) | (1 << 22)
    for _ in range(5):
        program = _programs.random_program(rng, extended=True, features=10)
        program["feature_spec_id"] = 3
        res, _ = _run(oracle, program, mask=mask)
        assert all((mask >> r["action"]) & 1 for r in res["trace"])


def test_restart_resets_to_global_best(oracle):
    res, prep = _run(oracle, _program([0], [9]), iterations=6)
    for r in res["trace"]:
        assert r["parent_cost"] == r["global_cost"]           # restart: parent <- global best
    assert res["cost"] <= prep["cost"]


def test_entropy_and_log2_are_exact_functions(oracle):
    L = oracle.lib()
    # uniform row: entropy 1 exactly; one-hot row: 0; log2 of powers of two exact
    assert L.orc_row_entropy_q(np.full(20, 3.0, np.float32), 20, L.orc_log2(20.0)) == 1 << 20
    assert all(L.orc_log2(float(2.0 ** e)) == e for e in range(-60, 60))


def _reference_conditional(oracle, trees, features, masks):
    """controller.py:60-84 restated on top of the joint scorer: per role, the
    tree's scores at the candidate actions prefix + i*stride, legality by the
    stride-wide mask window, the first maximum within 1e-6."""
    prefix = np.zeros(masks.size, np.int64)
    rows = np.arange(masks.size)
    for tree, width, stride in zip(trees, (2, 4, 4), (16, 4, 1)):
        scores, _ = oracle.score(tree, features, np.full(masks.size, 0xFFFFFFFF, np.uint32))
        action = prefix[:, None] + np.arange(width)[None, :] * stride
        values = scores[rows[:, None], action]
        legal = ((masks[:, None] >> action.astype(np.uint32)) & np.uint32((1 << stride) - 1)) != 0
        maximum = np.max(np.where(legal, values, -np.inf), axis=1)
        chosen = np.argmax(legal & (maximum[:, None] - values <= np.float32(1e-6)), axis=1)
        prefix += chosen * stride
    return prefix


@pytest.mark.parametrize("extended", [False, True])
def test_conditional_controllers_follow_the_reference_rule(oracle, extended):
    rng = np.random.default_rng(31 + extended)
    for _ in range(64):
        ctl = _programs.random_conditional(rng, extended=extended)
        features = rng.random((12, 9, 32), dtype=np.float32)
        features[:, :, :] = np.round(features * 4) / 4          # ties happen
        masks = rng.integers(1, 2**32, size=9, dtype=np.uint64).astype(np.uint32)
        masks[:3] = [1, 1 << 31, 0x00FF0000]
        _, actions = oracle.score_conditional(ctl["trees"], features, masks)
        want = _reference_conditional(oracle, ctl["trees"], features, masks)
        assert np.array_equal(actions, want)
        for c in range(masks.size):
            assert (int(masks[c]) >> int(actions[c])) & 1      # the action is legal

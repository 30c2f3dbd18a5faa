"""GP scoring oracle: golden vectors and the reference's score_cpu."""
import numpy as np
import pytest

from tests import _programs


def test_masked_tie_golden(oracle):
    # tests/python/test_native_scoring.py:40-46
    features = np.zeros((12, 3, 32), np.float32)
    program = dict(ir_version=1, numeric_spec_id=1, feature_spec_id=1, opcode=[0], operand=[4], constant_bits=[])
    masks = np.array([0xFFFFFFFF, 1 << 31, 1 << 7], np.uint32)
    _, actions = oracle.score(program, features, masks)
    assert actions.tolist() == [0, 31, 7]


@pytest.mark.parametrize("bad", [
    {"ir_version": 4},
    {"opcode": [0] + [7] * 6, "operand": [0] * 7},
    {"opcode": [0], "operand": [12]},
    {"opcode": [1], "operand": [0], "constant_bits": [0x7FC00000]},
    {"opcode": [0, 0, 3], "operand": [0, 1, 1]},
])
def test_rejected_programs_golden(oracle, bad):
    # tests/python/test_native_scoring.py:57-68 (the rejection cases that reach score_cpu)
    program = dict(ir_version=1, numeric_spec_id=1, feature_spec_id=1, opcode=[0], operand=[4], constant_bits=[])
    program.update(bad)
    with pytest.raises(ValueError):
        oracle.score(program, np.zeros((12, 3, 32), np.float32), np.ones(3, np.uint32))


def test_scores_match_reference_core(oracle, reference_core):
    rng = np.random.default_rng(6677)
    features = rng.random((12, 7, 32), dtype=np.float32)
    masks = rng.integers(1, 0xFFFFFFFF, size=7, dtype=np.uint32)
    masks[:3] = [1, 1 << 31, 0xFFFFFFFF]
    for _ in range(256):
        program = _programs.random_program(rng)
        scores, actions = oracle.score(program, features, masks)
        p = oracle.program_struct(program)
        ref_scores = np.zeros((7, 32), np.float32); ref_actions = np.zeros(7, np.int32)
        opcode = np.array(program["opcode"], np.uint8); operand = np.array(program["operand"], np.uint8)
        consts = np.array(program["constant_bits"], np.uint32).view(np.float32)
        consts = np.ascontiguousarray(consts if consts.size else np.zeros(1, np.float32))
        assert reference_core.ref_score(1, 1, 1, p.length, opcode, operand, p.constants_count, consts,
                                        features, masks, 7, ref_scores, ref_actions) == 0
        assert np.array_equal(scores, ref_scores)
        assert np.array_equal(actions, ref_actions)


def test_extended_grammar_semantics(oracle):
    lib = oracle.lib()
    assert lib.orc_apply_operation(9, 3.0, 0.0, 0.0) == 1.0          # protected division
    assert lib.orc_apply_operation(9, 3.0, 0.5, 0.0) == 6.0
    assert lib.orc_apply_operation(9, 3.0, 0.1, 0.0) == 8.0          # clipped to [-8, 8]
    assert lib.orc_apply_operation(10, 0.5, 1.0, -1.0) == 1.0        # if>0
    assert lib.orc_apply_operation(10, 0.0, 1.0, -1.0) == -1.0
    rng = np.random.default_rng(3)
    features = rng.random((12, 5, 32), dtype=np.float32)
    masks = np.full(5, 0xFFFFFFFF, np.uint32)
    for _ in range(64):
        program = _programs.random_program(rng, extended=True)
        scores, actions = oracle.score(program, features, masks)
        assert np.all(np.abs(scores) <= 8.0)
        assert np.all((actions >= 0) & (actions < 32))

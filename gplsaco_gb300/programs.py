"""Seeded random GP programs in the postfix IR, for initial populations and
tests (the reference grows them with DEAP's genHalfAndHalf,
tests/python/test_native_scoring.py:30-33; here trees are grown directly,
half full and half grow, without DEAP)."""
from __future__ import annotations

import numpy as np

REFERENCE_OPS = {2: 2, 3: 2, 4: 2, 5: 2, 6: 2, 7: 1, 8: 2}
EXTENDED_OPS = {**REFERENCE_OPS, 9: 2, 10: 3}


def _grow(rng, depth, max_depth, ops, features, n_consts, full):
    if depth == max_depth or (not full and depth > 0 and rng.random() < 0.3):
        if n_consts and rng.random() < 0.25:
            return [(1, int(rng.integers(n_consts)))]
        return [(0, int(rng.integers(features)))]
    op = int(rng.choice(list(ops)))
    out = []
    for _ in range(ops[op]):
        out += _grow(rng, depth + 1, max_depth, ops, features, n_consts, full)
    return out + [(op, 0)]


def _stack_peak(code, ops):
    top = peak = 0
    for op, _ in code:
        top = top + 1 if op in (0, 1) else top - ops[op] + 1
        peak = max(peak, top)
    return peak


def random_program(rng, *, extended=False, max_depth=None, features=12, stack_limit=None, feature_spec_id=1):
    ops = EXTENDED_OPS if extended else REFERENCE_OPS
    max_depth = max_depth if max_depth is not None else (6 if extended else 5)
    stack_limit = stack_limit or (16 if extended else 6)
    consts_range = 1.0 if extended else 2.0
    while True:
        n_consts = int(rng.integers(0, 5))
        code = _grow(rng, 0, int(rng.integers(0, max_depth + 1)), ops, features, n_consts, rng.random() < 0.5)
        if len(code) <= 63 and _stack_peak(code, ops) <= stack_limit:
            break
    used = sorted({a for op, a in code if op == 1})
    remap = {a: i for i, a in enumerate(used)}
    code = [(op, remap[a] if op == 1 else a) for op, a in code]
    consts = rng.uniform(-consts_range, consts_range, size=len(used)).astype(np.float32)
    return dict(ir_version=1, numeric_spec_id=2 if extended else 1, feature_spec_id=feature_spec_id,
                opcode=[op for op, _ in code], operand=[a for _, a in code],
                constant_bits=[int(b) for b in consts.view(np.uint32)])

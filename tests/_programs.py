"""Random GP programs for the tests (the generator lives in the package)."""
from gplsaco_gb300.programs import EXTENDED_OPS, REFERENCE_OPS, random_program  # noqa: F401


def random_conditional(rng, extended=False):
    """A conditional_three controller of feature spec 3 whose roles read no
    later decision's descriptor (role 0: not 7, 8; role 1: not 7)."""
    import numpy as _np  # noqa: F401
    trees = []
    for role in range(3):
        t = random_program(rng, extended=extended, max_depth=3, features=10, feature_spec_id=3)
        banned = {0: {7: 9, 8: 9}, 1: {7: 8}}.get(role, {})
        t["operand"] = [banned.get(a, a) if op == 0 else a for op, a in zip(t["opcode"], t["operand"])]
        trees.append(t)
    return {"controller_version": 1, "representation": "conditional_three", "controller_id": 1, "trees": trees}


ROLE_FEATURES_SPEC2 = ((0, 1, 2, 3, 4, 6, 7), (0, 1, 2, 3, 4, 6, 7, 8, 9, 10, 11), tuple(range(12)))


def random_conditional_spec2(rng, extended=False):
    """A conditional_three controller of feature spec 2 whose role trees read
    only their allowed features (python/gp_faco/controller.py:9)."""
    trees = []
    for role, allowed in enumerate(ROLE_FEATURES_SPEC2):
        t = random_program(rng, extended=extended, max_depth=3, features=12, feature_spec_id=2)
        t["operand"] = [allowed[a % len(allowed)] if op == 0 else a for op, a in zip(t["opcode"], t["operand"])]
        trees.append(t)
    return {"controller_version": 1, "representation": "conditional_three", "controller_id": 2, "trees": trees}

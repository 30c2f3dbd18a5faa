"""The GP evolution loop on the postfix IR (the reference's DEAP loop,
python/gp_faco/evolution.py:123-299): operators keep every program valid
under the C ABI's validator and inside the depth/size limits, runs are
reproducible from their seed, the ranking and elites follow the reference's
rules, and the state survives a round trip."""
import ctypes as C
import json

import numpy as np
import pytest

from gplsaco_gb300 import evolution as ev


@pytest.fixture(scope="module")
def validate():
    from gplsaco_gb300 import build, _lib
    from gplsaco_gb300.engine import program_to_c
    build.build()
    lib = _lib.load()

    def check(program):
        p = program_to_c(program)
        return lib.faco_validate_program(C.byref(p)) == 0
    return check


def _score(evo):
    # a deterministic stand-in fitness: prefer small programs reading feature 3
    return [len(t) + (0 if any(op == 0 and a == 3 for op, a in t) else 10) for t in evo.population]


@pytest.mark.parametrize("extended", [False, True])
def test_generations_stay_valid_and_bounded(validate, extended):
    settings = ev.EvolutionSettings(population=24, generations=6, elites=2, extended=extended)
    evo = ev.Evolution(settings, seed=11)
    evo.initialize()
    best = []
    while True:
        for program in evo.programs():
            assert validate(program), program
        for tree in evo.population:
            assert not evo._over_limit(tree)
        evo.begin_panel(f"p{evo.generation}")
        for i, value in enumerate(_score(evo)):
            evo.assign(i, float(value), f"p{evo.generation}", evo.program_ids[i])
        best.append(evo.finish_generation()["fitness"])
        if not evo.advance():
            break
    assert best == sorted(best, reverse=True) or all(b >= best[-1] for b in best)   # elites: never worse
    assert evo.variation_counts["crossovers"] > 0 and evo.variation_counts["mutations"] > 0
    shortlist = evo.shortlist()
    assert len(shortlist) == len({json.dumps(p, sort_keys=True) for p in shortlist})


def test_reproducible_and_state_round_trip():
    settings = ev.EvolutionSettings(population=16, generations=3, elites=1)
    runs = []
    for _ in range(2):
        evo = ev.Evolution(settings, seed=5)
        evo.initialize()
        evo.begin_panel("a")
        for i, v in enumerate(_score(evo)):
            evo.assign(i, float(v), "a", evo.program_ids[i])
        evo.finish_generation()
        evo.advance()
        runs.append(evo)
    assert runs[0].programs() == runs[1].programs()
    state = json.loads(json.dumps(runs[0].state_dict()))
    again = ev.Evolution.from_state_dict(state)
    assert again.programs() == runs[0].programs() and again.generation == 1
    assert again.rng.random() == runs[0].rng.random()


def test_protocol_errors():
    evo = ev.Evolution(ev.EvolutionSettings(population=4, generations=2, elites=1), seed=1)
    with pytest.raises(ValueError):
        evo.begin_panel("x")                      # not initialised
    evo.initialize()
    evo.begin_panel("x")
    with pytest.raises(ValueError):
        evo.assign(0, 1.0, "y", evo.program_ids[0])
    with pytest.raises(ValueError):
        evo.finish_generation()                   # unscored individuals
    evo.assign(0, 1.0, "x", evo.program_ids[0])
    with pytest.raises(ValueError):
        evo.assign(0, 2.0, "x", evo.program_ids[0])   # repeated score
    with pytest.raises(ValueError):
        ev.EvolutionSettings(initial_depth_max=6)
    with pytest.raises(ValueError):
        ev.EvolutionSettings(population=3.0)

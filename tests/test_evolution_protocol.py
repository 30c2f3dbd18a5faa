"""The GP evolution loop against the reference's generation protocol, the
checks of tests/python/test_evolution.py restated for this module's API:
every individual of a generation -- elites and duplicates included -- is
scored on the current panel before the generation ends; the last generation
stays scored; varAnd's operator counts and cloned parents; the static limit
falls back to an exact copy of a parent; a state restored mid-panel goes on
exactly like the original (scores assigned in either order) and leaves the
global random state alone; checkpoints keep a failed program's +inf, are
written atomically, and a state the protocol could not have produced is
refused."""
import copy
import json
import math
import random

import pytest

from gplsaco_gb300 import evolution as ev


def assign_all(evo, panel, reverse=False):
    indices = list(range(len(evo.population)))
    if reverse:
        indices.reverse()
    for i in indices:
        if evo.fitness[i] is None:
            evo.assign(i, float(i), panel, evo.program_ids[i])


def serialized(evo):
    return json.loads(json.dumps(evo.state_dict(), allow_nan=False))


def test_elites_and_duplicates_rescored_and_final_generation_scored():
    evo = ev.Evolution(ev.EvolutionSettings(population=8, generations=3, elites=2, crossover_probability=0,
                                            mutation_probability=0), 31)
    evo.initialize()
    evo.population = [list(evo.population[0]) for _ in evo.population]   # every tree the same
    evo.begin_panel("panel0")
    with pytest.raises(ValueError):
        evo.finish_generation()
    assign_all(evo, "panel0")
    evo.finish_generation()
    assert evo.advance()
    assert all(f is None for f in evo.fitness)
    evo.begin_panel("panel1")
    with pytest.raises(ValueError):
        evo.assign(0, 0.0, "panel0", evo.program_ids[0])
    assign_all(evo, "panel1", reverse=True)
    evo.finish_generation()
    assert evo.advance()
    evo.begin_panel("panel2")
    assign_all(evo, "panel2")
    evo.finish_generation()
    before = serialized(evo)
    assert not evo.advance()
    assert serialized(evo) == before
    assert len(evo.shortlist()) == 1 and all(f is not None for f in evo.fitness)


def test_crossover_and_mutation_counts_and_parents_cloned():
    evo = ev.Evolution(ev.EvolutionSettings(population=8, generations=2, elites=2, crossover_probability=1,
                                            mutation_probability=1), 77)
    evo.initialize()
    evo.begin_panel("g0")
    assign_all(evo, "g0")
    evo.finish_generation()
    originals = evo.population
    snapshot = copy.deepcopy(originals)
    evo.advance()
    # 6 offspring: 3 consecutive pairs crossed, each child mutated
    assert evo.variation_counts["crossovers"] == 3
    assert evo.variation_counts["mutations"] == 6
    assert originals == snapshot
    assert not {id(t) for t in originals} & {id(t) for t in evo.population}
    assert all(not evo._over_limit(t) for t in evo.population) and all(f is None for f in evo.fitness)


def test_static_limit_falls_back_to_an_exact_parent():
    evo = ev.Evolution(ev.EvolutionSettings(population=2, generations=2, elites=0, initial_depth_max=2,
                                            max_nodes=15, mutation_depth_min=5, mutation_depth_max=5), 994)
    evo.initialize()
    parent = evo.population[0]
    observed = 0
    for _ in range(32):
        before = evo.variation_counts["fallbacks"]
        (child,) = evo._limited([evo._mutation(list(parent))], [list(parent)])
        if evo.variation_counts["fallbacks"] > before:
            observed += 1
            assert child == parent
        assert not evo._over_limit(child)
    assert observed > 0


@pytest.mark.parametrize("extended", [False, True])
def test_restored_state_continues_like_the_original(extended):
    global_state = random.getstate()
    evo = ev.Evolution(ev.EvolutionSettings(population=12, generations=3, extended=extended), 1103)
    evo.initialize()
    assert random.getstate() == global_state
    evo.begin_panel("panel0")
    evo.assign(0, 0.5, "panel0", evo.program_ids[0])
    restored = ev.Evolution.from_state_dict(serialized(evo))
    assert serialized(restored) == serialized(evo)
    for generation in range(3):
        panel = f"panel{generation}"
        for current, reverse in ((evo, False), (restored, True)):
            if current.panel_id is None:
                current.begin_panel(panel)
            assign_all(current, panel, reverse)
            current.finish_generation()
            current.advance()
        assert serialized(evo) == serialized(restored)
    assert random.getstate() == global_state
    assert evo.shortlist() == restored.shortlist()


def test_checkpoint_keeps_infinite_fitness_and_is_atomic(tmp_path, monkeypatch):
    evo = ev.Evolution(ev.EvolutionSettings(population=4, generations=2, elites=1), 55)
    evo.initialize()
    evo.begin_panel("g0")
    evo.assign(0, math.inf, "g0", evo.program_ids[0])
    path = tmp_path / "checkpoint.json"
    ev.save_checkpoint(path, evo.state_dict())
    restored = ev.Evolution.from_state_dict(ev.load_checkpoint(path))
    assert restored.fitness[0] == math.inf and restored.fitness[1] is None
    before = path.read_bytes()

    def fail_replace(*args):
        raise OSError("injected before the rename")

    monkeypatch.setattr(ev.os, "replace", fail_replace)
    with pytest.raises(OSError):
        ev.save_checkpoint(path, {"new": "uncommitted"})
    assert path.read_bytes() == before and not list(tmp_path.glob("*.partial"))


def test_states_the_protocol_cannot_produce_are_refused():
    evo = ev.Evolution(ev.EvolutionSettings(population=4, generations=2, elites=1), 99)
    evo.initialize()
    evo.begin_panel("current")
    evo.assign(0, 1.0, "current", evo.program_ids[0])
    stale = serialized(evo)
    stale["population"][0]["evaluated_panel"] = "old"
    with pytest.raises(ValueError):
        ev.Evolution.from_state_dict(stale)
    broken = serialized(evo)
    broken["population"][0]["program"]["operand"][0] = 255
    broken["population"][0]["program"]["opcode"][0] = 0
    with pytest.raises(ValueError):
        ev.Evolution.from_state_dict(broken)
    unscored = serialized(evo)
    unscored["population"][1]["fitness"] = 3.0
    with pytest.raises(ValueError):
        ev.Evolution.from_state_dict(unscored)
    with pytest.raises(ValueError):
        ev.EvolutionSettings(population=4, elites=4)
    assign_all(evo, "current")
    evo.finish_generation()
    ev.Evolution.from_state_dict(serialized(evo))
    broken = serialized(evo)
    broken["winners"][0]["fitness"] = -1e9
    with pytest.raises(ValueError):
        ev.Evolution.from_state_dict(broken)
    early = serialized(evo)
    early["population"][2]["valid"] = False
    early["population"][2]["fitness"] = None
    early["population"][2]["evaluated_panel"] = None
    with pytest.raises(ValueError):
        ev.Evolution.from_state_dict(early)

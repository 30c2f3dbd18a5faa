"""Genetic programming of the colony controllers, driven by the GPU engine.

The reference evolves its controller trees with DEAP
(python/gp_faco/evolution.py:31-299): a half-and-half initial population,
tournament selection with a (fitness, size, program) ranking, elites,
one-point subtree crossover and uniform subtree mutation applied as in
DEAP's varAnd, and static depth/size limits that fall back to a parent.
This module follows that generation protocol and API (EvolutionSettings,
Evolution.initialize / begin_panel / assign / finish_generation / advance /
shortlist / state_dict / from_state_dict) with its own operators working
directly on the postfix IR (DEAP is not a dependency here), and adds
`evolve`, which evaluates each generation as one population batch on the
engine (FacoBatchEngine.evaluate_population_evaluations).

Programs are IR dicts of feature spec 3 (the engine's compact controller)
or, with EvolutionSettings(feature_spec_id=2), of the reference's 12-feature
controller.
"""
from __future__ import annotations

import math
import random
import struct
from dataclasses import asdict, dataclass

import numpy as np

from .programs import EXTENDED_OPS, REFERENCE_OPS

FEATURES = {2: 12, 3: 10}         # terminals of feature spec 2 (the reference's) and 3 (7 + 3 descriptors)


@dataclass(frozen=True)
class EvolutionSettings:
    population: int = 128
    generations: int = 50
    initial_depth_min: int = 1
    initial_depth_max: int = 3
    max_depth: int = 5
    max_nodes: int = 63
    tournament_size: int = 4
    elites: int = 4
    crossover_probability: float = 0.8
    mutation_probability: float = 0.2
    mutation_depth_min: int = 0
    mutation_depth_max: int = 2
    extended: bool = False        # the extended grammar (numeric spec 2) instead of the reference's
    feature_spec_id: int = 3      # 2: the reference's 12-feature controller; 3: the engine's

    def __post_init__(self) -> None:
        ints = {k: v for k, v in asdict(self).items()
                if k not in ("crossover_probability", "mutation_probability", "extended", "feature_spec_id")}
        if any(type(v) is not int for v in ints.values()):
            raise ValueError("evolution counts and tree limits must be integers")
        if not (2 <= self.population and 1 <= self.generations and 0 <= self.elites < self.population
                and 1 <= self.tournament_size
                and 0 <= self.initial_depth_min <= self.initial_depth_max <= self.max_depth <= 5
                and 0 <= self.mutation_depth_min <= self.mutation_depth_max <= self.max_depth
                and 1 <= self.max_nodes <= 63 and type(self.extended) is bool
                and type(self.feature_spec_id) is int and self.feature_spec_id in FEATURES):
            raise ValueError("evolution settings out of range")
        for p in (self.crossover_probability, self.mutation_probability):
            if type(p) not in (int, float) or not math.isfinite(p) or not 0 <= p <= 1:
                raise ValueError("crossover and mutation probabilities must be in [0, 1]")
        # initialisation never needs a redraw: a full binary tree of the
        # initial depth fits the node limit (ternary ops are excluded there)
        if 2 ** (self.initial_depth_max + 1) - 1 > self.max_nodes:
            raise ValueError("the initial depth can exceed the node limit")


# A tree is a postfix token list: (0, feature) | (1, float constant) | (op, None).
def _ops(extended: bool) -> dict:
    return EXTENDED_OPS if extended else REFERENCE_OPS


def _arity(token, ops) -> int:
    return 0 if token[0] in (0, 1) else ops[token[0]]


def _subtree_start(tree, end, ops) -> int:
    need = 1
    j = end
    while True:
        need += _arity(tree[j], ops) - 1
        if need == 0:
            return j
        j -= 1


def _height(tree, ops) -> int:
    stack = []
    for token in tree:
        a = _arity(token, ops)
        if a:
            top = stack[-a:]
            del stack[-a:]
            stack.append(1 + max(top))
        else:
            stack.append(0)
    return stack[0]


def _grow(rng: random.Random, depth: int, height: int, ops: dict, full: bool, min_depth: int = 0,
          features: int = FEATURES[3]) -> list:
    """DEAP's genFull / genGrow: a leaf at the target height, or (grow only,
    from `min_depth` on) with the terminal ratio; terminals are the features
    and one ephemeral constant uniform in [-1, 1] (FP32)."""
    terminals = features + 1
    if depth == height or (not full and depth >= min_depth and rng.random() < terminals / (terminals + len(ops))):
        pick = rng.randrange(terminals)
        if pick == features:
            return [(1, struct.unpack("<f", struct.pack("<f", rng.uniform(-1.0, 1.0)))[0])]
        return [(0, pick)]
    op = rng.choice(sorted(ops))
    out = []
    for _ in range(ops[op]):
        out += _grow(rng, depth + 1, height, ops, full, min_depth, features)
    return out + [(op, None)]


def to_ir(tree, extended: bool, feature_spec_id: int = 3) -> dict:
    constants = [c for op, c in tree if op == 1]
    operands, ci = [], 0
    for op, arg in tree:
        if op == 1:
            operands.append(ci)
            ci += 1
        else:
            operands.append(0 if arg is None else arg)
    return dict(ir_version=1, numeric_spec_id=2 if extended else 1, feature_spec_id=feature_spec_id,
                opcode=[op for op, _ in tree], operand=operands,
                constant_bits=[struct.unpack("<I", struct.pack("<f", c))[0] for c in constants])


def from_ir(program: dict) -> list:
    consts = [struct.unpack("<f", struct.pack("<I", b))[0] for b in program["constant_bits"]]
    tree = []
    for op, arg in zip(program["opcode"], program["operand"]):
        tree.append((0, arg) if op == 0 else (1, consts[arg]) if op == 1 else (op, None))
    return tree


def _key(tree) -> tuple:
    return tuple((op, -1 if arg is None else (arg if op == 0 else struct.pack("<f", arg))) for op, arg in tree)


class Evolution:
    """One evolution run; fitness is minimised (+inf marks a failed program)."""

    def __init__(self, settings: EvolutionSettings, seed: int):
        if type(seed) is not int or not 0 <= seed <= 0xFFFFFFFFFFFFFFFF:
            raise ValueError("the evolution seed must be a uint64")
        self.settings = settings
        self.ops = _ops(settings.extended)
        self.rng = random.Random(seed)
        self.generation = 0
        self.population: list[list] = []
        self.fitness: list[float | None] = []
        self.program_ids: list[str] = []
        self.panel_id: str | None = None
        self.winners: list[dict] = []
        self.variation_counts = {"crossovers": 0, "mutations": 0, "fallbacks": 0}

    # ---- operators --------------------------------------------------------
    def _over_limit(self, tree) -> bool:
        return _height(tree, self.ops) > self.settings.max_depth or len(tree) > self.settings.max_nodes

    def _crossover(self, left, right):
        """One-point crossover (DEAP cxOnePoint): a random non-root subtree of
        each parent swapped; trees of one node are left as they are."""
        if len(left) < 2 or len(right) < 2:
            return left, right
        i, j = self.rng.randrange(len(left) - 1), self.rng.randrange(len(right) - 1)
        si, sj = _subtree_start(left, i, self.ops), _subtree_start(right, j, self.ops)
        a = left[:si] + right[sj:j + 1] + left[i + 1:]
        b = right[:sj] + left[si:i + 1] + right[j + 1:]
        return a, b

    def _mutation(self, tree):
        """Uniform mutation: a random subtree replaced by a new full tree."""
        i = self.rng.randrange(len(tree))
        s = _subtree_start(tree, i, self.ops)
        height = self.rng.randint(self.settings.mutation_depth_min, self.settings.mutation_depth_max)
        return tree[:s] + _grow(self.rng, 0, height, self.ops, True,
                                features=FEATURES[self.settings.feature_spec_id]) + tree[i + 1:]

    def _limited(self, children, parents):
        """Static limit: an offspring over the depth or size limit is replaced
        by a copy of a random parent."""
        out = []
        for child in children:
            if self._over_limit(child):
                self.variation_counts["fallbacks"] += 1
                child = list(self.rng.choice(parents))
            out.append(child)
        return out

    # ---- generation protocol ----------------------------------------------
    def initialize(self) -> None:
        if self.population:
            raise ValueError("the population is already initialised")
        s = self.settings
        init_ops = {o: a for o, a in self.ops.items() if a <= 2}
        self.population = []
        for _ in range(s.population):
            # genHalfAndHalf: full or grow with equal odds, height in [min, max]
            height = self.rng.randint(s.initial_depth_min, s.initial_depth_max)
            full = self.rng.random() < 0.5
            self.population.append(_grow(self.rng, 0, height, init_ops, full, s.initial_depth_min,
                                         FEATURES[s.feature_spec_id]))
        self._reset_ids()

    def _reset_ids(self) -> None:
        self.program_ids = [f"g{self.generation + 1:03d}-i{i + 1:03d}" for i in range(len(self.population))]
        self.fitness = [None] * len(self.population)

    def programs(self) -> list[dict]:
        return [to_ir(tree, self.settings.extended, self.settings.feature_spec_id) for tree in self.population]

    def begin_panel(self, panel_id: str) -> None:
        if not self.population or self.panel_id is not None or not panel_id:
            raise ValueError("a panel cannot begin in this generation state")
        self.panel_id = panel_id
        self.fitness = [None] * len(self.population)

    def assign(self, index: int, value: float, panel_id: str, program_id: str) -> None:
        if panel_id != self.panel_id or self.panel_id is None:
            raise ValueError("the score belongs to another panel")
        if type(index) is not int or not 0 <= index < len(self.population):
            raise ValueError("individual index out of range")
        if self.fitness[index] is not None or self.program_ids[index] != program_id:
            raise ValueError("repeated score or program identity mismatch")
        if type(value) not in (int, float) or math.isnan(value) or value == -math.inf:
            raise ValueError("invalid fitness")
        self.fitness[index] = float(value)

    def _rank(self, i: int) -> tuple:
        if self.fitness[i] is None:
            raise ValueError("an individual has not been evaluated")
        return self.fitness[i], len(self.population[i]), _key(self.population[i])

    def finish_generation(self) -> dict:
        if self.panel_id is None or any(f is None for f in self.fitness):
            raise ValueError("every individual needs its score before the generation ends")
        if len(self.winners) != self.generation:
            raise ValueError("this generation is already archived")
        best = min(range(len(self.population)), key=self._rank)
        result = {"generation": self.generation, "panel_id": self.panel_id,
                  "program": to_ir(self.population[best], self.settings.extended, self.settings.feature_spec_id),
                  "fitness": self.fitness[best] if math.isfinite(self.fitness[best]) else None}
        self.winners.append(result)
        return result

    def advance(self) -> bool:
        if len(self.winners) != self.generation + 1:
            raise ValueError("the generation's winner must be archived first")
        s = self.settings
        if self.generation + 1 == s.generations:
            return False
        order = sorted(range(len(self.population)), key=self._rank)
        elites = [list(self.population[i]) for i in order[:s.elites]]
        parents = [list(self.population[min((self.rng.randrange(len(self.population))
                                             for _ in range(s.tournament_size)), key=self._rank)])
                   for _ in range(s.population - s.elites)]
        offspring = [list(p) for p in parents]
        # varAnd: crossover on consecutive pairs, then mutation of each child
        for i in range(1, len(offspring), 2):
            if self.rng.random() < s.crossover_probability:
                self.variation_counts["crossovers"] += 1
                pair = (offspring[i - 1], offspring[i])
                offspring[i - 1], offspring[i] = self._limited(self._crossover(*pair), pair)
        for i in range(len(offspring)):
            if self.rng.random() < s.mutation_probability:
                self.variation_counts["mutations"] += 1
                offspring[i] = self._limited([self._mutation(offspring[i])], [offspring[i]])[0]
        self.population = elites + offspring
        self.generation += 1
        self.panel_id = None
        self._reset_ids()
        if any(self._over_limit(t) for t in self.population):
            raise RuntimeError("the static limit let an offspring through")
        return True

    def shortlist(self) -> tuple[dict, ...]:
        if (self.generation + 1 != self.settings.generations or len(self.winners) != self.settings.generations
                or any(f is None for f in self.fitness)):
            raise ValueError("only an evaluated final generation forms a shortlist")
        unique = {}
        for program in [w["program"] for w in self.winners] + self.programs():
            unique.setdefault(_key(from_ir(program)), program)
        return tuple(unique[k] for k in sorted(unique))

    def state_dict(self) -> dict:
        return {"version": 1, "settings": asdict(self.settings), "generation": self.generation,
                "panel_id": self.panel_id, "winners": [dict(w) for w in self.winners],
                "rng_state": self.rng.getstate(), "variation_counts": dict(self.variation_counts),
                "population": [{"program": p, "fitness": f, "program_id": i}
                               for p, f, i in zip(self.programs(), self.fitness, self.program_ids)]}

    @classmethod
    def from_state_dict(cls, state: dict) -> "Evolution":
        if state.get("version") != 1:
            raise ValueError("unknown evolution state version")
        evo = cls(EvolutionSettings(**state["settings"]), 0)
        evo.generation = state["generation"]
        evo.panel_id = state["panel_id"]
        evo.winners = [dict(w) for w in state["winners"]]
        rng_state = state["rng_state"]
        evo.rng.setstate((rng_state[0], tuple(rng_state[1]), rng_state[2]))
        evo.variation_counts = dict(state["variation_counts"])
        evo.population = [from_ir(item["program"]) for item in state["population"]]
        evo.fitness = [item["fitness"] for item in state["population"]]
        evo.program_ids = [item["program_id"] for item in state["population"]]
        return evo


def panel_fitness(result: dict, references: np.ndarray) -> float:
    """Mean relative length over the panel (length / reference length)."""
    costs = np.array([item["cost"] for item in result["items"]], np.float64)
    return float(np.mean(costs / references))


def evolve(engine, instance_keys, seeds, references, iterations: int, settings: EvolutionSettings, seed: int,
           log=None) -> Evolution:
    """Runs a whole evolution: every generation is one population batch of
    `iterations` ant batches per colony on `engine` (a FacoBatchEngine with
    colonies = panel size and population_size >= settings.population);
    fitness = mean length relative to `references` over the panel."""
    evo = Evolution(settings, seed)
    evo.initialize()
    references = np.asarray(references, np.float64)
    while True:
        panel = f"g{evo.generation + 1:03d}"
        evo.begin_panel(panel)
        results = engine.evaluate_population_evaluations(instance_keys, seeds, engine.ants * iterations,
                                                         evo.programs())
        for index, result in enumerate(results):
            evo.assign(index, panel_fitness(result, references), panel, evo.program_ids[index])
        winner = evo.finish_generation()
        if log:
            log(f"generation {winner['generation']}: best fitness {winner['fitness']:.6f}")
        if not evo.advance():
            return evo

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

State and checkpoints follow the reference's rules
(python/gp_faco/evolution.py:250-388, python/gp_faco/checkpoint.py:12-69):
a state holds every individual's program, whether it is scored, its score
(a failed program's +inf written as null) and the panel that scored it;
restoring checks the state against the generation protocol (scores only
from the current panel, the archived winner equal to the population's best,
programs valid and inside the limits) and refuses it otherwise; checkpoint
files are written atomically (a temporary file in the same directory,
fsync, rename).  DEAP is not available here, so its operators are restated
on the postfix IR rather than called: runs follow the reference's protocol,
operator order and probabilities, not its random draws bit for bit.
"""
from __future__ import annotations

import json
import math
import os
import random
import struct
from dataclasses import asdict, dataclass
from pathlib import Path

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
        """JSON-ready state (no NaN or infinity: a failed program's score is
        written as null beside valid=True)."""
        population = []
        for tree, f in zip(self.population, self.fitness):
            population.append({"program": to_ir(tree, self.settings.extended, self.settings.feature_spec_id),
                               "valid": f is not None,
                               "fitness": f if f is not None and math.isfinite(f) else None,
                               "evaluated_panel": self.panel_id if f is not None else None})
        return {"version": 1, "settings": asdict(self.settings), "generation": self.generation,
                "panel_id": self.panel_id, "winners": [dict(w) for w in self.winners],
                "rng_state": self.rng.getstate(), "variation_counts": dict(self.variation_counts),
                "population": population}

    def _check_program(self, program) -> list:
        """The program as a tree, or ValueError: the IR of this run's grammar
        and feature spec, one tree, inside the depth and size limits."""
        s = self.settings
        keys = {"ir_version", "numeric_spec_id", "feature_spec_id", "opcode", "operand", "constant_bits"}
        if type(program) is not dict or set(program) != keys:
            raise ValueError("malformed program")
        if (program["ir_version"] != 1 or program["numeric_spec_id"] != (2 if s.extended else 1)
                or program["feature_spec_id"] != s.feature_spec_id):
            raise ValueError("the program belongs to another grammar or feature spec")
        opcode, operand, bits = program["opcode"], program["operand"], program["constant_bits"]
        if (type(opcode) is not list or type(operand) is not list or type(bits) is not list
                or len(opcode) != len(operand) or not opcode):
            raise ValueError("malformed program")
        depth, constants = 0, 0
        for op, arg in zip(opcode, operand):
            if type(op) is not int or type(arg) is not int:
                raise ValueError("malformed program")
            if op == 0:
                if not 0 <= arg < FEATURES[s.feature_spec_id]:
                    raise ValueError("feature operand out of range")
                depth += 1
            elif op == 1:
                if arg != constants:
                    raise ValueError("constants out of order")
                constants += 1
                depth += 1
            elif op in self.ops:
                if depth < self.ops[op]:
                    raise ValueError("operator without operands")
                depth += 1 - self.ops[op]
            else:
                raise ValueError("unknown opcode")
        if depth != 1 or constants != len(bits) or any(type(b) is not int or not 0 <= b < 2**32 for b in bits):
            raise ValueError("malformed program")
        tree = from_ir(program)
        if any(op == 1 and not math.isfinite(c) for op, c in tree):
            raise ValueError("non-finite constant")
        if self._over_limit(tree):
            raise ValueError("the program exceeds the tree limits")
        return tree

    @classmethod
    def from_state_dict(cls, state: dict) -> "Evolution":
        """Restores a state, refusing one that the generation protocol could
        not have produced (the reference's checks,
        python/gp_faco/evolution.py:274-385)."""
        expected = {"version", "settings", "generation", "panel_id", "winners", "rng_state", "variation_counts",
                    "population"}
        if type(state) is not dict or set(state) != expected or state["version"] != 1:
            raise ValueError("unknown evolution state structure")
        evo = cls(EvolutionSettings(**state["settings"]), 0)
        s = evo.settings
        generation = state["generation"]
        if type(generation) is not int or not 0 <= generation < s.generations:
            raise ValueError("generation out of range")
        evo.generation = generation
        panel = state["panel_id"]
        if panel is not None and (type(panel) is not str or not panel):
            raise ValueError("invalid panel identity")
        evo.panel_id = panel
        items = state["population"]
        if type(items) is not list or len(items) != s.population:
            raise ValueError("population size differs from the settings")
        for item in items:
            if type(item) is not dict or set(item) != {"program", "valid", "fitness", "evaluated_panel"} \
                    or type(item["valid"]) is not bool:
                raise ValueError("malformed individual")
            tree = evo._check_program(item["program"])
            value = item["fitness"]
            if item["valid"]:
                if panel is None or item["evaluated_panel"] != panel:
                    raise ValueError("a score from another panel")
                if value is not None and (type(value) not in (int, float) or not math.isfinite(value)):
                    raise ValueError("a score is finite or null (a failed program)")
                fitness = math.inf if value is None else float(value)
            else:
                if value is not None or item["evaluated_panel"] is not None:
                    raise ValueError("an unscored individual carries a score or a panel")
                fitness = None
            evo.population.append(tree)
            evo.fitness.append(fitness)
        evo.program_ids = [f"g{generation + 1:03d}-i{i + 1:03d}" for i in range(s.population)]
        winners = state["winners"]
        if type(winners) is not list or len(winners) not in (generation, generation + 1):
            raise ValueError("winner count does not match the generation")
        for index, w in enumerate(winners):
            if (type(w) is not dict or set(w) != {"generation", "panel_id", "program", "fitness"}
                    or w["generation"] != index or type(w["panel_id"]) is not str or not w["panel_id"]
                    or (w["fitness"] is not None
                        and (type(w["fitness"]) not in (int, float) or not math.isfinite(w["fitness"])))):
                raise ValueError("malformed winner record")
            evo._check_program(w["program"])
        if len(winners) == generation + 1:
            if panel is None or any(f is None for f in evo.fitness):
                raise ValueError("a winner archived before the whole generation was scored")
            best = min(range(s.population), key=evo._rank)
            best_fitness = evo.fitness[best]
            if (winners[-1]["panel_id"] != panel
                    or _key(from_ir(winners[-1]["program"])) != _key(evo.population[best])
                    or winners[-1]["fitness"] != (best_fitness if math.isfinite(best_fitness) else None)):
                raise ValueError("the current winner is not the population's best")
        evo.winners = [dict(w) for w in winners]
        counts = state["variation_counts"]
        if (type(counts) is not dict or set(counts) != set(evo.variation_counts)
                or any(type(v) is not int or v < 0 for v in counts.values())):
            raise ValueError("invalid variation counts")
        evo.variation_counts = dict(counts)
        evo.rng.setstate(_tuples(state["rng_state"]))
        return evo


def _tuples(value):
    return tuple(_tuples(v) for v in value) if isinstance(value, (list, tuple)) else value


def _unique_pairs(pairs):
    out = {}
    for key, item in pairs:
        if key in out:
            raise ValueError("duplicate key in the checkpoint")
        out[key] = item
    return out


def save_checkpoint(path, state: dict) -> None:
    """Writes {"checkpoint_version": 2, "state": state} as JSON, atomically:
    a temporary file in the target's directory, flushed and fsynced, renamed
    over the target, then the directory fsynced.  A failure leaves the old
    file as it was and no temporary file behind."""
    if type(state) is not dict:
        raise ValueError("a checkpoint state is a JSON object")
    normalized = json.loads(json.dumps(state, allow_nan=False), object_pairs_hook=_unique_pairs)
    payload = json.dumps({"checkpoint_version": 2, "state": normalized}, sort_keys=True, separators=(",", ":"),
                         allow_nan=False) + "\n"
    target = Path(path).resolve()
    target.parent.mkdir(parents=True, exist_ok=True)
    temporary = target.with_name(f".{target.name}.{os.getpid()}.{os.urandom(8).hex()}.partial")
    try:
        with temporary.open("x", encoding="utf-8") as stream:
            stream.write(payload)
            stream.flush()
            os.fsync(stream.fileno())
        os.replace(temporary, target)
        directory = os.open(target.parent, os.O_RDONLY | os.O_DIRECTORY)
        try:
            os.fsync(directory)
        finally:
            os.close(directory)
    finally:
        temporary.unlink(missing_ok=True)


def load_checkpoint(path) -> dict:
    """The state of a checkpoint file written by save_checkpoint."""
    envelope = json.loads(Path(path).read_text(encoding="utf-8"), object_pairs_hook=_unique_pairs)
    if (type(envelope) is not dict or set(envelope) != {"checkpoint_version", "state"}
            or envelope["checkpoint_version"] != 2 or type(envelope["state"]) is not dict):
        raise ValueError("unknown checkpoint structure")
    return envelope["state"]


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

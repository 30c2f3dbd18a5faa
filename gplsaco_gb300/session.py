"""GpuSession.solve -- the call pattern of the reference's resident solve
session (python/gp_faco/gpu_session.py:62-129), without its site-specific GPU
leasing: one engine per instance size, instances registered once, a fixed
panel of (instance, seed) pairs solved for `iterations` ant batches."""
from __future__ import annotations

import time

import numpy as np

from .engine import FacoBatchEngine, FixedFacoSettings, faco_ants


class Instance:
    """Minimal problem record: numeric id and f64 [n,2] integer coordinates."""

    def __init__(self, numeric_id: int, coordinates):
        self.numeric_id = int(numeric_id)
        self.coordinates = np.ascontiguousarray(coordinates, dtype=np.float64)
        self.dimension = self.coordinates.shape[0]


class GpuSession:
    def __init__(self, *, colonies: int = 32, settings: FixedFacoSettings | None = None, device: int = 0):
        self.colonies = colonies
        self.settings = settings
        self.device = device
        self.engines: dict[int, FacoBatchEngine] = {}
        self.registered: dict[int, set] = {}
        self.population_engines: dict[tuple, FacoBatchEngine] = {}
        self.population_registered: dict[tuple, set] = {}

    def _engine(self, n: int) -> FacoBatchEngine:
        if n not in self.engines:
            base = self.settings or FixedFacoSettings()
            settings = FixedFacoSettings(**{**base.__dict__, "ants": base.ants or faco_ants(n)})
            self.engines[n] = FacoBatchEngine(n, self.colonies, settings, device=self.device)
            self.registered[n] = set()
        return self.engines[n]

    def solve(self, problems, pairs, iterations, controller=None, *, checkpoints=()):
        if len(pairs) != self.colonies:
            raise ValueError("FACO needs one complete fixed panel")
        if controller is not None and not ("uniform_mne" in controller or "opcode" in controller
                                           or "controller_version" in controller):
            raise ValueError("unknown controller: expected {'uniform_mne': m}, a program or a controller dict")
        n = problems[pairs[0][0]].dimension
        engine = self._engine(n)
        before = time.perf_counter()
        for name, _ in pairs:
            problem = problems[name]
            if problem.dimension != n:
                raise ValueError("the panel mixes instance sizes")
            if name not in self.registered[n]:
                engine.register_problem(problem.numeric_id, problem.coordinates)
                self.registered[n].add(name)
        registration_seconds = time.perf_counter() - before
        keys = np.asarray([problems[name].numeric_id for name, _ in pairs], dtype=np.uint64)
        seeds = np.asarray([seed for _, seed in pairs], dtype=np.uint64)
        before = time.perf_counter()
        if controller is None or "uniform_mne" in controller:
            result = engine.evaluate_faco_evaluations(
                keys, seeds, engine.ants * iterations, 8 if controller is None else controller["uniform_mne"],
                "cached", checkpoint_iterations=list(checkpoints))
        elif "controller_version" in controller:
            result = engine.evaluate_controller_evaluations(keys, seeds, engine.ants * iterations, controller)
        else:
            result = engine.evaluate_program_evaluations(keys, seeds, engine.ants * iterations, controller, "cached",
                                                         checkpoint_iterations=list(checkpoints))
        return result, {"registration_seconds": registration_seconds,
                        "solve_seconds": time.perf_counter() - before}

    def solve_population(self, problems, pairs, iterations, programs, *, experiment_mask=0xFFFFFFFF):
        """solve_population (gpu_session.py:139-171): every program runs the
        whole panel in one batch; returns one result dict per program."""
        if len(pairs) != self.colonies or not 1 <= len(programs) <= 128:
            raise ValueError("a population shard needs the complete panel and 1..128 programs")
        n = problems[pairs[0][0]].dimension
        key = n, len(programs)
        before = time.perf_counter()
        if key not in self.population_engines:
            base = self.settings or FixedFacoSettings()
            settings = FixedFacoSettings(**{**base.__dict__, "ants": base.ants or faco_ants(n)})
            self.population_engines[key] = FacoBatchEngine(n, self.colonies, settings,
                                                           population_size=len(programs), device=self.device)
            self.population_registered[key] = set()
        engine = self.population_engines[key]
        for name in dict.fromkeys(name for name, _ in pairs):
            if name not in self.population_registered[key]:
                problem = problems[name]
                if problem.dimension != n:
                    raise ValueError("the panel mixes instance sizes")
                engine.register_problem(problem.numeric_id, problem.coordinates)
                self.population_registered[key].add(name)
        registration = time.perf_counter() - before
        keys = np.asarray([problems[name].numeric_id for name, _ in pairs], dtype=np.uint64)
        seeds = np.asarray([seed for _, seed in pairs], dtype=np.uint64)
        before = time.perf_counter()
        result = engine.evaluate_population_evaluations(keys, seeds, engine.ants * iterations, programs,
                                                        experiment_mask)
        return result, {"registration_seconds": registration, "solve_seconds": time.perf_counter() - before}

    def close(self):
        for engine in list(self.engines.values()) + list(self.population_engines.values()):
            engine.close()
        self.engines.clear()
        self.population_engines.clear()

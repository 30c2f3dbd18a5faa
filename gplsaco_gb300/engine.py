"""Reference-facing host API, mirroring the pybind11 module gp_faco_ext of
LinHuanli/GPLSACO (cpp/src/bindings.cpp:500-1046): FixedFacoSettings,
FacoBatchEngine (register_problem, evaluate_faco_evaluations), score_cuda, with
the same argument meaning, result dictionary keys and error behaviour
(ValueError for invalid input, RuntimeError for CUDA failures).  Everything
runs through the C ABI of the CUDA library; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import math
import struct
import threading
from dataclasses import dataclass

import numpy as np

from . import _lib


def _exact_int(value, name: str, lo: int = 0, hi: int = 2**64 - 1) -> int:
    # JSON bools are ints in Python; the reference rejects them (bindings.cpp:131-145)
    if type(value) is not int:
        raise ValueError(f"{name} must be an int (not bool/float)")
    if not lo <= value <= hi:
        raise ValueError(f"{name} out of range")
    return value


@dataclass
class FixedFacoSettings:
    """FixedFacoSettings (cpp/include/gp_faco/fixed_faco_gpu.hpp:10-21)."""
    ants: int = 0
    primary_width: int = 16
    backup_width: int = 64
    ls_width: int = 20
    beta: float = 1.0
    retention: float = 0.5
    p_best: float = 0.1
    epoch_source_probability: float = 0.01
    ls_evaluation_limit: int = 100000
    initial_ls_evaluation_limit: int = 100000
    ls_mode: int = _lib.FACO_LS_TWO_OPT
    autotune: int = 1
    workspace: int = 0      # 0 auto, 1 shared memory, 2 global memory (ant tour/inverse placement)
    force_fingerprint_collisions: int = 0   # diagnostic: all 12-feature-controller fingerprints 0
    chains: int = 0         # independent colony chains per graph (0 auto); results do not depend on it
    follow: int = 0         # 0 auto, 1 off, 2 on: parent-following construction steps in batches
                            # (auto: when every ant warp fits in one wave); results do not depend on it

    def to_c(self) -> _lib.Settings:
        s = _lib.Settings()
        for name in ("ants", "primary_width", "backup_width", "ls_width", "ls_evaluation_limit",
                     "initial_ls_evaluation_limit", "ls_mode", "autotune", "workspace",
                     "force_fingerprint_collisions", "chains", "follow"):
            setattr(s, name, _exact_int(getattr(self, name), name))
        for name in ("beta", "retention", "p_best", "epoch_source_probability"):
            value = getattr(self, name)
            if type(value) not in (int, float) or not math.isfinite(value):
                raise ValueError(f"{name} must be a finite number")
            setattr(s, name, float(value))
        return s


def faco_ants(dimension: int) -> int:
    """64 * ceil(sqrt(n)/16) ants (python/gp_faco/worker.py:30-34)."""
    if type(dimension) is not int or dimension < 3:
        raise ValueError("TSP size must be an int >= 3")
    return 64 * (math.isqrt(dimension - 1) // 16 + 1)


def _u64_array(a, name: str) -> np.ndarray:
    if not isinstance(a, np.ndarray) or a.dtype != np.uint64 or a.ndim != 1 or not a.flags.c_contiguous:
        raise ValueError(f"{name} must be a contiguous 1-D uint64 array")
    return a


class FacoBatchEngine:
    """FacoBatchEngine(dimension, colonies, settings, population_size=1)
    (bindings.cpp:558-573).

    `dimension` is the largest instance size accepted; instances of different
    sizes may share an evaluation.  `colonies` is the panel size; an engine
    with population_size P holds P copies of the panel, one per individual of
    evaluate_population_evaluations.  One evaluation at a time per engine.
    """

    def __init__(self, dimension, colonies, settings: FixedFacoSettings, constraint_mode="unrestricted",
                 population_size=1, device: int = 0):
        _exact_int(dimension, "dimension")
        _exact_int(colonies, "colonies", 1, 2**32 - 1)
        _exact_int(population_size, "population_size", 1, 128)
        if constraint_mode != "unrestricted":
            raise ValueError("only the unrestricted candidate graph is supported")
        self._L = _lib.load()
        self._handle = C.c_void_p()
        _lib.check(self._L.faco_engine_create(dimension, colonies * population_size, C.byref(settings.to_c()),
                                              device, C.byref(self._handle)))
        self.dimension, self.colonies, self.population_size = dimension, colonies, population_size
        self.settings = settings
        self.ants = settings.ants or faco_ants(dimension)
        self._sizes: dict[int, int] = {}
        self._spec = 0          # feature spec of the active stepwise evaluation (0: plain FACO)
        self._lock = threading.Lock()

    def close(self) -> None:
        if self._handle:
            self._L.faco_engine_destroy(self._handle)
            self._handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def register_problem(self, instance_key, coordinates) -> dict:
        """register_problem(instance_key, coordinates f64[n,2]) (bindings.cpp:623-638)."""
        key = _exact_int(instance_key, "instance_key")
        if (not isinstance(coordinates, np.ndarray) or coordinates.dtype != np.float64 or coordinates.ndim != 2
                or coordinates.shape[1] != 2 or not coordinates.flags.c_contiguous):
            raise ValueError("coordinates must be a C-contiguous float64 [n, 2] array")
        info = _lib.Registration()
        _lib.check(self._L.faco_register_problem(self._handle, key, coordinates.ctypes.data, coordinates.shape[0],
                                                 C.byref(info)))
        self._sizes[key] = coordinates.shape[0]
        return {"cheap_seconds": info.cheap_seconds, "preparation_seconds": info.preparation_seconds,
                "initial_cost": int(info.initial_cost)}

    def problem_rows(self, instance_key) -> dict:
        n = self._sizes[instance_key]
        s = self.settings
        k = min(s.primary_width, n - 1)
        b = min(s.backup_width, n - 1 - k)
        w = min(s.ls_width, n - 1)
        out = dict(initial_tour=np.zeros(n, np.uint32), primary=np.zeros((n, k), np.uint32),
                   backup=np.zeros((n, max(b, 1)), np.uint32), ls=np.zeros((n, w), np.uint32))
        _lib.check(self._L.faco_problem_rows(self._handle, instance_key, *(out[x].ctypes.data for x in
                                                                          ("initial_tour", "primary", "backup",
                                                                           "ls"))))
        out["backup"] = out["backup"][:, :b]
        return out

    def evaluate_faco_evaluations(self, instance_keys, seeds, evaluation_limit_per_colony, mne=8,
                                  preparation_mode="cached", *, checkpoint_iterations=(), profile_events_only=False,
                                  trace=False) -> dict:
        """evaluate_faco_evaluations (bindings.cpp:701-720): plain FACO with a
        constant MNE target, budget in ant-tour evaluations per colony."""
        mne = _exact_int(mne, "mne", 1, 2**32 - 1)
        return self._evaluate(instance_keys, seeds, evaluation_limit_per_colony, mne, preparation_mode,
                              checkpoint_iterations, profile_events_only, trace, None, 0xFFFFFFFF)

    def evaluate_program_evaluations(self, instance_keys, seeds, evaluation_limit_per_colony, program,
                                     preparation_mode="cached", experiment_mask=0xFFFFFFFF, *,
                                     checkpoint_iterations=(), initial_mne=8, trace=False,
                                     decision_iterations=()) -> dict:
        """evaluate_program_evaluations (bindings.cpp:721-757): every colony is
        driven by one GP controller program -- feature spec 2 (the
        reference's 12 features) or 3 (this engine's).  decision_iterations
        (spec 2) records the decisions before the given 1-based batches."""
        return self._programs(_u64_array(instance_keys, "instance_keys"), _u64_array(seeds, "seeds"),
                              evaluation_limit_per_colony, [program], experiment_mask, checkpoint_iterations,
                              initial_mne, trace, preparation_mode, decisions=decision_iterations)

    def evaluate_controller_evaluations(self, instance_keys, seeds, evaluation_limit_per_colony, controller,
                                        experiment_mask=0xFFFFFFFF, *, decision_iterations=()) -> dict:
        """evaluate_controller_evaluations (bindings.cpp:758-775,
        cuda/batch_engine.cu:439-447): a controller dict (read_controller,
        bindings.cpp:58-73) -- a bare program, or {controller_version: 1,
        representation, controller_id, trees}.  A joint_single controller is
        its one tree; a conditional_three controller's role trees pick restart,
        start region and MNE level in turn (faco_evaluate_controllers).
        decision_iterations (feature spec 2) records the decisions before the
        given 1-based batches under "decisions"."""
        if not isinstance(controller, dict):
            raise ValueError("controller must be a dict")
        if "opcode" in controller:
            program = controller
        else:
            if (len(controller) != 4 or type(controller.get("controller_version")) is not int
                    or controller["controller_version"] != 1 or "controller_id" not in controller
                    or "trees" not in controller):
                raise ValueError("unknown controller version or fields")
            kind = controller.get("representation")
            if kind not in ("joint_single", "conditional_three"):
                raise ValueError("unknown controller representation")
            trees = list(controller["trees"])
            if len(trees) != (3 if kind == "conditional_three" else 1):
                raise ValueError("wrong number of role trees for the controller representation")
            if kind == "conditional_three":
                return self._controllers(_u64_array(instance_keys, "instance_keys"), _u64_array(seeds, "seeds"),
                                         evaluation_limit_per_colony, [controller], experiment_mask,
                                         decision_iterations)
            program = trees[0]
        return self._programs(_u64_array(instance_keys, "instance_keys"), _u64_array(seeds, "seeds"),
                              evaluation_limit_per_colony, [program], experiment_mask, (), 8, False,
                              "cached_charged", decisions=decision_iterations)

    def evaluate_population_evaluations(self, instance_keys, seeds, evaluation_limit_per_colony, programs,
                                        experiment_mask=0xFFFFFFFF, *, factorial_policy=None,
                                        profile_events_only=False, checkpoint_iterations=(), initial_mne=8,
                                        trace=False) -> list:
        """evaluate_population_evaluations (bindings.cpp:776-817,
        cuda/batch_engine.cu:379-437): every program (individual) runs the
        whole panel of `colonies` (instance, seed) tasks; all individuals share
        one batch (colony i*colonies + j = individual i, task j).  Returns one
        result dict per individual; its time is an equal share of the batch
        (`population_actual_seconds` keeps the batch's)."""
        if not isinstance(programs, (list, tuple)) or not 1 <= len(programs) <= self.population_size:
            raise ValueError("the population needs 1..population_size programs")
        if factorial_policy is not None:
            raise ValueError("factorial policies are not supported by this engine")
        keys = _u64_array(instance_keys, "instance_keys")
        seeds = _u64_array(seeds, "seeds")
        if keys.size != self.colonies or seeds.size != self.colonies:
            raise ValueError("the population entry needs the complete shared panel")
        count = len(programs)
        if any(isinstance(p, dict) and "opcode" not in p for p in programs):
            if checkpoint_iterations or trace or initial_mne != 8:
                raise ValueError("controller populations take no checkpoints, traces or initial MNE")
            batch = self._controllers(np.tile(keys, count), np.tile(seeds, count), evaluation_limit_per_colony,
                                      programs, experiment_mask)
        else:
            batch = self._programs(np.tile(keys, count), np.tile(seeds, count), evaluation_limit_per_colony,
                                   programs, experiment_mask, checkpoint_iterations, initial_mne, trace,
                                   "cached_charged", profile_events_only)
        out = []
        G = self.colonies
        for i in range(count):
            part = dict(batch)
            share = batch["actual_seconds"] / count
            part["items"] = [dict(it, completed_seconds=it["completed_seconds"] / count)
                             for it in batch["items"][i * G:(i + 1) * G]]
            work = batch["colony_work"][i * G:(i + 1) * G]
            part.update(population_size=count, population_actual_seconds=batch["actual_seconds"],
                        time_accounting="equal_share_of_population_batch", actual_seconds=share,
                        elapsed_seconds=share, total_tour_evaluations=batch["completed_tour_evaluations_per_colony"] * G,
                        completed_construction_steps=int(work[:, 0].sum()),
                        completed_ls_evaluations=int(work[:, 1].sum()), reversed_elements=int(work[:, 2].sum()),
                        colony_work=work)
            if "control_states" in batch:
                part["control_states"] = batch["control_states"][i * G:(i + 1) * G]
            if "checkpoints" in batch:
                part["checkpoints"] = [{"iterations": cp["iterations"], "tours": cp["tours"][i * G:(i + 1) * G]}
                                       for cp in batch["checkpoints"]]
            if trace:
                part["trace"] = batch["trace"][:, i * G:(i + 1) * G]
            out.append(part)
        return out

    def _controllers(self, keys, seeds, limit, controllers, experiment_mask, decisions=()) -> dict:
        arr, kinds = controller_arrays(controllers)
        mask = _exact_int(experiment_mask, "experiment_mask", 1, 0xFFFFFFFF)
        return self._evaluate(keys, seeds, limit, 8, "cached_charged", (), False, False, (arr, kinds), mask,
                              decisions)

    def _programs(self, keys, seeds, limit, programs, experiment_mask, checkpoint_iterations, initial_mne, trace,
                  preparation_mode, profile_events_only=False, decisions=()) -> dict:
        if not isinstance(programs, (list, tuple)) or not programs:
            raise ValueError("programs must be a non-empty list of IR dicts")
        mask = _exact_int(experiment_mask, "experiment_mask", 1, 0xFFFFFFFF)
        mne = _exact_int(initial_mne, "initial_mne", 1, 2**32 - 1)
        arr = (_lib.Program * len(programs))(*[program_to_c(p) for p in programs])
        if any(p.feature_spec_id not in (2, 3) for p in arr) or len({p.feature_spec_id for p in arr}) != 1:
            raise ValueError("controller programs use one feature spec, 2 or 3")
        return self._evaluate(keys, seeds, limit, mne, preparation_mode, checkpoint_iterations, profile_events_only,
                              trace, arr, mask, decisions)

    def _evaluate(self, instance_keys, seeds, evaluation_limit_per_colony, mne, preparation_mode,
                  checkpoint_iterations, profile_events_only, trace, programs, mask, decisions=()) -> dict:
        keys = _u64_array(instance_keys, "instance_keys")
        seeds = _u64_array(seeds, "seeds")
        if keys.size != seeds.size:
            raise ValueError("instance_keys and seeds differ in length")
        limit = _exact_int(evaluation_limit_per_colony, "evaluation_limit_per_colony")
        if preparation_mode not in ("cached", "cached_charged"):
            raise ValueError("unknown preparation mode")
        if type(profile_events_only) is not bool or type(trace) is not bool:
            raise ValueError("flags must be bool")
        cps = np.asarray([_exact_int(c, "checkpoint") for c in checkpoint_iterations], dtype=np.uint64)
        points = np.asarray([_exact_int(d, "decision iteration", 1, 2**32 - 1) for d in decisions], dtype=np.uint32)
        count = keys.size
        D = self.dimension
        iterations = limit // self.ants if self.ants else 0
        tours = np.zeros((count, D), np.uint32)
        costs = np.zeros(count, np.int64)
        trace_rows = np.zeros((iterations, count), _lib.TRACE_DTYPE) if trace else None
        cp_tours = np.zeros((cps.size, count, D), np.uint32) if cps.size else None
        work = np.zeros((count, 3), np.uint64)
        control = np.zeros(count, _lib.CONTROL_STATE_DTYPE)
        out = _lib.Outputs(tours.ctypes.data, costs.ctypes.data, _lib.ptr(trace_rows), _lib.ptr(cp_tours))
        out.colony_work = work.ctypes.data
        out.control_states = control.ctypes.data
        dec = None
        if points.size:
            dec = dict(features=np.zeros((points.size, count, 12, 32), np.float32),
                       scores=np.zeros((points.size, count, 32), np.float32),
                       masks=np.zeros((points.size, count), np.uint32),
                       actions=np.zeros((points.size, count), np.int32))
            out.decision_iterations = points.ctypes.data
            out.n_decisions = points.size
            out.decision_features = dec["features"].ctypes.data
            out.decision_scores = dec["scores"].ctypes.data
            out.decision_masks = dec["masks"].ctypes.data
            out.decision_actions = dec["actions"].ctypes.data
        if not self._lock.acquire(blocking=False):
            raise RuntimeError("only one active evaluation per engine")
        try:
            cp_ptr = _lib.ptr(cps) if cps.size else None
            if programs is None:
                code = self._L.faco_evaluate(self._handle, keys.ctypes.data, seeds.ctypes.data, count, limit, mne,
                                             cp_ptr, cps.size, C.byref(out))
            elif isinstance(programs, tuple):
                arr, kinds = programs
                code = self._L.faco_evaluate_controllers(self._handle, keys.ctypes.data, seeds.ctypes.data, count,
                                                         limit, C.cast(arr, C.c_void_p), kinds.ctypes.data,
                                                         kinds.size, mask, mne, cp_ptr, cps.size, C.byref(out))
            else:
                code = self._L.faco_evaluate_programs(self._handle, keys.ctypes.data, seeds.ctypes.data, count, limit,
                                                      C.cast(programs, C.c_void_p), len(programs), mask, mne, cp_ptr,
                                                      cps.size, C.byref(out))
            _lib.check(code)
        finally:
            self._lock.release()
        items = []
        for c in range(count):
            n = self._sizes[int(keys[c])]
            items.append({"has_incumbent": True, "tour": tours[c, :n].tolist(), "cost": int(costs[c]),
                          "completed_seconds": out.solve_seconds})
        result = {
            "items": items,
            "budget_seconds": None,
            "budget_kind": "search_tour_evaluations",
            "evaluation_limit_per_colony": limit,
            "completed_tour_evaluations_per_colony": int(out.completed_batches) * self.ants,
            "total_tour_evaluations": int(out.completed_batches) * self.ants * count,
            "completed_batches": int(out.completed_batches),
            "completed_construction_steps": int(out.construction_steps),
            "completed_ls_evaluations": int(out.ls_evaluations),
            "reversed_elements": int(out.reversed_elements),
            "colony_work": work,
            "production_kernel_milliseconds": {"iteration_loop": out.kernel_milliseconds},
            "elapsed_seconds": out.solve_seconds,
            "actual_seconds": out.solve_seconds,
            "preparation_mode": preparation_mode,
        }
        if programs is not None:
            spec, kinds = _feature_spec(programs)
            result["control_states"] = control_state_dicts(control, spec)
            if dec is not None:
                result["decisions"] = decision_rows(points, dec, kinds, count)
        if cps.size:
            result["checkpoints"] = [
                {"iterations": int(cps[i]),
                 "tours": [cp_tours[i, c, :self._sizes[int(keys[c])]].tolist() for c in range(count)]}
                for i in range(cps.size)]
        if trace:
            result["trace"] = trace_rows
        return result

    # ---- stepwise evaluation (caller-driven ant batches) -------------------
    def begin(self, instance_keys, seeds, mne=8, *, trace_iterations: int = 0) -> None:
        keys = _u64_array(instance_keys, "instance_keys")
        seeds = _u64_array(seeds, "seeds")
        if keys.size != seeds.size:
            raise ValueError("instance_keys and seeds differ in length")
        _exact_int(mne, "mne", 1, 2**32 - 1)
        _exact_int(trace_iterations, "trace_iterations", 0, 2**32 - 1)
        _lib.check(self._L.faco_begin(self._handle, keys.ctypes.data, seeds.ctypes.data, keys.size, mne,
                                      trace_iterations))
        self._spec = 0
        self._active = (keys.copy(), trace_iterations, 0)

    def step(self, iterations: int) -> None:
        """Enqueues `iterations` ant batches on the engine stream (asynchronous)."""
        _exact_int(iterations, "iterations", 0, 2**32 - 1)
        _lib.check(self._L.faco_step(self._handle, iterations))
        keys, cap, done = self._active
        self._active = (keys, cap, done + iterations)

    def step_timed(self, iterations: int) -> tuple[float, float]:
        """Runs ant batches with a CUDA event around every kernel; returns the
        summed device milliseconds (ant kernel, colony update)."""
        _exact_int(iterations, "iterations", 0, 2**32 - 1)
        ant_ms, update_ms = C.c_double(), C.c_double()
        _lib.check(self._L.faco_step_timed(self._handle, iterations, C.byref(ant_ms), C.byref(update_ms)))
        keys, cap, done = self._active
        self._active = (keys, cap, done + iterations)
        return ant_ms.value, update_ms.value

    def launch_plan(self) -> dict:
        """The active (or most recent) evaluation's size classes, colony
        chains, iterations per graph replay and kernel launches per iteration."""
        plan = _lib.LaunchPlan()
        _lib.check(self._L.faco_get_launch_plan(self._handle, C.byref(plan)))
        return {name: int(getattr(plan, name)) for name, _ in plan._fields_}

    def finish(self) -> dict:
        keys, cap, done = self._active
        count, D = keys.size, self.dimension
        tours = np.zeros((count, D), np.uint32)
        costs = np.zeros(count, np.int64)
        trace_rows = np.zeros((min(cap, done), count), _lib.TRACE_DTYPE) if cap else None
        work = np.zeros((count, 3), np.uint64)
        control = np.zeros(count, _lib.CONTROL_STATE_DTYPE)
        out = _lib.Outputs(tours.ctypes.data, costs.ctypes.data, _lib.ptr(trace_rows), None)
        out.colony_work = work.ctypes.data
        out.control_states = control.ctypes.data
        self._active = None
        _lib.check(self._L.faco_finish(self._handle, C.byref(out)))
        res = {"tours": [tours[c, :self._sizes[int(keys[c])]] for c in range(count)], "costs": costs,
               "completed_batches": int(out.completed_batches),
               "construction_steps": int(out.construction_steps), "ls_evaluations": int(out.ls_evaluations),
               "reversed_elements": int(out.reversed_elements), "colony_work": work, "trace": trace_rows}
        if self._spec:
            res["control_states"] = control_state_dicts(control, self._spec)
        return res

    def begin_programs(self, instance_keys, seeds, programs, experiment_mask=0xFFFFFFFF, *, initial_mne=8,
                       total_iterations, trace_iterations: int = 0) -> None:
        """begin() for GP-controlled colonies (programs as in
        evaluate_population_evaluations, replicated panel order)."""
        keys = _u64_array(instance_keys, "instance_keys")
        seeds = _u64_array(seeds, "seeds")
        if keys.size != seeds.size:
            raise ValueError("instance_keys and seeds differ in length")
        arr = self._program_array(programs)
        self._spec = arr[0].feature_spec_id
        _lib.check(self._L.faco_begin_programs(self._handle, keys.ctypes.data, seeds.ctypes.data, keys.size,
                                               C.cast(arr, C.c_void_p), len(arr),
                                               _exact_int(experiment_mask, "experiment_mask", 1, 0xFFFFFFFF),
                                               _exact_int(initial_mne, "initial_mne", 1, 2**32 - 1),
                                               _exact_int(total_iterations, "total_iterations", 1, 2**32 - 1),
                                               _exact_int(trace_iterations, "trace_iterations", 0, 2**32 - 1)))
        self._active = (keys.copy(), trace_iterations, 0)

    def capture_state(self) -> CountedState:
        """Snapshot of the active stepwise evaluation (it stays active)."""
        size = C.c_uint64()
        _lib.check(self._L.faco_snapshot(self._handle, None, 0, C.byref(size)))
        buf = (C.c_ubyte * size.value)()
        _lib.check(self._L.faco_snapshot(self._handle, C.cast(buf, C.c_void_p), size.value, C.byref(size)))
        return CountedState(bytes(buf))

    def restore_state(self, state: CountedState, *, trace_iterations: int = 0) -> None:
        """Begins a stepwise evaluation from a snapshot; step() continues it."""
        if not isinstance(state, CountedState):
            raise ValueError("state must be a CountedState")
        data = state.to_bytes()
        _lib.check(self._L.faco_restore(self._handle, data, len(data),
                                        _exact_int(trace_iterations, "trace_iterations", 0, 2**32 - 1)))
        info = state.describe()
        self._spec = info["feature_spec"] if info["controlled"] else 0
        self._active = (np.asarray(info["instance_keys"], np.uint64), trace_iterations, info["completed_batches"])

    def _stepwise_output(self, res: dict, limit: int) -> dict:
        keys = self._active_keys
        items = [{"has_incumbent": True, "tour": tour.tolist(), "cost": int(cost), "completed_seconds": None}
                 for tour, cost in zip(res["tours"], res["costs"])]
        return {"items": items, "budget_seconds": None, "budget_kind": "search_tour_evaluations",
                "evaluation_limit_per_colony": limit,
                "completed_tour_evaluations_per_colony": res["completed_batches"] * self.ants,
                "total_tour_evaluations": res["completed_batches"] * self.ants * len(keys),
                "completed_batches": res["completed_batches"],
                "completed_construction_steps": res["construction_steps"],
                "completed_ls_evaluations": res["ls_evaluations"], "reversed_elements": res["reversed_elements"],
                "colony_work": res["colony_work"],
                **({"control_states": res["control_states"]} if "control_states" in res else {})}

    def _batches(self, evaluations, name: str) -> int:
        value = _exact_int(evaluations, name)
        if value % self.ants:
            raise ValueError(f"{name} must be a whole number of ant batches ({self.ants} ants)")
        return value // self.ants

    def capture_faco_state(self, instance_keys, seeds, capture_after_evaluations, mne=8) -> dict:
        """Plain FACO for `capture_after_evaluations` per colony, then a
        snapshot: {"evaluation": result so far, "state": CountedState}."""
        batches = self._batches(capture_after_evaluations, "capture_after_evaluations")
        self.begin(instance_keys, seeds, mne)
        self._active_keys = self._active[0]
        self.step(batches)
        state = self.capture_state()
        return {"evaluation": self._stepwise_output(self.finish(), capture_after_evaluations), "state": state}

    def capture_program_state(self, instance_keys, seeds, source_evaluation_limit_per_colony,
                              capture_after_evaluations, program, experiment_mask=0xFFFFFFFF) -> dict:
        """capture_program_state (bindings.cpp:880-894): a controlled run
        budgeted for `source_evaluation_limit_per_colony`, captured after
        `capture_after_evaluations`."""
        total = self._batches(source_evaluation_limit_per_colony, "source_evaluation_limit_per_colony")
        batches = self._batches(capture_after_evaluations, "capture_after_evaluations")
        if batches > total:
            raise ValueError("capture point beyond the source budget")
        self.begin_programs(instance_keys, seeds, [program], experiment_mask, total_iterations=max(1, total))
        self._active_keys = self._active[0]
        self.step(batches)
        state = self.capture_state()
        return {"evaluation": self._stepwise_output(self.finish(), capture_after_evaluations), "state": state}

    def continue_faco_state(self, state: CountedState, additional_evaluations_per_colony) -> dict:
        batches = self._batches(additional_evaluations_per_colony, "additional_evaluations_per_colony")
        if state.describe()["controlled"]:
            raise ValueError("the state is of a controlled run: use continue_program_state")
        self.restore_state(state)
        self._active_keys = self._active[0]
        self.step(batches)
        return self._stepwise_output(self.finish(), additional_evaluations_per_colony)

    def continue_program_state(self, state: CountedState, additional_evaluations_per_colony, program) -> dict:
        """continue_program_state (bindings.cpp:922-928): resumes a captured
        controlled run for more evaluations; `program` must be the captured one."""
        batches = self._batches(additional_evaluations_per_colony, "additional_evaluations_per_colony")
        info = state.describe()
        if not info["controlled"] or info["programs"] != 1:
            raise ValueError("the state is not of a single-program controlled run")
        captured = state.to_bytes()[_SNAPSHOT_HEADER.itemsize + 24 * info["colonies"]:][:C.sizeof(_lib.Program)]
        if bytes(program_to_c(program)) != captured:
            raise ValueError("program differs from the captured one")
        self.restore_state(state)
        self._active_keys = self._active[0]
        self.step(batches)
        return self._stepwise_output(self.finish(), additional_evaluations_per_colony)

    def _program_array(self, programs):
        if not isinstance(programs, (list, tuple)) or not programs:
            raise ValueError("programs must be a non-empty list of IR dicts")
        arr = (_lib.Program * len(programs))(*[program_to_c(p) for p in programs])
        if any(p.feature_spec_id not in (2, 3) for p in arr) or len({p.feature_spec_id for p in arr}) != 1:
            raise ValueError("controller programs use one feature spec, 2 or 3")
        return arr

    # ---- learned edge prior on the active stepwise evaluation ---------------
    def edge_data(self, features: bool = True, labels: bool = True):
        """Candidate-edge features (BF16 bits [E, 8]) and labels (edge of each
        colony's global-best tour) of the current colony states."""
        rows = C.c_uint64()
        _lib.check(self._L.faco_edge_data(self._handle, None, None, 0, C.byref(rows)))
        x = np.zeros((rows.value, 8), np.uint16) if features else None
        y = np.zeros(rows.value, np.float32) if labels else None
        _lib.check(self._L.faco_edge_data(self._handle, _lib.ptr(x), _lib.ptr(y), rows.value, C.byref(rows)))
        return x, y

    def prior_set(self, params, enabled, floor: float = 0.05, gamma: int = 1, departures: bool = False) -> None:
        """Reweights eta by (floor + p)^gamma on colonies with enabled[c]; the
        others use the plain heuristic.  params None keeps the loaded network.
        departures: the prior only re-ranks the departures from the parent
        tour (parent-tour entries keep the plain heuristic, the others keep
        the plain total weight per node)."""
        enabled = np.ascontiguousarray(enabled, np.uint8)
        p = None if params is None else np.ascontiguousarray(params, np.float32)
        if type(departures) is not bool:
            raise ValueError("departures must be a bool")
        _lib.check(self._L.faco_prior_set(self._handle, _lib.ptr(p), float(floor), _exact_int(gamma, "gamma", 1, 2),
                                          enabled.ctypes.data, int(departures)))

    def prior_refresh(self) -> None:
        _lib.check(self._L.faco_prior_refresh(self._handle))

    def colony_rows(self, colony: int) -> dict:
        """One colony's trails, heuristic (eta, the prior's when it is set)
        and products, [n, k] float32 each, after the work queued so far."""
        keys = self._active[0]
        c = _exact_int(colony, "colony", 0, keys.size - 1)
        n = self._sizes[int(keys[c])]
        k = min(self.settings.primary_width, n - 1)
        out = {name: np.zeros((n, k), np.float32) for name in ("trails", "eta", "products")}
        _lib.check(self._L.faco_colony_rows(self._handle, c, out["trails"].ctypes.data, out["eta"].ctypes.data,
                                            out["products"].ctypes.data, n * k))
        return out

    def current_costs(self, count: int):
        costs = np.zeros(count, np.int64)
        it = C.c_uint32()
        _lib.check(self._L.faco_current_costs(self._handle, costs.ctypes.data, C.byref(it)))
        return costs, int(it.value)

    def set_mne_targets(self, targets) -> None:
        """Per-colony MNE targets of the active plain stepwise evaluation from
        the next batch on (one per colony, each >= 1)."""
        t = np.ascontiguousarray([_exact_int(int(v) if isinstance(v, np.integer) else v, "MNE target", 1,
                                             2**32 - 1) for v in targets], dtype=np.uint32)
        _lib.check(self._L.faco_set_mne_targets(self._handle, t.ctypes.data, t.size))

    @property
    def stream_ptr(self) -> int:
        """The engine's cudaStream_t as an integer (torch.cuda.ExternalStream)."""
        return int(self._L.faco_engine_stream(self._handle) or 0)


_SNAPSHOT_HEADER = np.dtype([
    ("magic", "S8"), ("version", "<u4"), ("count", "<u4"), ("ants", "<u4"), ("k_common", "<u4"),
    ("mne_target", "<u4"), ("n_programs", "<u4"), ("action_mask", "<u4"), ("total_iterations", "<u4"),
    ("controlled", "<u4"), ("done", "<u4"), ("feature_spec", "<u4"), ("reserved1", "<u4"),
    ("settings_digest", "<u8"), ("tau_total", "<u8"), ("node_total", "<u8")])
_COLONY_STATE_BYTES = 104      # sizeof(ColonyState); global_cost at byte 8


class CountedState:
    """A colony snapshot (the reference's CountedState,
    cpp/include/gp_faco/counted_state.hpp:23-38): opaque bytes made by
    FacoBatchEngine.capture_state and accepted by restore_state."""

    def __init__(self, data: bytes):
        data = bytes(data)
        if len(data) < _SNAPSHOT_HEADER.itemsize + 8 or data[:8] != b"FACOSNP1":
            raise ValueError("not a colony snapshot")
        self._data = data

    @staticmethod
    def from_bytes(data) -> "CountedState":
        return CountedState(data)

    def to_bytes(self) -> bytes:
        return self._data

    def describe(self) -> dict:
        h = np.frombuffer(self._data, _SNAPSHOT_HEADER, count=1)[0]
        c = int(h["count"])
        off = _SNAPSHOT_HEADER.itemsize
        keys = np.frombuffer(self._data, "<u8", c, off)
        seeds = np.frombuffer(self._data, "<u8", c, off + 8 * c)
        off += 24 * c + int(h["n_programs"]) * (3 * C.sizeof(_lib.Program) + 4)
        costs = [int(np.frombuffer(self._data, "<i8", 1, off + _COLONY_STATE_BYTES * i + 8)[0]) for i in range(c)]
        return {"version": int(h["version"]), "colonies": c, "completed_batches": int(h["done"]),
                "instance_keys": keys.tolist(), "seeds": seeds.tolist(), "global_costs": costs,
                "controlled": bool(h["controlled"]), "programs": int(h["n_programs"]),
                "mne_target": int(h["mne_target"]), "total_iterations": int(h["total_iterations"]),
                "feature_spec": int(h["feature_spec"]), "bytes": len(self._data)}


class FixedFacoGpu:
    """FixedFacoGpu(coordinates f64[n,2], instance_key, settings)
    (bindings.cpp:972-1006, cuda/fixed_faco.cu:105-177): one instance, one
    colony.  Every run_iterations call restarts the colony from the prepared
    initial tour and runs `batches` ant batches with a constant MNE target."""

    def __init__(self, coordinates, instance_key, settings: FixedFacoSettings, device: int = 0):
        key = _exact_int(instance_key, "instance_key")
        if (not isinstance(coordinates, np.ndarray) or coordinates.dtype != np.float64 or coordinates.ndim != 2
                or coordinates.shape[1] != 2):
            raise ValueError("coordinates must be a float64 [n, 2] array")
        self._key = key
        self._engine = FacoBatchEngine(int(coordinates.shape[0]), 1, settings, device=device)
        self._registration = self._engine.register_problem(key, np.ascontiguousarray(coordinates))

    def run_iterations(self, seed, batches, mne_target) -> dict:
        seed = _exact_int(seed, "seed")
        batches = _exact_int(batches, "batches", 0, 2**32 - 1)
        mne = _exact_int(mne_target, "mne_target", 1, 2**32 - 1)
        e = self._engine
        res = e.evaluate_faco_evaluations(np.array([self._key], np.uint64), np.array([seed], np.uint64),
                                          batches * e.ants, mne)
        item = res["items"][0]
        return {"tour": item["tour"], "cost": item["cost"], "initial_cost": self._registration["initial_cost"],
                "preparation_seconds": self._registration["preparation_seconds"],
                "solve_seconds": res["elapsed_seconds"], "batches": res["completed_batches"],
                "construction_steps": res["completed_construction_steps"],
                "ls_evaluations": res["completed_ls_evaluations"]}

    def close(self) -> None:
        self._engine.close()


def program_to_c(program: dict) -> _lib.Program:
    """read_program (bindings.cpp:22-56): strict IR dict -> Program struct."""
    if not isinstance(program, dict):
        raise ValueError("program must be a dict")
    if len(program) != 6 and not (len(program) == 7 and "program_id" in program):
        raise ValueError("wrong number of IR fields")
    p = _lib.Program()
    for name in ("ir_version", "numeric_spec_id", "feature_spec_id"):
        setattr(p, name, _exact_int(program[name], name, 0, 0xFFFF))
    ops, operands, bits = program["opcode"], program["operand"], program["constant_bits"]
    for seq in (ops, operands, bits):
        for v in seq:
            if type(v) is not int:
                raise ValueError("opcodes, operands and bit patterns must be ints")
    if not 1 <= len(ops) <= 63 or len(operands) != len(ops) or len(bits) > 63:
        raise ValueError("IR array sizes out of range")
    p.length, p.constants_count = len(ops), len(bits)
    for i, (o, a) in enumerate(zip(ops, operands)):
        if not (0 <= o <= 255 and 0 <= a <= 255):
            raise ValueError("opcode/operand out of uint8 range")
        p.opcode[i], p.operand[i] = o, a
    for i, b in enumerate(bits):
        if not 0 <= b <= 0xFFFFFFFF:
            raise ValueError("constant bits out of uint32 range")
        p.constants[i] = struct.unpack("<f", struct.pack("<I", b))[0]
    _lib.check(_lib.load().faco_validate_program(C.byref(p)))
    return p


def _feature_spec(programs):
    """(feature spec, kinds) of the program array or (slots, kinds) pair."""
    if isinstance(programs, tuple):
        arr, kinds = programs
        return arr[0].feature_spec_id, [int(k) for k in kinds]
    return programs[0].feature_spec_id, [0] * len(programs)


def control_state_dicts(rows, spec=3) -> list[dict]:
    """Per-colony controller feedback after the last batch (the
    control_states list of bindings.cpp:395-407).  Feature spec 2: the
    reference's fields (archive size, stagnant batches, return rate, LS work,
    batches since the last restart, restarts); spec 3: restarts, batches since
    the last global improvement, and the start region (4 = all nodes) and MNE
    target of the next batch."""
    if spec == 2:
        return [{"archive_size": int(r["archive_size"]), "stagnant_batches": int(r["stagnant_batches"]),
                 "return_rate": float(r["return_rate"]), "ls_work": float(r["ls_work"]),
                 "epoch_batches": int(r["epoch_batches"]), "restarts": int(r["restarts"])} for r in rows]
    return [{"restarts": int(r["restarts"]), "stagnant_batches": int(r["stagnant_batches"]),
             "start_region": int(r["start_region"]), "mne_target": int(r["mne_target"])} for r in rows]


def controller_stages(scores, mask: int, action: int) -> list[dict]:
    """The three role decisions of a conditional controller (bindings.cpp:76-91)."""
    stages, prefix = [], 0
    for role, (width, stride, offset) in enumerate(((2, 16, 0), (4, 4, 2), (4, 1, 6))):
        legal = [bool((mask >> (prefix + i * stride)) & ((1 << stride) - 1)) for i in range(width)]
        selected = (action - prefix) // stride
        stages.append({"scores": [float(x) for x in scores[offset:offset + width]], "legal": legal,
                       "selected": selected})
        prefix += selected * stride
    return stages


def decision_rows(points, dec, kinds, count) -> list[dict]:
    """Captured decisions as the reference returns them (bindings.cpp:323-346):
    one row per (iteration, colony) with its legal mask, action, 12 x 32
    features and 32 scores (conditional controllers: the role stages)."""
    rows = []
    per = count // len(kinds)
    for i, point in enumerate(points):
        for c in range(count):
            row = {"iteration": int(point), "colony": c, "legal_mask": int(dec["masks"][i, c]),
                   "action": int(dec["actions"][i, c]),
                   "features": [dec["features"][i, c, f].tolist() for f in range(12)]}
            if kinds[c // per] == 1:
                row["stages"] = controller_stages(dec["scores"][i, c], row["legal_mask"], row["action"])
            else:
                row["scores"] = [float(x) if np.isfinite(x) else None for x in dec["scores"][i, c]]
            rows.append(row)
    return rows


def controller_arrays(controllers):
    """Controller dicts (or bare program dicts) as three program slots each
    and their kinds (0 joint_single, 1 conditional_three); validated like
    read_controller (bindings.cpp:58-73)."""
    if not isinstance(controllers, (list, tuple)) or not controllers:
        raise ValueError("controllers must be a non-empty list")
    slots, kinds = [], []
    for c in controllers:
        if not isinstance(c, dict):
            raise ValueError("a controller must be a dict")
        if "opcode" in c:
            trees, kind = [c], 0
        else:
            if (len(c) != 4 or type(c.get("controller_version")) is not int or c["controller_version"] != 1
                    or "controller_id" not in c or "trees" not in c):
                raise ValueError("unknown controller version or fields")
            rep = c.get("representation")
            if rep not in ("joint_single", "conditional_three"):
                raise ValueError("unknown controller representation")
            trees = list(c["trees"])
            kind = 1 if rep == "conditional_three" else 0
            if len(trees) != (3 if kind else 1):
                raise ValueError("wrong number of role trees for the controller representation")
        structs = [program_to_c(t) for t in trees]
        while len(structs) < 3:
            structs.append(_lib.Program())
        slots += structs
        kinds.append(kind)
    arr = (_lib.Program * len(slots))(*slots)
    kinds = np.asarray(kinds, np.uint32)
    L = _lib.load()
    for i in range(kinds.size):
        _lib.check(L.faco_validate_controller(C.cast(C.byref(arr, 3 * i * C.sizeof(_lib.Program)), C.c_void_p),
                                              int(kinds[i])))
    return arr, kinds


def score_controller_cuda(controller, features, masks) -> dict:
    """score_controller_cuda (bindings.cpp:1010-1016, gp_score.cu:32-47):
    joint controllers score all 32 actions, conditional_three ones return
    their role scores in slots 0-1, 2-5 and 6-9; actions chosen per colony."""
    arr, kinds = controller_arrays([controller])
    features = np.ascontiguousarray(features, dtype=np.float32)
    masks = np.ascontiguousarray(masks, dtype=np.uint32)
    if features.ndim != 3 or features.shape[0] != 12 or features.shape[2] != 32 or masks.shape != (features.shape[1],):
        raise ValueError("features must be [12, C, 32] and masks [C]")
    scores = np.zeros((masks.size, 32), np.float32)
    actions = np.zeros(masks.size, np.int32)
    _lib.check(_lib.load().faco_score_controllers(C.cast(arr, C.c_void_p), kinds.ctypes.data, 1,
                                                  features.ctypes.data, 12, masks.ctypes.data, masks.size,
                                                  scores.ctypes.data, actions.ctypes.data))
    return {"scores": scores, "actions": actions}


def score_cuda(programs, features, masks) -> dict:
    """score_cuda(program, features f32[12,C,32], masks u32[C]) (bindings.cpp:
    504-506,1007-1009).  `programs` may be one IR dict or a list of them (the
    colonies are split evenly between programs)."""
    if isinstance(programs, dict):
        programs = [programs]
    if (not isinstance(features, np.ndarray) or features.dtype != np.float32 or features.ndim != 3
            or features.shape[0] != 12 or features.shape[2] != 32 or not features.flags.c_contiguous):
        raise ValueError("features must be C-contiguous float32 [12, colonies, 32]")
    if (not isinstance(masks, np.ndarray) or masks.dtype != np.uint32 or masks.ndim != 1
            or masks.shape[0] != features.shape[1] or not masks.flags.c_contiguous):
        raise ValueError("masks must be C-contiguous uint32 [colonies]")
    arr = (_lib.Program * len(programs))(*[program_to_c(p) for p in programs])
    colonies = masks.shape[0]
    scores = np.zeros((colonies, 32), np.float32)
    actions = np.zeros(colonies, np.int32)
    _lib.check(_lib.load().faco_score(C.cast(arr, C.c_void_p), len(programs), features.ctypes.data, 12,
                                      masks.ctypes.data, colonies, scores.ctypes.data, actions.ctypes.data))
    return {"scores": scores, "actions": actions}


def ant_diagnostic(xy, ls_rows, tours, mne_targets, evaluation_limit, *, visits=None, uniforms=None, starts=None,
                   primary=None, products=None, backup=None, checklist_capacity=None,
                   ls_mode: int = _lib.FACO_LS_TWO_OPT) -> dict:
    """cuda_faco_diagnostic (cpp/include/gp_faco/faco_cuda_diagnostic.hpp:36-39):
    explicit-choice (visits) or injected-uniform construction + local search,
    one warp-ant per task."""
    xy = np.ascontiguousarray(xy, dtype=np.int32)
    n = xy.shape[0]
    ls_rows = np.ascontiguousarray(ls_rows, dtype=np.uint32)
    tours = np.ascontiguousarray(tours, dtype=np.uint32).reshape(-1, n)
    tasks = tours.shape[0]
    targets = np.ascontiguousarray(mne_targets, dtype=np.uint32)
    cap = checklist_capacity or 8 * n + 8
    outs = dict(construction_tours=np.zeros((tasks, n), np.uint32), tours=np.zeros((tasks, n), np.uint32),
                positions=np.zeros((tasks, n), np.uint32), selected=np.zeros((tasks, n), np.uint32),
                checklists=np.zeros((tasks, cap), np.uint32), construction_costs=np.zeros(tasks, np.int64),
                final_costs=np.zeros(tasks, np.int64), counters=np.zeros((tasks, 10), np.uint64))
    o = _lib.AntOutputs(outs["construction_tours"].ctypes.data, outs["tours"].ctypes.data,
                        outs["positions"].ctypes.data, outs["selected"].ctypes.data, outs["checklists"].ctypes.data,
                        cap, outs["construction_costs"].ctypes.data, outs["final_costs"].ctypes.data,
                        outs["counters"].ctypes.data)
    keep = []

    def arr(a, dt):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dt)
        keep.append(a)
        return a.ctypes.data

    k = 0 if primary is None else np.asarray(primary).shape[1]
    b = 0 if backup is None else np.asarray(backup).shape[1]
    _lib.check(_lib.load().faco_ant_diagnostic(
        xy.ctypes.data, n, ls_rows.ctypes.data, ls_rows.shape[1], tours.ctypes.data, arr(visits, np.uint32),
        arr(uniforms, np.float64), arr(starts, np.uint32), arr(primary, np.uint32), arr(products, np.float32), k,
        arr(backup, np.uint32) if b else None, b, targets.ctypes.data, tasks, evaluation_limit,
        _exact_int(ls_mode, "ls_mode", 0, 1), C.byref(o)))
    return outs


def pheromone_step(primary, parent, trails, eta, *, retention, minimum, maximum, increment):
    """One MMAS evaporate/deposit step on FP32 trails (cuda/colony_state.cuh:210-229)."""
    primary = np.ascontiguousarray(primary, dtype=np.uint32)
    n, k = primary.shape
    parent = np.ascontiguousarray(parent, dtype=np.uint32)
    trails = np.array(trails, dtype=np.float32, order="C", copy=True).reshape(n, k)
    eta = np.ascontiguousarray(eta, dtype=np.float32).reshape(n, k)
    products = np.zeros((n, k), np.float32)
    _lib.check(_lib.load().faco_pheromone_step(n, k, primary.ctypes.data, parent.ctypes.data, retention, minimum,
                                               maximum, increment, eta.ctypes.data, trails.ctypes.data,
                                               products.ctypes.data))
    return trails, products

"""ctypes view of the engine's C ABI (include/faco_gb300.h).

There is no fallback: if the CUDA library is missing or fails to load, every
entry point raises.  Build it with ``python -m gplsaco_gb300.build``.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libfaco_gb300.so"

FACO_OK = 0
FACO_EINVAL = -1
FACO_ECUDA = -2
FACO_EBUSY = -3
FACO_EDEVICE = -4
FACO_ENOMEM = -5

FACO_LS_TWO_OPT = 0
FACO_LS_TWO_OPT_OR_OPT = 1

FACO_FOLLOW_AUTO, FACO_FOLLOW_OFF, FACO_FOLLOW_ON = 0, 1, 2

EXPORTED = (
    "faco_default_settings", "faco_last_error", "faco_engine_create", "faco_engine_destroy",
    "faco_register_problem", "faco_problem_rows", "faco_evaluate", "faco_validate_program", "faco_score",
    "faco_ant_diagnostic", "faco_pheromone_step", "faco_begin", "faco_step", "faco_step_timed", "faco_finish",
    "faco_engine_stream", "faco_evaluate_programs", "faco_mlp_param_count", "faco_mlp_forward", "faco_mlp_gradient",
    "faco_mlp_train", "faco_edge_data", "faco_prior_set", "faco_prior_refresh", "faco_current_costs",
    "faco_colony_rows",
    "faco_set_mne_targets", "faco_get_launch_plan",
    "faco_pheromone_step_noalloc", "faco_begin_programs", "faco_snapshot", "faco_restore",
    "faco_evaluate_controllers", "faco_validate_controller", "faco_score_controllers",
)


class Settings(C.Structure):
    _fields_ = [("ants", C.c_uint32), ("primary_width", C.c_uint32), ("backup_width", C.c_uint32),
                ("ls_width", C.c_uint32), ("beta", C.c_double), ("retention", C.c_double),
                ("p_best", C.c_double), ("epoch_source_probability", C.c_double),
                ("ls_evaluation_limit", C.c_uint64), ("initial_ls_evaluation_limit", C.c_uint64),
                ("ls_mode", C.c_uint32), ("autotune", C.c_uint32), ("workspace", C.c_uint32),
                ("force_fingerprint_collisions", C.c_uint32), ("chains", C.c_uint32), ("follow", C.c_uint32)]


class LaunchPlan(C.Structure):
    _fields_ = [("size_classes", C.c_uint32), ("chains", C.c_uint32), ("graph_iterations", C.c_uint32),
                ("launches_per_iteration", C.c_uint32), ("follow", C.c_uint32)]


class Registration(C.Structure):
    _fields_ = [("cheap_seconds", C.c_double), ("preparation_seconds", C.c_double),
                ("initial_cost", C.c_int64), ("n", C.c_uint32), ("reserved", C.c_uint32)]


class TraceRow(C.Structure):
    _fields_ = [("iteration_best_cost", C.c_int64), ("global_cost", C.c_int64), ("parent_cost", C.c_int64),
                ("iteration_best", C.c_uint32), ("source_is_epoch", C.c_uint32), ("tau_min", C.c_float),
                ("tau_max", C.c_float), ("mne_target", C.c_uint32), ("action", C.c_int32),
                ("construction_steps", C.c_uint64), ("ls_evaluations", C.c_uint64)]


TRACE_DTYPE = np.dtype([("iteration_best_cost", "<i8"), ("global_cost", "<i8"), ("parent_cost", "<i8"),
                        ("iteration_best", "<u4"), ("source_is_epoch", "<u4"), ("tau_min", "<f4"),
                        ("tau_max", "<f4"), ("mne_target", "<u4"), ("action", "<i4"),
                        ("construction_steps", "<u8"), ("ls_evaluations", "<u8")])


class Outputs(C.Structure):
    _fields_ = [("tours", C.c_void_p), ("costs", C.c_void_p), ("trace", C.c_void_p),
                ("checkpoint_tours", C.c_void_p), ("completed_batches", C.c_uint64),
                ("construction_steps", C.c_uint64), ("ls_evaluations", C.c_uint64),
                ("reversed_elements", C.c_uint64), ("kernel_milliseconds", C.c_double),
                ("solve_seconds", C.c_double), ("colony_work", C.c_void_p),
                ("control_states", C.c_void_p), ("decision_iterations", C.c_void_p),
                ("n_decisions", C.c_uint32), ("decision_features", C.c_void_p), ("decision_scores", C.c_void_p),
                ("decision_masks", C.c_void_p), ("decision_actions", C.c_void_p)]


# faco_control_state
CONTROL_STATE_DTYPE = np.dtype([("restarts", "<u8"), ("stagnant_batches", "<u8"), ("epoch_batches", "<u8"),
                                ("return_rate", "<f4"), ("ls_work", "<f4"), ("archive_size", "<u4"),
                                ("start_region", "<u4"), ("mne_target", "<u4"), ("reserved", "<u4")])


class Program(C.Structure):
    _fields_ = [("ir_version", C.c_uint16), ("numeric_spec_id", C.c_uint16), ("feature_spec_id", C.c_uint16),
                ("length", C.c_uint16), ("constants_count", C.c_uint16), ("opcode", C.c_uint8 * 63),
                ("operand", C.c_uint8 * 63), ("constants", C.c_float * 63)]


class AntOutputs(C.Structure):
    _fields_ = [("construction_tours", C.c_void_p), ("tours", C.c_void_p), ("positions", C.c_void_p),
                ("selected", C.c_void_p), ("checklists", C.c_void_p), ("checklist_capacity", C.c_uint32),
                ("construction_costs", C.c_void_p), ("final_costs", C.c_void_p), ("counters", C.c_void_p)]


_lib = None


class FacoError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


def check(code: int) -> None:
    if code == FACO_OK:
        return
    message = load().faco_last_error().decode(errors="replace")
    if code == FACO_EINVAL:
        raise ValueError(message)
    raise FacoError(code, message)


def load():
    """Loads the CUDA engine library; raises if it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"GB300 FACO engine library missing: {LIB_PATH} (run python -m gplsaco_gb300.build)")
    L = C.CDLL(str(LIB_PATH))
    vp = C.c_void_p
    L.faco_last_error.restype = C.c_char_p
    L.faco_default_settings.argtypes = [C.POINTER(Settings)]
    L.faco_engine_create.argtypes = [C.c_uint32, C.c_uint32, C.POINTER(Settings), C.c_int, C.POINTER(vp)]
    L.faco_engine_destroy.argtypes = [vp]
    L.faco_register_problem.argtypes = [vp, C.c_uint64, vp, C.c_uint32, C.POINTER(Registration)]
    L.faco_problem_rows.argtypes = [vp, C.c_uint64, vp, vp, vp, vp]
    L.faco_evaluate.argtypes = [vp, vp, vp, C.c_uint32, C.c_uint64, C.c_uint32, vp, C.c_uint32,
                                C.POINTER(Outputs)]
    L.faco_validate_program.argtypes = [C.POINTER(Program)]
    L.faco_score.argtypes = [vp, C.c_uint32, vp, C.c_uint32, vp, C.c_uint32, vp, vp]
    L.faco_ant_diagnostic.argtypes = [vp, C.c_uint32, vp, C.c_uint32, vp, vp, vp, vp, vp, vp, C.c_uint32, vp,
                                      C.c_uint32, vp, C.c_uint32, C.c_uint64, C.c_uint32, C.POINTER(AntOutputs)]
    L.faco_pheromone_step.argtypes = [C.c_uint32, C.c_uint32, vp, vp, C.c_float, C.c_float, C.c_float, C.c_float,
                                      vp, vp, vp]
    L.faco_evaluate_controllers.argtypes = [vp, vp, vp, C.c_uint32, C.c_uint64, vp, vp, C.c_uint32, C.c_uint32,
                                            C.c_uint32, vp, C.c_uint32, C.POINTER(Outputs)]
    L.faco_validate_controller.argtypes = [vp, C.c_uint32]
    L.faco_score_controllers.argtypes = [vp, vp, C.c_uint32, vp, C.c_uint32, vp, C.c_uint32, vp, vp]
    L.faco_begin_programs.argtypes = [vp, vp, vp, C.c_uint32, vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                      C.c_uint32]
    L.faco_snapshot.argtypes = [vp, vp, C.c_uint64, C.POINTER(C.c_uint64)]
    L.faco_restore.argtypes = [vp, vp, C.c_uint64, C.c_uint32]
    L.faco_pheromone_step_noalloc.argtypes = [C.c_uint32, C.c_uint32, vp, vp, C.c_float, C.c_float, C.c_float,
                                              C.c_float, vp, vp, vp, vp]
    L.faco_evaluate_programs.argtypes = [vp, vp, vp, C.c_uint32, C.c_uint64, vp, C.c_uint32, C.c_uint32,
                                         C.c_uint32, vp, C.c_uint32, C.POINTER(Outputs)]
    L.faco_mlp_param_count.argtypes = []
    L.faco_mlp_forward.argtypes = [vp, vp, C.c_uint32, vp]
    L.faco_mlp_gradient.argtypes = [vp, vp, vp, C.c_uint32, vp, vp]
    L.faco_mlp_train.argtypes = [vp, vp, vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, vp]
    L.faco_edge_data.argtypes = [vp, vp, vp, C.c_uint64, C.POINTER(C.c_uint64)]
    L.faco_prior_set.argtypes = [vp, vp, C.c_float, C.c_int, vp, C.c_uint32]
    L.faco_prior_refresh.argtypes = [vp]
    L.faco_current_costs.argtypes = [vp, vp, C.POINTER(C.c_uint32)]
    L.faco_colony_rows.argtypes = [vp, C.c_uint32, vp, vp, vp, C.c_uint64]
    L.faco_set_mne_targets.argtypes = [vp, vp, C.c_uint32]
    L.faco_begin.argtypes = [vp, vp, vp, C.c_uint32, C.c_uint32, C.c_uint32]
    L.faco_step.argtypes = [vp, C.c_uint32]
    L.faco_step_timed.argtypes = [vp, C.c_uint32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.faco_get_launch_plan.argtypes = [vp, C.POINTER(LaunchPlan)]
    L.faco_finish.argtypes = [vp, C.POINTER(Outputs)]
    L.faco_engine_stream.argtypes = [vp]
    L.faco_engine_stream.restype = vp
    for name in EXPORTED:
        if name not in ("faco_default_settings", "faco_last_error", "faco_engine_destroy", "faco_engine_stream"):
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


def ptr(a) -> int | None:
    return None if a is None else a.ctypes.data

"""ctypes binding for the CPU oracle (oracle/faco_oracle.c) and, when it was
built in this container, the reference-core shim (oracle/_ref).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py -- never by the gplsaco_gb300 package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libfaco_oracle.so"
REF_LIB = HERE / "_ref" / "libgplsaco_ref.so"

u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def build(force: bool = False) -> Path:
    """Compile the oracle with the host compiler (contractions off)."""
    sources = [HERE / "faco_oracle.c", HERE / "control_oracle.c"]
    newest = max(p.stat().st_mtime for p in sources + [HERE / "faco_oracle.h"])
    if force or not LIB.exists() or LIB.stat().st_mtime < newest:
        LIB.parent.mkdir(exist_ok=True)
        tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
        subprocess.check_call(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                               *map(str, sources), "-o", str(tmp), "-lm"])
        os.replace(tmp, LIB)
    return LIB


class DistT(C.Structure):
    _fields_ = [("n", C.c_uint32), ("xy", C.c_void_p), ("matrix", C.c_void_p)]


class LsStats(C.Structure):
    _fields_ = [("processed_nodes", C.c_uint64), ("candidate_checks", C.c_uint64),
                ("move_evaluations", C.c_uint64), ("accepted_moves", C.c_uint64),
                ("reactivations", C.c_uint64), ("evaluation_limit_reached", C.c_uint32)]


class ConsStats(C.Structure):
    _fields_ = [("mne", C.c_uint32), ("steps", C.c_uint32), ("nonidentity_relocations", C.c_uint32),
                ("legal_exhausted", C.c_uint32)]


class Choices(C.Structure):
    _fields_ = [("visit", C.c_void_p), ("uniforms", C.c_void_p), ("start", C.c_uint32),
                ("primary", C.c_void_p), ("products32", C.c_void_p), ("products64", C.c_void_p),
                ("k", C.c_uint32), ("backup", C.c_void_p), ("b", C.c_uint32)]


class AntInfo(C.Structure):
    _fields_ = [("construction_cost", C.c_int64), ("final_cost", C.c_int64), ("cons", ConsStats),
                ("ls", LsStats), ("start_node", C.c_uint32), ("checklist_len", C.c_uint32)]


class PrepCfg(C.Structure):
    _fields_ = [("k", C.c_uint32), ("b", C.c_uint32), ("w", C.c_uint32),
                ("initial_ls_evaluation_limit", C.c_uint64)]


class RunCfg(C.Structure):
    _fields_ = [("ants", C.c_uint32), ("k", C.c_uint32), ("b", C.c_uint32), ("w", C.c_uint32),
                ("mne_target", C.c_uint32), ("beta", C.c_double), ("retention", C.c_double),
                ("p_best", C.c_double), ("epoch_source_probability", C.c_double),
                ("ls_evaluation_limit", C.c_uint64), ("threads", C.c_uint32), ("ls_mode", C.c_uint32)]


class IterTrace(C.Structure):
    _fields_ = [("iteration_best_cost", C.c_int64), ("global_cost", C.c_int64), ("parent_cost", C.c_int64),
                ("iteration_best", C.c_uint32), ("source_is_epoch", C.c_uint32), ("tau_min", C.c_float),
                ("tau_max", C.c_float), ("mne_target", C.c_uint32), ("action", C.c_int32),
                ("construction_steps", C.c_uint64), ("ls_evaluations", C.c_uint64)]


class Program(C.Structure):
    _fields_ = [("ir_version", C.c_uint16), ("numeric_spec_id", C.c_uint16), ("feature_spec_id", C.c_uint16),
                ("length", C.c_uint16), ("constants_count", C.c_uint16), ("opcode", C.c_uint8 * 63),
                ("operand", C.c_uint8 * 63), ("constants", C.c_float * 63)]


class PriorSchedule(C.Structure):
    _fields_ = [("count", C.c_uint32), ("at", C.c_void_p), ("etas", C.c_void_p), ("departures", C.c_void_p)]


class Fp(C.Structure):
    _fields_ = [("first", C.c_uint64), ("second", C.c_uint64)]


class Feedback(C.Structure):
    _fields_ = [("return_rate", C.c_float), ("ls_work", C.c_float), ("stagnant_batches", C.c_uint64),
                ("epoch_batches", C.c_uint64), ("restarts", C.c_uint64)]


class Archive(C.Structure):
    _fields_ = [("n", C.c_uint32), ("size", C.c_uint32), ("tours", C.c_void_p), ("pos", C.c_void_p),
                ("cost", C.c_int64 * 4), ("id", Fp * 4), ("zero_ids", C.c_uint32)]


class ControlIn(C.Structure):
    _fields_ = [("n", C.c_uint32), ("xy", C.c_void_p), ("primary", C.c_void_p), ("k", C.c_uint32),
                ("samples", C.c_void_p), ("sample_count", C.c_uint32), ("local_scale", C.c_void_p),
                ("epsilon", C.c_double), ("active_tour", C.c_void_p), ("active_pos", C.c_void_p),
                ("active_cost", C.c_int64), ("active_id", Fp), ("archive", C.c_void_p), ("feedback", Feedback),
                ("trails", C.c_void_p), ("default_trail", C.c_double), ("tau_min", C.c_double),
                ("tau_max", C.c_double), ("elapsed_ratio", C.c_double), ("solve_key", C.c_uint64),
                ("batch", C.c_uint32), ("experiment_mask", C.c_uint32)]


class ControlIO(C.Structure):
    _fields_ = [("instance_key", C.c_uint64), ("points", C.c_void_p), ("count", C.c_uint32),
                ("features", C.c_void_p), ("scores", C.c_void_p), ("masks", C.c_void_p), ("actions", C.c_void_p),
                ("archive_size", C.c_uint32), ("feedback", Feedback), ("force_collisions", C.c_uint32)]


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        L = _lib
        L.orc_euc2d.restype = C.c_int32
        L.orc_euc2d.argtypes = [C.c_int64] * 4
        L.orc_ant.restype = C.c_int
        L.orc_ant.argtypes = [u32p, C.POINTER(DistT), u32p, C.c_uint32, C.POINTER(Choices), C.c_uint32,
                              C.c_uint64, C.c_uint32, u32p, u32p, u32p, u32p, u32p, C.POINTER(AntInfo)]
        L.orc_select_next.restype = C.c_uint32
        L.orc_select_next.argtypes = [C.c_uint32, u32p, f64p, C.c_uint32, u32p, C.c_uint32, u8p,
                                      C.POINTER(DistT), C.c_double, C.POINTER(C.c_int)]
        L.orc_trail_limits.argtypes = [C.c_uint32, C.c_double, C.c_double, C.c_double,
                                       C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_pheromone64.argtypes = [C.c_uint32, C.c_uint32, u32p, u32p, C.c_double, C.c_double, C.c_double,
                                      C.c_double, f64p, C.POINTER(C.c_double)]
        L.orc_pheromone32.argtypes = [C.c_uint32, C.c_uint32, u32p, u32p, C.c_float, C.c_float, C.c_float,
                                      C.c_float, f32p, f32p, f32p, C.POINTER(C.c_float)]
        L.orc_philox4x32.argtypes = [C.c_uint32] * 6 + [u32p]
        L.orc_uniform.restype = C.c_double
        L.orc_uniform.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32]
        L.orc_start_node.restype = C.c_uint32
        L.orc_start_node.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32]
        L.orc_source_uniform.restype = C.c_double
        L.orc_source_uniform.argtypes = [C.c_uint64, C.c_uint32]
        L.orc_colony_key.restype = C.c_uint64
        L.orc_colony_key.argtypes = [C.c_uint64, C.c_uint64]
        L.orc_prepare.restype = C.c_int64
        L.orc_prepare.argtypes = [C.c_uint32, i32p, C.POINTER(PrepCfg), u32p, u32p, u32p, u32p]
        L.orc_run_colony.restype = C.c_int
        L.orc_run_colony.argtypes = [C.c_uint32, i32p, u32p, u32p, u32p, u32p, C.c_int64, C.POINTER(RunCfg),
                                     C.c_uint64, C.c_uint32, u32p, C.POINTER(C.c_int64), C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                     C.c_void_p]
        L.orc_run_colony_prior.restype = C.c_int
        L.orc_run_colony_prior.argtypes = L.orc_run_colony.argtypes + [C.POINTER(PriorSchedule)]
        L.orc_prior_eta.argtypes = [C.c_size_t, f32p, f32p, C.c_float, C.c_int, f32p]
        L.orc_departure_rows.argtypes = [C.c_uint32, C.c_uint32, u32p, u32p, f32p, f32p, f32p, f32p]
        L.orc_ctl_mix.restype = C.c_uint64
        L.orc_ctl_mix.argtypes = [C.c_uint64]
        L.orc_fingerprint.restype = Fp
        L.orc_fingerprint.argtypes = [u32p, C.c_uint32]
        L.orc_sample_nodes.argtypes = [C.c_uint32, C.c_uint64, u32p]
        L.orc_build_region.argtypes = [u32p, C.c_uint32, u32p, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32,
                                       C.c_uint32, u32p]
        L.orc_archive_update.restype = C.c_int
        L.orc_archive_update.argtypes = [C.POINTER(Archive), u32p, C.c_int64, u32p, i64p, C.c_uint32]
        L.orc_control_features.restype = C.c_uint32
        L.orc_control_features.argtypes = [C.POINTER(ControlIn), f32p, u32p, C.POINTER(C.c_uint32)]
        L.orc_local_scale.argtypes = [C.c_uint32, i32p, f64p, C.POINTER(C.c_double)]
        L.orc_score_conditional.argtypes = [C.c_void_p, f32p, u32p, C.c_uint32, f32p, i32p]
        L.orc_control_choose_conditional.restype = C.c_int32
        L.orc_control_choose_conditional.argtypes = [C.c_void_p, f32p, C.c_uint32, f32p]
        L.orc_log2.restype = C.c_float
        L.orc_log2.argtypes = [C.c_float]
        L.orc_row_entropy_q.restype = C.c_uint32
        L.orc_row_entropy_q.argtypes = [f32p, C.c_uint32, C.c_float]
        L.orc_regions.argtypes = [C.c_uint32, i32p, u32p, u32p]
        L.orc_control_choose.restype = C.c_int32
        L.orc_control_choose.argtypes = [C.POINTER(Program), f32p, C.c_uint32, f32p]
        L.orc_validate_program.restype = C.c_int
        L.orc_validate_program.argtypes = [C.POINTER(Program)]
        L.orc_score.argtypes = [C.POINTER(Program), C.c_uint32, f32p, u32p, C.c_uint32, f32p, i32p]
        L.orc_apply_operation.restype = C.c_float
        L.orc_apply_operation.argtypes = [C.c_int, C.c_float, C.c_float, C.c_float]
    return _lib


def ref():
    """The reference-core shim, or None when it was not built here."""
    global _ref
    if _ref is None and REF_LIB.exists():
        R = C.CDLL(str(REF_LIB))
        R.ref_ant.restype = C.c_int
        R.ref_ant.argtypes = [C.c_uint32, f64p, u32p, C.c_uint32, u32p, u32p, C.c_uint32, C.c_uint64, u32p,
                              C.POINTER(C.c_double), u32p, u32p, C.POINTER(C.c_double), u32p, C.c_uint32, u64p]
        R.ref_select_next.restype = C.c_int
        R.ref_select_next.argtypes = [C.c_uint32, f64p, C.c_uint32, u32p, f64p, C.c_uint32, u32p, C.c_uint32,
                                      u8p, C.c_double, C.POINTER(C.c_uint32), C.POINTER(C.c_int)]
        R.ref_trail_limits.restype = C.c_int
        R.ref_trail_limits.argtypes = [C.c_uint32, C.c_double, C.c_double, C.c_double,
                                       C.POINTER(C.c_double), C.POINTER(C.c_double)]
        R.ref_pheromone.restype = C.c_int
        R.ref_pheromone.argtypes = [C.c_uint32, C.c_uint32, u32p, u32p, C.c_double, C.c_double, C.c_double,
                                    C.c_double, C.c_double, C.c_uint32, f64p, C.POINTER(C.c_double)]
        R.ref_score.restype = C.c_int
        R.ref_score.argtypes = [C.c_uint16, C.c_uint16, C.c_uint16, C.c_uint16, u8p, u8p, C.c_uint16, f32p,
                                f32p, u32p, C.c_uint32, f32p, i32p]
        R.ref_fingerprint.argtypes = [u32p, C.c_uint32, u64p]
        R.ref_sample_nodes.argtypes = [C.c_uint32, C.c_uint64, u32p]
        R.ref_build_region.argtypes = [u32p, C.c_uint32, u32p, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32,
                                       C.c_uint32, u32p]
        R.ref_archive_update.restype = C.c_int
        R.ref_archive_update.argtypes = [C.c_uint32, f64p, u32p, C.c_uint32, u32p, u32p, C.c_uint32, u32p, f64p,
                                         u64p, C.POINTER(C.c_uint32)]
        R.ref_action_snapshot.restype = C.c_int
        R.ref_action_snapshot.argtypes = [C.c_uint32, f64p, u32p, C.c_uint32, u32p, C.c_uint32, f64p, C.c_double,
                                          u32p, u32p, C.c_uint32, f64p, u32p, C.c_double, C.c_double, C.c_double,
                                          C.c_double, C.c_double, C.c_uint32, C.c_double, C.c_uint64, C.c_uint32,
                                          C.c_uint32, f32p, u32p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                          f64p, C.POINTER(C.c_double)]
        R.ref_colony.restype = C.c_int
        R.ref_colony.argtypes = [C.c_uint32, f64p, u32p, C.c_uint32, u32p, C.c_uint32, u32p, C.c_uint32, u32p,
                                 C.c_double, C.c_uint32, C.c_uint32, C.c_uint32, C.c_double, C.c_double,
                                 C.c_double, C.c_double, C.c_uint64, C.c_uint64, u32p, C.POINTER(C.c_double)]
        _ref = R
    return _ref


def ref_colony(xy, prep, *, ants, k, b, w, mne, iterations, seed, beta=1.0, retention=0.98, p_best=0.1,
               epoch_source_probability=0.01, ls_limit=100000):
    """A whole colony run by the reference's own CPU core (needs oracle/_ref),
    on the EUC_2D integer metric, from the oracle's prepared rows; draws from
    std::mt19937_64(seed).  Returns (tour, cost)."""
    R = ref()
    if R is None:
        raise RuntimeError("oracle/_ref is not built")
    xy = np.ascontiguousarray(xy, dtype=np.int32)
    n = xy.shape[0]
    matrix = np.ascontiguousarray(euc2d_matrix(xy), dtype=np.float64)
    kk, bb = prep["primary"].shape[1], prep["backup"].shape[1]
    backup = np.ascontiguousarray(prep["backup"] if bb else np.zeros((n, 1), np.uint32), dtype=np.uint32)
    tour = np.zeros(n, np.uint32)
    cost = C.c_double()
    code = R.ref_colony(n, matrix, np.ascontiguousarray(prep["primary"], np.uint32), kk, backup, bb,
                        np.ascontiguousarray(prep["ls"], np.uint32), prep["ls"].shape[1],
                        np.ascontiguousarray(prep["initial"], np.uint32), float(prep["cost"]), ants,
                        mne, iterations, beta, retention, p_best, epoch_source_probability, ls_limit, seed, tour,
                        C.byref(cost))
    if code != 0:
        raise RuntimeError(f"ref_colony failed ({code})")
    return tour, cost.value


# ---------------------------------------------------------------- helpers

def euc2d_matrix(xy: np.ndarray) -> np.ndarray:
    """Dense EUC_2D matrix (int32) -- floor(sqrt(dx^2+dy^2)+0.5)."""
    xy = np.asarray(xy, dtype=np.int64)
    d = xy[:, None, :] - xy[None, :, :]
    s = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]).astype(np.float64)
    return np.floor(np.sqrt(s) + 0.5).astype(np.int32)


def dist_struct(n, xy=None, matrix=None):
    keep = []
    xy_ptr = mat_ptr = None
    if xy is not None:
        xy = np.ascontiguousarray(xy, dtype=np.int32); keep.append(xy); xy_ptr = xy.ctypes.data
    if matrix is not None:
        matrix = np.ascontiguousarray(matrix, dtype=np.int32); keep.append(matrix); mat_ptr = matrix.ctypes.data
    return DistT(n, xy_ptr, mat_ptr), keep


def distance_ordered(rows: np.ndarray, matrix: np.ndarray) -> np.ndarray:
    """Stable sort of every candidate row by distance (DistanceOrderedCandidates)."""
    rows = np.asarray(rows, dtype=np.uint32)
    out = rows.copy()
    for a in range(rows.shape[0]):
        keys = matrix[a, rows[a]]
        out[a] = rows[a][np.argsort(keys, kind="stable")]
    return out


def ant(parent, ls_rows, mne_target, cap, *, xy=None, matrix=None, visit=None, uniforms=None, start=0,
        primary=None, products32=None, products64=None, backup=None, ls_mode=0):
    """One focused construction + checklist 2-opt.  Returns a dict."""
    parent = np.ascontiguousarray(parent, dtype=np.uint32)
    n = parent.size
    ls_rows = np.ascontiguousarray(ls_rows, dtype=np.uint32)
    w = ls_rows.shape[1]
    d, keep = dist_struct(n, xy, matrix)
    arrays = {}

    def ptr(name, a, dt):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dt); arrays[name] = a
        return a.ctypes.data

    k = 0 if primary is None else np.asarray(primary).shape[1]
    b = 0 if backup is None else np.asarray(backup).shape[1]
    ch = Choices(ptr("visit", visit, np.uint32), ptr("uniforms", uniforms, np.float64), start,
                 ptr("primary", primary, np.uint32), ptr("p32", products32, np.float32),
                 ptr("p64", products64, np.float64), k, ptr("backup", backup, np.uint32), b)
    cons_tour = np.zeros(n, np.uint32); tour = np.zeros(n, np.uint32); pos = np.zeros(n, np.uint32)
    checklist = np.zeros(8 * n + 8, np.uint32); selected = np.zeros(n, np.uint32)
    info = AntInfo()
    rc = lib().orc_ant(parent, C.byref(d), ls_rows, w, C.byref(ch), mne_target, cap, ls_mode, cons_tour, tour, pos,
                       checklist, selected, C.byref(info))
    if rc != 0:
        raise RuntimeError(f"oracle ant failed ({rc})")
    steps = info.cons.steps
    return dict(construction_tour=cons_tour, tour=tour, positions=pos,
                checklist=checklist[:info.checklist_len].copy(), selected=selected[:steps + 1].copy(),
                construction_cost=info.construction_cost, final_cost=info.final_cost,
                mne=info.cons.mne, steps=steps, nonidentity=info.cons.nonidentity_relocations,
                processed=info.ls.processed_nodes, checks=info.ls.candidate_checks,
                evaluations=info.ls.move_evaluations, accepted=info.ls.accepted_moves,
                reactivations=info.ls.reactivations, limit_reached=info.ls.evaluation_limit_reached,
                start=info.start_node)


def heuristic(xy, primary, beta=1.0) -> np.ndarray:
    """The instance heuristic eta = 1/d^beta (1 at d = 0) as FP32 [n, k],
    the value the colony run starts from."""
    d = euc2d_matrix(xy)[np.arange(len(xy))[:, None], np.asarray(primary, np.int64)].astype(np.float64)
    with np.errstate(divide="ignore"):
        v = 1.0 / d if beta == 1.0 else 1.0 / np.power(d, beta)
    return np.where(d > 0, v, 1.0).astype(np.float32)


def prior_eta(eta, prob, floor, gamma) -> np.ndarray:
    """eta * (floor + p)^gamma in FP32, one rounding per operation."""
    eta = np.ascontiguousarray(eta, np.float32)
    prob = np.ascontiguousarray(prob, np.float32).reshape(eta.shape)
    out = np.zeros_like(eta)
    lib().orc_prior_eta(eta.size, eta.reshape(-1), prob.reshape(-1), np.float32(floor), int(gamma), out.reshape(-1))
    return out


def departure_rows(primary, parent, trails, eta, prior_eta_rows) -> np.ndarray:
    """Products of a colony whose prior re-ranks departures only."""
    primary = np.ascontiguousarray(primary, np.uint32)
    n, k = primary.shape
    out = np.zeros((n, k), np.float32)
    lib().orc_departure_rows(n, k, primary, np.ascontiguousarray(parent, np.uint32),
                             np.ascontiguousarray(trails, np.float32).reshape(-1),
                             np.ascontiguousarray(eta, np.float32).reshape(-1),
                             np.ascontiguousarray(prior_eta_rows, np.float32).reshape(-1), out.reshape(-1))
    return out


def alpha_nearness(xy, primary, backup, ls) -> np.ndarray:
    """Alpha-nearness of every primary candidate entry [n, k] (Helsgaun,
    EJOR 126 (2000)): length minus the longest edge on the path between the
    ends in a minimum spanning tree of the candidate graph (the union of the
    primary, backup and LS rows); length where the ends lie in different
    components.  The path maximum is the minimax (bottleneck) length, the same
    for every minimum tree, found here by a walk over the tree from each node."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import minimum_spanning_tree
    xy = np.asarray(xy, np.int64)
    n = len(xy)
    m = euc2d_matrix(xy).astype(np.int64)
    rows = [np.asarray(r, np.int64) for r in (primary, backup, ls) if r is not None and np.asarray(r).size]
    a = np.concatenate([np.repeat(np.arange(n), r.shape[1]) for r in rows])
    c = np.concatenate([r.reshape(-1) for r in rows])
    keep = a != c
    pairs = np.unique(np.stack([np.minimum(a[keep], c[keep]), np.maximum(a[keep], c[keep])], axis=1), axis=0)
    lo, hi = pairs[:, 0], pairs[:, 1]
    # weights + 1: the tree routine drops explicit zeros (coincident points)
    g = coo_matrix((m[lo, hi] + 1, (lo, hi)), shape=(n, n)).tocsr()
    t = minimum_spanning_tree(g).tocoo()
    adj = [[] for _ in range(n)]
    for u, v, wt in zip(t.row, t.col, t.data):
        adj[u].append((v, int(wt) - 1))
        adj[v].append((u, int(wt) - 1))
    primary = np.asarray(primary, np.int64)
    out = np.zeros(primary.shape, np.float32)
    for i in range(n):
        best = np.full(n, -1, np.int64)
        best[i] = 0
        stack = [i]
        while stack:
            v = stack.pop()
            for u, wt in adj[v]:
                if best[u] < 0:
                    best[u] = max(best[v], wt)
                    stack.append(u)
        for r, j in enumerate(primary[i]):
            out[i, r] = m[i, j] - best[j] if best[j] >= 0 else m[i, j]
    return out


def prepare(xy, k, b, w, initial_ls_limit=100000):
    xy = np.ascontiguousarray(xy, dtype=np.int32)
    n = xy.shape[0]
    cfg = PrepCfg(k, b, w, initial_ls_limit)
    primary = np.zeros((n, k), np.uint32); backup = np.zeros((n, max(b, 1)), np.uint32)
    ls = np.zeros((n, w), np.uint32); initial = np.zeros(n, np.uint32)
    cost = lib().orc_prepare(n, xy, C.byref(cfg), primary, backup, ls, initial)
    return dict(primary=primary, backup=backup[:, :b].copy(), ls=ls, initial=initial, cost=int(cost))


def run_colony(xy, prep, *, ants, k, b, w, mne, iterations, key, beta=1.0, retention=0.98, p_best=0.1,
               epoch_source_probability=0.01, ls_limit=100000, threads=1, want_trace=True, ls_mode=0,
               program=None, mask=0xFFFFFFFF, total_iterations=None, instance_key=0, decision_iterations=(),
               force_collisions=False, prior=None):
    """One colony run.  A program (or controller) of feature spec 2 runs the
    reference's 12-feature controller; `instance_key` seeds its sample nodes
    and `decision_iterations` (1-based) capture its decisions, returned under
    "decisions" with the final "control_state".  `prior`: a learned-prior
    schedule, entries (batch, eta [n, k] float32, departures) in batch order
    -- from that batch on the colony's heuristic is eta (the instance's own
    eta for plain FACO), products by the departure rule when departures."""
    xy = np.ascontiguousarray(xy, dtype=np.int32)
    n = xy.shape[0]
    cfg = RunCfg(ants, k, b, w, mne, beta, retention, p_best, epoch_source_probability, ls_limit, threads, ls_mode)
    tour = np.zeros(n, np.uint32)
    cost = C.c_int64()
    trace = (IterTrace * max(iterations, 1))() if want_trace else None
    trails = np.zeros(n * k, np.float32); products = np.zeros(n * k, np.float32)
    backup = np.ascontiguousarray(prep["backup"] if b else np.zeros((n, 1), np.uint32), dtype=np.uint32)
    slots, kind = controller_slots(program) if program is not None else (None, 0)
    points = np.ascontiguousarray(decision_iterations, dtype=np.uint32)
    dec = dict(features=np.zeros((max(points.size, 1), 12, 32), np.float32),
               scores=np.zeros((max(points.size, 1), 32), np.float32), masks=np.zeros(max(points.size, 1), np.uint32),
               actions=np.zeros(max(points.size, 1), np.int32))
    io = ControlIO(instance_key, points.ctypes.data, points.size, dec["features"].ctypes.data,
                   dec["scores"].ctypes.data, dec["masks"].ctypes.data, dec["actions"].ctypes.data)
    io.force_collisions = int(bool(force_collisions))
    args = (n, xy, np.ascontiguousarray(prep["primary"], dtype=np.uint32), backup,
            np.ascontiguousarray(prep["ls"], dtype=np.uint32),
            np.ascontiguousarray(prep["initial"], dtype=np.uint32), prep["cost"], C.byref(cfg),
            key, iterations, tour, C.byref(cost),
            C.cast(trace, C.c_void_p) if trace is not None else None,
            trails.ctypes.data, products.ctypes.data,
            C.cast(slots, C.c_void_p) if slots is not None else None, mask,
            total_iterations or iterations, kind, C.addressof(io))
    if prior is None:
        rc = lib().orc_run_colony(*args)
    else:
        at = np.ascontiguousarray([int(b) for b, _, _ in prior], dtype=np.uint32)
        etas = np.ascontiguousarray(np.stack([np.asarray(e, np.float32).reshape(n * k) for _, e, _ in prior]))
        dep = np.ascontiguousarray([1 if d else 0 for _, _, d in prior], dtype=np.uint32)
        if np.any(np.diff(at.astype(np.int64)) < 0):
            raise ValueError("prior schedule entries must be in batch order")
        sched = PriorSchedule(at.size, at.ctypes.data, etas.ctypes.data, dep.ctypes.data)
        rc = lib().orc_run_colony_prior(*args, C.byref(sched))
    if rc != 0:
        raise RuntimeError(f"oracle colony run failed ({rc})")
    rows = None
    if trace is not None:
        rows = [dict(iteration_best_cost=t.iteration_best_cost, global_cost=t.global_cost,
                     parent_cost=t.parent_cost, iteration_best=t.iteration_best,
                     source_is_epoch=t.source_is_epoch, tau_min=t.tau_min, tau_max=t.tau_max,
                     mne_target=t.mne_target, action=t.action,
                     construction_steps=t.construction_steps, ls_evaluations=t.ls_evaluations)
                for t in trace[:iterations]]
    out = dict(tour=tour, cost=int(cost.value), trace=rows, trails=trails.reshape(n, k),
               products=products.reshape(n, k))
    if slots is not None and slots[0].feature_spec_id == 2:
        fb = io.feedback
        out["control_state"] = dict(archive_size=io.archive_size, stagnant_batches=fb.stagnant_batches,
                                    return_rate=fb.return_rate, ls_work=fb.ls_work,
                                    epoch_batches=fb.epoch_batches, restarts=fb.restarts)
        out["decisions"] = [dict(iteration=int(points[i]), legal_mask=int(dec["masks"][i]),
                                 action=int(dec["actions"][i]), features=dec["features"][i],
                                 scores=dec["scores"][i]) for i in range(points.size)]
    return out


def controller_slots(controller: dict):
    """A program dict (joint) or a controller dict {controller_version: 1,
    representation: joint_single | conditional_three, trees} as the C array
    of program slots (3 for conditional) and the kind (0 joint, 1 conditional)."""
    if "opcode" in controller:
        trees, kind = [controller], 0
    else:
        kind = 1 if controller["representation"] == "conditional_three" else 0
        trees = list(controller["trees"])
    arr = (Program * max(3, len(trees)))()
    for i, t in enumerate(trees):
        arr[i] = program_struct(t)
    return arr, kind


def score_conditional(trees: list, features: np.ndarray, masks: np.ndarray):
    """score_controller of a conditional_three controller (role scores in
    slots 0-9 of each colony's row, the rest 0)."""
    features = np.ascontiguousarray(features, dtype=np.float32)
    masks = np.ascontiguousarray(masks, dtype=np.uint32)
    arr = (Program * 3)(*[program_struct(t) for t in trees])
    scores = np.zeros((masks.size, 32), np.float32)
    actions = np.zeros(masks.size, np.int32)
    lib().orc_score_conditional(C.cast(arr, C.c_void_p), features.reshape(-1), masks, masks.size,
                                scores.reshape(-1), actions)
    return scores, actions


def program_struct(d: dict) -> Program:
    p = Program()
    p.ir_version = d["ir_version"]; p.numeric_spec_id = d["numeric_spec_id"]
    p.feature_spec_id = d["feature_spec_id"]
    ops, operands, bits = d["opcode"], d["operand"], d["constant_bits"]
    p.length = len(ops); p.constants_count = len(bits)
    for i, (o, a) in enumerate(zip(ops, operands)):
        p.opcode[i] = o; p.operand[i] = a
    consts = np.asarray(bits, dtype=np.uint32).view(np.float32)
    for i, c in enumerate(consts):
        p.constants[i] = float(c)
    return p


def score(program: dict, features: np.ndarray, masks: np.ndarray):
    features = np.ascontiguousarray(features, dtype=np.float32)
    masks = np.ascontiguousarray(masks, dtype=np.uint32)
    colonies = masks.size
    p = program_struct(program)
    if lib().orc_validate_program(C.byref(p)) != 0:
        raise ValueError("invalid program")
    scores = np.zeros((colonies, 32), np.float32); actions = np.zeros(colonies, np.int32)
    lib().orc_score(C.byref(p), features.shape[0], features, masks, colonies, scores, actions)
    return scores, actions


# ------------------------------------------- the 12-feature controller pieces

def fingerprint(tour) -> tuple[int, int]:
    tour = np.ascontiguousarray(tour, dtype=np.uint32)
    f = lib().orc_fingerprint(tour, tour.size)
    return int(f.first), int(f.second)


def sample_nodes(n: int, instance_key: int) -> np.ndarray:
    out = np.zeros(min(n, 64), np.uint32)
    lib().orc_sample_nodes(n, instance_key, out)
    return out


def build_region(tour, primary, key, batch, mode, region) -> np.ndarray:
    tour = np.ascontiguousarray(tour, dtype=np.uint32)
    primary = np.ascontiguousarray(primary, dtype=np.uint32)
    out = np.zeros(16, np.uint32)
    lib().orc_build_region(tour, tour.size, primary, primary.shape[1], key, batch, mode, region, out)
    return out[:min(tour.size, 16)]


def local_scale(xy):
    xy = np.ascontiguousarray(xy, dtype=np.int32)
    out = np.zeros(xy.shape[0], np.float64)
    eps = C.c_double()
    lib().orc_local_scale(xy.shape[0], xy, out, C.byref(eps))
    return out, eps.value


class ControlArchive:
    """An archive seeded with entries[0] and updated once with global =
    entries[0] and the other entries as the batch (the reference's
    ReferenceArchive built the same way)."""

    def __init__(self, xy, entries):
        self.xy = np.ascontiguousarray(xy, dtype=np.int32)
        n = self.xy.shape[0]
        self.tours = np.zeros((4, n), np.uint32)
        self.pos = np.zeros((4, n), np.uint32)
        self.s = Archive(n, 1, self.tours.ctypes.data, self.pos.ctypes.data)
        e0 = np.ascontiguousarray(entries[0], dtype=np.uint32)
        self.tours[0] = e0
        self.pos[0, e0] = np.arange(n, dtype=np.uint32)
        self.s.cost[0] = self.length(e0)
        f = lib().orc_fingerprint(e0, n)
        self.s.id[0] = f
        self.update(e0, entries[1:])

    def length(self, tour) -> int:
        return int(np.sum(euc2d_matrix(self.xy)[tour, np.roll(tour, -1)].astype(np.int64)))

    def update(self, global_tour, batch):
        n = self.xy.shape[0]
        g = np.ascontiguousarray(global_tour, dtype=np.uint32)
        cands = np.ascontiguousarray(np.asarray(batch, dtype=np.uint32).reshape(-1, n))
        costs = np.array([self.length(t) for t in cands], np.int64)
        if lib().orc_archive_update(C.byref(self.s), g, self.length(g), cands.reshape(-1) if cands.size
                                    else np.zeros(1, np.uint32), costs if costs.size else np.zeros(1, np.int64),
                                    cands.shape[0]) != 0:
            raise RuntimeError("archive update failed")

    def entries(self):
        return [(self.tours[i].copy(), int(self.s.cost[i]), (int(self.s.id[i].first), int(self.s.id[i].second)))
                for i in range(self.s.size)]


def control_features(xy, primary, samples, scale, epsilon, active, archive: ControlArchive, feedback, trails,
                     default_trail, tau_min, tau_max, elapsed, solve_key, batch, mask):
    """make_action_snapshot in the oracle: features [12][32], regions
    [2][4][16], alternative slot, legal mask."""
    xy = np.ascontiguousarray(xy, dtype=np.int32)
    n = xy.shape[0]
    primary = np.ascontiguousarray(primary, dtype=np.uint32)
    samples = np.ascontiguousarray(samples, dtype=np.uint32)
    scale = np.ascontiguousarray(scale, dtype=np.float64)
    active = np.ascontiguousarray(active, dtype=np.uint32)
    apos = np.zeros(n, np.uint32)
    apos[active] = np.arange(n, dtype=np.uint32)
    trails = np.ascontiguousarray(trails, dtype=np.float64)
    fb = Feedback(feedback[0], feedback[1], int(feedback[2]), int(feedback[3]), int(feedback[4]))
    f = lib().orc_fingerprint(active, n)
    cin = ControlIn(n, xy.ctypes.data, primary.ctypes.data, primary.shape[1], samples.ctypes.data, samples.size,
                    scale.ctypes.data, epsilon, active.ctypes.data, apos.ctypes.data, archive.length(active), f,
                    C.addressof(archive.s), fb, trails.ctypes.data, default_trail, tau_min, tau_max, elapsed,
                    solve_key, batch, mask)
    features = np.zeros((12, 32), np.float32)
    regions = np.zeros((2, 4, 16), np.uint32)
    alt = C.c_uint32()
    legal = lib().orc_control_features(C.byref(cin), features.reshape(-1), regions.reshape(-1), C.byref(alt))
    return dict(features=features, regions=regions, alternative=alt.value, legal=legal)

"""ctypes binding of libcafe_gb300.so (the C ABI in include/cafe_gb300.h).

The library is the only compute path: if it is missing or does not load,
import fails loudly; there is no fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcafe_gb300.so")

CAFE_OK = 0
STATUS = {0: "ok", 1: "oom", 2: "missing matrix", 3: "saturated", 4: "underflow", 5: "timeout",
          6: "invalid", 7: "cuda", 8: "busy", 9: "not found"}
MODEL_BASE, MODEL_GAMMA = 0, 1
LAMBDA_SINGLE, LAMBDA_MULTIPLE = 0, 1
PREC_FP64_REF, PREC_FP64_BINNED, PREC_MIXED_TF32X3 = 0, 1, 2

# every symbol the header declares
EXPORTS = [
    "cafe_ctx_create", "cafe_ctx_destroy", "cafe_last_error", "cafe_status_string", "cafe_version",
    "cafe_tree_upload", "cafe_families_upload", "cafe_families_update", "cafe_families_free",
    "cafe_prior_set", "cafe_error_model_set", "cafe_matrices_build", "cafe_matrix_get",
    "cafe_matrix_cache_size", "cafe_matrix_cache_clear", "cafe_is_saturated", "cafe_score",
    "cafe_score_device", "cafe_submit", "cafe_poll", "cafe_serving_stats", "cafe_profile_enable",
    "cafe_profile_read", "cafe_prune_fp64_noalloc", "cafe_optimize", "cafe_discrete_gamma",
    "cafe_nelder_mead", "cafe_score_batch", "cafe_score_batch_device", "cafe_serving_counters", "cafe_autotune",
    "cafe_reconstruct", "cafe_branch_probabilities", "cafe_pvalues", "cafe_simulate", "cafe_debug_set",
]
DEBUG_TC_WAIT_LIMIT = 1
OPT_LAMBDA, OPT_LAMBDA_ALPHA, OPT_LAMBDA_EPSILON, OPT_ALPHA = 0, 1, 2, 3


class Config(C.Structure):
    _fields_ = [("device", C.c_int), ("matrix_cache_bytes", C.c_size_t), ("n_streams", C.c_int),
                ("max_bins", C.c_int)]


class Request(C.Structure):
    _fields_ = [("tree_id", C.c_int), ("set_id", C.c_int), ("model", C.c_int), ("lambda_kind", C.c_int),
                ("n_lambdas", C.c_int), ("lambdas", C.c_void_p), ("n_categories", C.c_int),
                ("multipliers", C.c_void_p), ("cat_probs", C.c_void_p), ("use_error_model", C.c_int),
                ("max_family_size", C.c_int), ("max_root_family_size", C.c_int), ("precision", C.c_int),
                ("dedupe", C.c_int)]


class Result(C.Structure):
    _fields_ = [("family_lnl", C.c_void_p), ("category_lnl", C.c_void_p), ("total_neg_lnl", C.c_double),
                ("status", C.c_int), ("n_failed", C.c_int64), ("n_fallback", C.c_int64),
                ("device_ms", C.c_double)]


class Timings(C.Structure):
    _fields_ = [("matrix_ms", C.c_double), ("prune_ms", C.c_double), ("finish_ms", C.c_double),
                ("other_ms", C.c_double), ("prune_flops", C.c_double), ("launches", C.c_int64),
                ("prune_launches", C.c_int64), ("matrices_built", C.c_int64), ("host_keys_ms", C.c_double),
                ("host_plan_ms", C.c_double), ("host_total_ms", C.c_double), ("host_build_ms", C.c_double)]


class OptConfig(C.Structure):
    _fields_ = [("kind", C.c_int), ("n_params", C.c_int), ("initial", C.c_void_p), ("max_iterations", C.c_int),
                ("reflection", C.c_double), ("expansion", C.c_double)]


OBJECTIVE = C.CFUNCTYPE(C.c_double, C.POINTER(C.c_double), C.c_int, C.c_void_p)


class OptResult(C.Structure):
    _fields_ = [("values", C.c_void_p), ("score", C.c_double), ("iterations", C.c_int),
                ("evaluations", C.c_int), ("converged", C.c_int)]


class TuneResult(C.Structure):
    _fields_ = [("width", C.c_int), ("ctas_per_sm", C.c_int), ("stages", C.c_int), ("ms", C.c_double)]


class ServingInfo(C.Structure):
    _fields_ = [("batches", C.c_int64), ("merged", C.c_int64), ("retried", C.c_int64), ("enqueue_ms", C.c_double),
                ("wait_ms", C.c_double), ("device_ms", C.c_double), ("overlap_ms", C.c_double)]


class Reconstruction(C.Structure):
    _fields_ = [("node_count", C.c_void_p), ("node_mean", C.c_void_p), ("category_state", C.c_void_p),
                ("root_max", C.c_void_p), ("exhaustive", C.c_int), ("n_failed", C.c_int64),
                ("device_ms", C.c_double)]


class PvaluesOut(C.Structure):
    _fields_ = [("n_simulations", C.c_int), ("seed", C.c_uint32), ("pvalues", C.c_void_p),
                ("conditional", C.c_void_p), ("root_likelihood", C.c_void_p), ("device_ms", C.c_double),
                ("host_ms", C.c_double), ("device_sampling", C.c_int)]


class Simulation(C.Structure):
    _fields_ = [("n_families", C.c_int), ("root_sizes", C.c_void_p), ("seed", C.c_uint32), ("sizes", C.c_void_p),
                ("lambdas", C.c_void_p)]


_lib = None


class CafeError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


def load(path: str = LIB_PATH) -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    i, p, d, i64, sz = C.c_int, C.c_void_p, C.c_double, C.c_int64, C.c_size_t
    P = C.POINTER
    sig = {
        "cafe_ctx_create": (i, [P(Config), P(p)]),
        "cafe_ctx_destroy": (i, [p]),
        "cafe_last_error": (C.c_char_p, [p]),
        "cafe_status_string": (C.c_char_p, [i]),
        "cafe_version": (i, []),
        "cafe_tree_upload": (i, [p, i, p, p, p, P(i)]),
        "cafe_families_upload": (i, [p, i, p, i64, i, P(i)]),
        "cafe_families_update": (i, [p, i, p]),
        "cafe_families_free": (i, [p, i]),
        "cafe_prior_set": (i, [p, p, i]),
        "cafe_error_model_set": (i, [p, p, i, i]),
        "cafe_matrices_build": (i, [p, p, i, p, i, i]),
        "cafe_matrix_get": (i, [p, d, d, i, p]),
        "cafe_matrix_cache_size": (i, [p, P(i64)]),
        "cafe_matrix_cache_clear": (i, [p]),
        "cafe_is_saturated": (i, [d, d]),
        "cafe_score": (i, [p, P(Request), P(Result)]),
        "cafe_score_batch": (i, [p, p, i, p]),
        "cafe_score_batch_device": (i, [p, p, i, p, p, p]),
        "cafe_autotune": (i, [p, p, i, i, p, i, P(i)]),
        "cafe_score_device": (i, [p, P(Request), p, p, p]),
        "cafe_submit": (i, [p, P(Request), P(Result), P(C.c_uint64)]),
        "cafe_poll": (i, [p, C.c_uint64, i]),
        "cafe_serving_stats": (i, [p, P(i64), P(d), P(d), P(i)]),
        "cafe_serving_counters": (i, [p, P(ServingInfo)]),
        "cafe_profile_enable": (i, [p, i]),
        "cafe_profile_read": (i, [p, P(Timings)]),
        "cafe_prune_fp64_noalloc": (i, [i, p, p, i, p, i64, i, i, i, p, i, i, p, p]),
        "cafe_optimize": (i, [p, P(Request), P(OptConfig), P(OptResult)]),
        "cafe_discrete_gamma": (i, [i, d, p, p]),
        "cafe_nelder_mead": (i, [P(OptConfig), OBJECTIVE, p, P(OptResult)]),
        "cafe_reconstruct": (i, [p, P(Request), P(Reconstruction)]),
        "cafe_branch_probabilities": (i, [p, P(Request), p, p]),
        "cafe_pvalues": (i, [p, P(Request), P(PvaluesOut)]),
        "cafe_simulate": (i, [p, P(Request), P(Simulation)]),
        "cafe_debug_set": (i, [p, i, i64]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib

"""Loader of the native library (ferrolearn_gb300/_build/libferrokmeans.so).

There is no fallback: if the library cannot be built or loaded, every entry
point raises. The library itself needs a CUDA driver only when a context is
created, so loading and symbol checks work on a machine without a GPU.
"""
import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libferrokmeans.so")

_lock = threading.Lock()
_lib = None

# Every symbol declared in include/ferrokmeans.h.
EXPORTS = [
    "fk_ctx_create", "fk_ctx_destroy", "fk_last_error_message", "fk_version", "fk_debug_launch_count",
    "fk_kmeans_params_default", "fk_draws_f64",
    "fk_kmeans_fit_f64", "fk_kmeans_fit_f32", "fk_kmeans_fit_f32x64",
    "fk_lloyd_step_f64", "fk_lloyd_step_f32", "fk_lloyd_step_f32x64",
    "fk_kmeans_predict_f64", "fk_kmeans_predict_f32", "fk_kmeans_predict_f32x64",
    "fk_kmeans_transform_f64", "fk_kmeans_transform_f32",
    "fk_kmeans_plus_plus_f64", "fk_kmeans_plus_plus_f32", "fk_debug_tc_probe",
    "fk_debug_measure_peaks", "fk_debug_measure_tc_peaks", "fk_kmeans_score_f64_noalloc", "fk_kmeans_fit_batched_f32", "fk_debug_tc_plan",
    "fk_minibatch_params_default", "fk_minibatch_fit_f64", "fk_minibatch_fit_f32", "fk_minibatch_batch_indices",
    "fk_bisecting_params_default", "fk_bisecting_fit_f64", "fk_bisecting_fit_f32",
]


class BisectingParams(C.Structure):
    _fields_ = [
        ("n_clusters", C.c_int64),
        ("max_iter", C.c_int64),
        ("n_init", C.c_int64),
        ("random_state", C.c_uint64),
        ("has_random_state", C.c_int32),
        ("strategy", C.c_int32),
    ]


class MiniBatchParams(C.Structure):
    _fields_ = [
        ("n_clusters", C.c_int64),
        ("batch_size", C.c_int64),
        ("max_iter", C.c_int64),
        ("tol", C.c_double),
        ("n_init", C.c_int64),
        ("random_state", C.c_uint64),
        ("has_random_state", C.c_int32),
        ("init", C.c_int32),
    ]


class BatchProblem(C.Structure):
    """fk_batch_problem."""

    _fields_ = [
        ("x", C.c_void_p),
        ("n", C.c_int64),
        ("d", C.c_int64),
        ("n_clusters", C.c_int64),
        ("max_iter", C.c_int64),
        ("tol", C.c_double),
        ("n_init", C.c_int64),
        ("random_state", C.c_uint64),
        ("init", C.c_void_p),
        ("centers_out", C.c_void_p),
        ("labels_out", C.c_void_p),
        ("inertia_out", C.c_void_p),
        ("n_iter_out", C.c_void_p),
        ("best_run_out", C.c_void_p),
    ]


class BatchReport(C.Structure):
    """fk_batch_report."""

    _fields_ = [
        ("fits", C.c_int64),
        ("iterations_total", C.c_int64),
        ("graph_launches", C.c_int64),
        ("tuned_buckets", C.c_int64),
        ("bucket_variant", C.c_int32 * 20),
        ("ms_upload", C.c_double),
        ("ms_init", C.c_double),
        ("ms_tune", C.c_double),
        ("ms_lloyd", C.c_double),
        ("ms_download", C.c_double),
        ("ms_total", C.c_double),
        ("fit_inertia", C.c_void_p),
        ("fit_n_iter", C.c_void_p),
    ]


class KMeansParams(C.Structure):
    _fields_ = [
        ("n_clusters", C.c_int64),
        ("max_iter", C.c_int64),
        ("tol", C.c_double),
        ("n_init", C.c_int64),
        ("random_state", C.c_uint64),
        ("has_random_state", C.c_int32),
        ("precision", C.c_int32),
        ("draws", C.c_void_p),
        ("n_draws", C.c_int64),
        ("collect_timing", C.c_int32),
        ("reserved", C.c_int32),
    ]


class FitReport(C.Structure):
    _fields_ = [
        ("best_run", C.c_int64),
        ("iterations_total", C.c_int64),
        ("rows_assigned", C.c_int64),
        ("rows_rechecked", C.c_int64),
        ("rows_full_rescan", C.c_int64),
        ("rows_fp64", C.c_int64),
        ("rows_second_pass", C.c_int64),
        ("rows_few", C.c_int64),
        ("rows_exhaustive", C.c_int64),
        ("near_tie_rows", C.c_int64),
        ("ms_init", C.c_double),
        ("ms_assign", C.c_double),
        ("ms_contract", C.c_double),
        ("ms_update", C.c_double),
        ("ms_total", C.c_double),
        ("precision_used", C.c_int32),
        ("reserved", C.c_int32),
        ("rows_moved", C.c_int64),
        ("updates_incremental", C.c_int64),
        ("count_iterations", C.c_int64),
        ("ms_count_pass", C.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


def _declare(lib):
    p, i64, u64, i32 = C.c_void_p, C.c_int64, C.c_uint64, C.c_int32
    st = C.c_int
    lib.fk_ctx_create.argtypes = [C.POINTER(C.c_void_p), i32, p]
    lib.fk_ctx_create.restype = st
    lib.fk_ctx_destroy.argtypes = [p]
    lib.fk_ctx_destroy.restype = st
    lib.fk_last_error_message.argtypes = []
    lib.fk_last_error_message.restype = C.c_char_p
    lib.fk_version.argtypes = []
    lib.fk_version.restype = C.c_char_p
    lib.fk_debug_launch_count.argtypes = []
    lib.fk_debug_launch_count.restype = C.c_uint64
    lib.fk_kmeans_params_default.argtypes = [C.POINTER(KMeansParams), i64]
    lib.fk_kmeans_params_default.restype = None
    lib.fk_draws_f64.argtypes = [u64, i64, p]
    lib.fk_draws_f64.restype = st
    for suf in ("f64", "f32", "f32x64"):
        f = getattr(lib, f"fk_kmeans_fit_{suf}")
        f.argtypes = [p, p, i64, i64, C.POINTER(KMeansParams), p, p, p, p, p, C.POINTER(FitReport)]
        f.restype = st
        f = getattr(lib, f"fk_lloyd_step_{suf}")
        f.argtypes = [p, p, i64, i64, p, i64, i32, p, p, p, p, C.POINTER(FitReport)]
        f.restype = st
        f = getattr(lib, f"fk_kmeans_predict_{suf}")
        f.argtypes = [p, p, i64, i64, p, i64, i64, i32, p]
        f.restype = st
    for suf in ("f64", "f32"):
        f = getattr(lib, f"fk_kmeans_transform_{suf}")
        f.argtypes = [p, p, i64, i64, p, i64, i64, p]
        f.restype = st
        f = getattr(lib, f"fk_kmeans_plus_plus_{suf}")
        f.argtypes = [p, p, i64, i64, i64, p, i64, u64, p, p]
        f.restype = st
    lib.fk_debug_tc_probe.argtypes = [p, p, i64, i64, p, i64, i32, p, p, p, p, p, p, p]
    lib.fk_debug_tc_probe.restype = st
    lib.fk_debug_measure_peaks.argtypes = [p, p]
    lib.fk_debug_measure_peaks.restype = st
    lib.fk_debug_measure_tc_peaks.argtypes = [p, p]
    lib.fk_debug_measure_tc_peaks.restype = st
    lib.fk_kmeans_score_f64_noalloc.argtypes = [p, i64, i64, p, i64, p, p, p]
    lib.fk_kmeans_score_f64_noalloc.restype = st
    lib.fk_kmeans_fit_batched_f32.argtypes = [p, C.POINTER(BatchProblem), i64, i32, C.POINTER(BatchReport)]
    lib.fk_kmeans_fit_batched_f32.restype = st
    lib.fk_debug_tc_plan.argtypes = [i64, i64, i64, i32, i32, i32, p]
    lib.fk_debug_tc_plan.restype = st
    lib.fk_minibatch_params_default.argtypes = [C.POINTER(MiniBatchParams), i64]
    lib.fk_minibatch_params_default.restype = None
    for suf in ("f64", "f32"):
        f = getattr(lib, f"fk_minibatch_fit_{suf}")
        f.argtypes = [p, p, i64, i64, C.POINTER(MiniBatchParams), p, p, p, p, p, p, C.POINTER(FitReport)]
        f.restype = st
    lib.fk_minibatch_batch_indices.argtypes = [u64, i64, i64, i64, i64, p]
    lib.fk_minibatch_batch_indices.restype = st
    lib.fk_bisecting_params_default.argtypes = [C.POINTER(BisectingParams), i64]
    lib.fk_bisecting_params_default.restype = None
    for suf in ("f64", "f32"):
        f = getattr(lib, f"fk_bisecting_fit_{suf}")
        f.argtypes = [p, p, i64, i64, C.POINTER(BisectingParams), p, p, p, p]
        f.restype = st


def lib():
    """Load (building first if needed) the native library; raises on failure."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                from . import build as _build
                _build.build()
            handle = C.CDLL(LIB_PATH)
            missing = [s for s in EXPORTS if not hasattr(handle, s)]
            if missing:
                raise ImportError(f"{LIB_PATH} lacks symbols: {missing}")
            _declare(handle)
            _lib = handle
    return _lib


def last_error():
    msg = lib().fk_last_error_message()
    return msg.decode("utf-8", "replace") if msg else ""

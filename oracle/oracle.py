"""ctypes wrapper around the CPU oracle (oracle/kmeans_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, always as the result compared against (or
timed as the CPU baseline). The product library
(ferrolearn_gb300) never imports this module.

Each function restates one item of ferrolearn-cluster/src/kmeans.rs (the C
file cites the lines). Arrays are numpy, row-major, f64 or f32.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = C.CDLL(path)
        i64, u64, p = C.c_int64, C.c_uint64, C.c_void_p
        for suf, T in (("f64", C.c_double), ("f32", C.c_float)):
            getattr(_lib, f"orc_assign_{suf}").argtypes = [p, i64, i64, p, i64, p, p, C.c_int]
            getattr(_lib, f"orc_assign_{suf}").restype = T
            getattr(_lib, f"orc_update_{suf}").argtypes = [p, i64, i64, p, p, i64, p, p]
            getattr(_lib, f"orc_update_{suf}").restype = T
            getattr(_lib, f"orc_kmeanspp_{suf}").argtypes = [p, i64, i64, i64, p, i64, u64, p, p]
            getattr(_lib, f"orc_lloyd_step_{suf}").argtypes = [p, i64, i64, p, i64, p, p, p, p, C.c_int]
            getattr(_lib, f"orc_fit_{suf}").argtypes = [p, i64, i64, i64, i64, T, i64, p, p, i64, u64,
                                                        p, p, p, p, p, C.c_int]
            getattr(_lib, f"orc_predict_{suf}").argtypes = [p, i64, i64, p, i64, i64, p, C.c_int]
            getattr(_lib, f"orc_transform_{suf}").argtypes = [p, i64, i64, p, i64, i64, p, C.c_int]
            getattr(_lib, f"orc_minibatch_fit_{suf}").argtypes = [p, i64, i64, i64, i64, i64, T, i64, u64, C.c_int,
                                                                  p, p, p, p, p, p, p, p]
            getattr(_lib, f"orc_bisecting_fit_{suf}").argtypes = [p, i64, i64, i64, i64, i64, u64, C.c_int, p, p,
                                                                  p, p]
        _lib.orc_mb_batch_indices.argtypes = [u64, i64, i64, i64, i64, p]
        _lib.orc_draws_f64.argtypes = [u64, i64, p]
        _lib.orc_draws_f64.restype = None
        _lib.orc_fit_runs_f32.argtypes = [p, i64, i64, i64, i64, C.c_float, i64, p, u64, C.c_int, p, p, p, p,
                                          C.c_int]
        _lib.orc_update_given_labels_f32x64.argtypes = [p, i64, i64, p, p, i64, p, p, C.c_int]
        _lib.orc_update_rows_f64.argtypes = [p, i64, i64, p, i64, p, p]
        _lib.orc_update_finish_f64.argtypes = [p, p, p, i64, i64, p, p]
    return _lib


def _threads(nthreads):
    if nthreads is None:
        return os.cpu_count() or 1
    return int(nthreads)


def _suffix(dtype):
    if dtype == np.float64:
        return "f64", C.c_double
    if dtype == np.float32:
        return "f32", C.c_float
    raise TypeError(f"oracle supports float64/float32, got {dtype}")


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleError(Exception):
    def __init__(self, code):
        super().__init__(f"oracle status {code}")
        self.code = code


def draws(seed, count):
    out = np.empty(count, dtype=np.float64)
    lib().orc_draws_f64(seed, count, _ptr(out))
    return out


def assign(x, centers, nthreads=None):
    """assign_clusters_into (kmeans.rs:279-352) -> (labels int64, inertia)."""
    x = np.ascontiguousarray(x)
    c = np.ascontiguousarray(centers, dtype=x.dtype)
    suf, _ = _suffix(x.dtype)
    n, d = x.shape
    labels = np.empty(n, dtype=np.int64)
    inertia = getattr(lib(), f"orc_assign_{suf}")(_ptr(x), n, d, _ptr(c), c.shape[0], _ptr(labels), None,
                                                  _threads(nthreads))
    return labels, inertia


def lloyd_step(x, centers, nthreads=None):
    """One iteration of kmeans.rs:468-488: (labels, new_centers, inertia, max_shift)."""
    x = np.ascontiguousarray(x)
    c = np.ascontiguousarray(centers, dtype=x.dtype)
    suf, T = _suffix(x.dtype)
    n, d = x.shape
    k = c.shape[0]
    labels = np.empty(n, dtype=np.int64)
    nc = np.empty_like(c)
    inertia, shift = T(), T()
    rc = getattr(lib(), f"orc_lloyd_step_{suf}")(_ptr(x), n, d, _ptr(c), k, _ptr(labels), _ptr(nc),
                                                 C.byref(inertia), C.byref(shift), _threads(nthreads))
    if rc:
        raise OracleError(rc)
    return labels, nc, inertia.value, shift.value


def update_given_labels(x32, labels, centers, nthreads=None):
    """recompute_centroids_into (kmeans.rs:358-401) for KMeans<f64> on f32
    rows widened exactly, from the given labels, and the inertia of those
    labels against `centers` folded in row order -> (new_centers, inertia)."""
    x32 = np.ascontiguousarray(x32, dtype=np.float32)
    lab = np.ascontiguousarray(labels, dtype=np.int64)
    c = np.ascontiguousarray(centers, dtype=np.float64)
    n, d = x32.shape
    nc = np.empty_like(c)
    inertia = C.c_double()
    rc = lib().orc_update_given_labels_f32x64(_ptr(x32), n, d, _ptr(lab), _ptr(c), c.shape[0], _ptr(nc),
                                              C.byref(inertia), _threads(nthreads))
    if rc:
        raise OracleError(rc)
    return nc, inertia.value


def update_rows(x, labels, sums, counts):
    """The first loop of recompute_centroids_into (kmeans.rs:370-375), F = f64,
    over the given rows, adding into sums (k x d) and counts (k) in place."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    lab = np.ascontiguousarray(labels, dtype=np.int64)
    assert sums.dtype == np.float64 and sums.flags.c_contiguous and counts.dtype == np.float64
    rc = lib().orc_update_rows_f64(_ptr(x), x.shape[0], x.shape[1], _ptr(lab), sums.shape[0], _ptr(sums),
                                   _ptr(counts))
    if rc:
        raise OracleError(rc)


def update_finish(sums, counts, centers):
    """The rest of recompute_centroids_into (kmeans.rs:377-400) -> (new_centers, max_shift)."""
    c = np.ascontiguousarray(centers, dtype=np.float64)
    nc = np.empty_like(c)
    shift = C.c_double()
    rc = lib().orc_update_finish_f64(_ptr(sums), _ptr(counts), _ptr(c), c.shape[0], c.shape[1], _ptr(nc),
                                     C.byref(shift))
    if rc:
        raise OracleError(rc)
    return nc, shift.value


def kmeanspp(x, k, draws_arr=None, seed=0):
    """kmeans_plus_plus (kmeans.rs:169-253) -> (centers, draws consumed)."""
    x = np.ascontiguousarray(x)
    suf, _ = _suffix(x.dtype)
    n, d = x.shape
    out = np.empty((k, d), dtype=x.dtype)
    used = C.c_int64()
    dr = None if draws_arr is None else np.ascontiguousarray(draws_arr, dtype=np.float64)
    rc = getattr(lib(), f"orc_kmeanspp_{suf}")(_ptr(x), n, d, k, _ptr(dr), 0 if dr is None else dr.size,
                                               seed, _ptr(out), C.byref(used))
    if rc:
        raise OracleError(rc)
    return out, used.value


def fit(x, k, max_iter=300, tol=1e-4, n_init=10, init=None, draws_arr=None, seed=0, nthreads=None):
    """Fit::fit (kmeans.rs:417-512) -> dict(centers, labels, inertia, n_iter, best_run)."""
    x = np.ascontiguousarray(x)
    suf, T = _suffix(x.dtype)
    n, d = x.shape if x.ndim == 2 else (0, 0)
    out_c = np.empty((max(k, 0), d), dtype=x.dtype)
    out_l = np.empty(n, dtype=np.int64)
    inertia, n_iter, best = T(), C.c_int64(), C.c_int64()
    ini = None if init is None else np.ascontiguousarray(init, dtype=x.dtype)
    dr = None if draws_arr is None else np.ascontiguousarray(draws_arr, dtype=np.float64)
    rc = getattr(lib(), f"orc_fit_{suf}")(_ptr(x), n, d, k, max_iter, T(tol), n_init, _ptr(ini), _ptr(dr),
                                          0 if dr is None else dr.size, seed, _ptr(out_c), _ptr(out_l),
                                          C.byref(inertia), C.byref(n_iter), C.byref(best),
                                          _threads(nthreads))
    if rc:
        raise OracleError(rc)
    return dict(centers=out_c, labels=out_l, inertia=inertia.value, n_iter=n_iter.value,
                best_run=best.value)


def predict(centers, x, nthreads=None):
    x = np.ascontiguousarray(x)
    c = np.ascontiguousarray(centers, dtype=x.dtype)
    suf, _ = _suffix(x.dtype)
    n, d = x.shape
    labels = np.empty(n, dtype=np.int64)
    rc = getattr(lib(), f"orc_predict_{suf}")(_ptr(c), c.shape[0], c.shape[1], _ptr(x), n, d, _ptr(labels),
                                              _threads(nthreads))
    if rc:
        raise OracleError(rc)
    return labels


def transform(centers, x, nthreads=None):
    x = np.ascontiguousarray(x)
    c = np.ascontiguousarray(centers, dtype=x.dtype)
    suf, _ = _suffix(x.dtype)
    n, d = x.shape
    out = np.empty((n, c.shape[0]), dtype=x.dtype)
    rc = getattr(lib(), f"orc_transform_{suf}")(_ptr(c), c.shape[0], c.shape[1], _ptr(x), n, d, _ptr(out),
                                                _threads(nthreads))
    if rc:
        raise OracleError(rc)
    return out


def fit_runs(x, k, max_iter=300, tol=1e-4, n_init=10, init=None, seed=0, wide_sums=False, nthreads=None):
    """Fit::fit (kmeans.rs:417-512) for f32 with every run kept (run r seeds
    k-means++ with seed + r): dict(centers (n_init,k,d), labels (n_init,n),
    inertia (n_init,) f64, n_iter (n_init,)). wide_sums: centroid sums and
    inertia in f64 (the batched entry point's FP64 reduction variant)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    n, d = x.shape
    out_c = np.empty((n_init, k, d), dtype=np.float32)
    out_l = np.empty((n_init, n), dtype=np.int64)
    out_i = np.empty(n_init, dtype=np.float64)
    out_n = np.empty(n_init, dtype=np.int64)
    ini = None if init is None else np.ascontiguousarray(init, dtype=np.float32)
    rc = lib().orc_fit_runs_f32(_ptr(x), n, d, k, max_iter, C.c_float(tol), n_init, _ptr(ini), seed,
                                1 if wide_sums else 0, _ptr(out_c), _ptr(out_l), _ptr(out_i), _ptr(out_n),
                                _threads(nthreads))
    if rc:
        raise OracleError(rc)
    return dict(centers=out_c, labels=out_l, inertia=out_i, n_iter=out_n)


def minibatch_fit(x, k, batch_size=1024, max_iter=100, tol=0.0, n_init=3, seed=0, init="kmeans++", init_centers=None):
    """MiniBatchKMeans::fit (mini_batch_kmeans.rs:492-591) with the library's
    uniform stream: dict(centers, labels, inertia, n_iter, best_run,
    run_n_iter, run_inertia). init: "kmeans++" or "random"; init_centers
    ((n_init, k, d)) replaces either."""
    x = np.ascontiguousarray(x)
    suf, T = _suffix(x.dtype)
    n, d = x.shape if x.ndim == 2 else (0, 0)
    out_c = np.empty((max(k, 0), d), dtype=x.dtype)
    out_l = np.empty(n, dtype=np.int64)
    inertia, n_iter, best = T(), C.c_int64(), C.c_int64()
    runs = max(n_init, 1)
    run_n = np.zeros(runs, dtype=np.int64)
    run_i = np.zeros(runs, dtype=x.dtype)
    ini = None if init_centers is None else np.ascontiguousarray(init_centers, dtype=x.dtype)
    mode = {"kmeans++": 0, "random": 1}[init]
    rc = getattr(lib(), f"orc_minibatch_fit_{suf}")(_ptr(x), n, d, k, batch_size, max_iter, T(tol), n_init, seed,
                                                    mode, _ptr(ini), _ptr(out_c), _ptr(out_l), C.byref(inertia),
                                                    C.byref(n_iter), C.byref(best), _ptr(run_n), _ptr(run_i))
    if rc:
        raise OracleError(rc)
    return dict(centers=out_c, labels=out_l, inertia=inertia.value, n_iter=n_iter.value, best_run=best.value,
                run_n_iter=run_n, run_inertia=run_i)


def minibatch_indices(seed, pos, n, batch_size, iters):
    """sample_batch_indices (mini_batch_kmeans.rs:451-472) for `iters`
    iterations from stream position pos: (iters, min(batch_size, n)) int64."""
    m = min(batch_size, n)
    out = np.empty((iters, m), dtype=np.int64)
    rc = lib().orc_mb_batch_indices(seed, pos, n, batch_size, iters, _ptr(out))
    if rc:
        raise OracleError(rc)
    return out


def bisecting_fit(x, k, max_iter=300, n_init=10, seed=0, strategy="largest_cluster"):
    """BisectingKMeans::fit (bisecting_kmeans.rs:326-505) with the library's
    uniform stream (run r of split s seeded with seed + s * 1000 + r):
    dict(centers (n_clusters, d), labels, inertia, n_clusters)."""
    x = np.ascontiguousarray(x)
    suf, T = _suffix(x.dtype)
    n, d = x.shape if x.ndim == 2 else (0, 0)
    out_c = np.zeros((max(k, 0), d), dtype=x.dtype)
    out_l = np.zeros(n, dtype=np.int64)
    inertia, nc = T(), C.c_int64()
    strat = {"largest_cluster": 0, "largest_sse": 1}[strategy]
    rc = getattr(lib(), f"orc_bisecting_fit_{suf}")(_ptr(x), n, d, k, max_iter, n_init, seed, strat, _ptr(out_c),
                                                    _ptr(out_l), C.byref(inertia), C.byref(nc))
    if rc:
        raise OracleError(rc)
    return dict(centers=out_c[:nc.value].copy(), labels=out_l, inertia=inertia.value, n_clusters=nc.value)

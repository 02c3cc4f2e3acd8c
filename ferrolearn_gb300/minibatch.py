"""Host-side mirror of ferrolearn-cluster's MiniBatchKMeans over the C ABI.

Mirrors ferrolearn-cluster/src/mini_batch_kmeans.rs:
  MiniBatchKMeans<F>     builder (:78-161): new / with_batch_size /
                         with_max_iter / with_tol / with_n_init /
                         with_random_state / with_init
  MiniBatchKMeansInit    "kmeans++" (KMeansPlusPlus) or "random" (Random)
  Fit::fit               :492-591 -> FittedMiniBatchKMeans
  FittedMiniBatchKMeans  getters cluster_centers / labels / inertia / n_iter
                         (:173-208); predict (:607-630) and transform
                         (:632-682) are KMeans's (nearest centre with the
                         lowest index on ties; Euclidean distances)
  fit_predict            :601-604

One builder method has no reference counterpart: with_init_centers (explicit
initial centres per run). The reference draws from rand's StdRng, which
cannot be reproduced here; run r draws the library's uniform stream seeded
with random_state + r * 1000003 instead (fk_minibatch_fit_* in
include/ferrokmeans.h), and the oracle restates the same stream.

F is chosen with dtype: "f64" (MiniBatchKMeans<f64>) or "f32".
"""
import ctypes as C

import numpy as np

from . import _native
from .kmeans import (FittedKMeans, InvalidParameter, ShapeMismatch, _as_matrix, _check, _check_out, _ptr,
                     default_context)

_INITS = {"kmeans++": 0, "k-means++": 0, "kmeansplusplus": 0, "random": 1}


def _dtypes(kind):
    if kind == "f64":
        return np.float64, "f64"
    if kind == "f32":
        return np.float32, "f32"
    raise ValueError(f"dtype must be 'f64' or 'f32', got {kind!r}")


class FittedMiniBatchKMeans(FittedKMeans):
    """FittedMiniBatchKMeans<F> (mini_batch_kmeans.rs:173-208)."""


class MiniBatchKMeans:
    """MiniBatchKMeans<F> configuration (unfitted); mini_batch_kmeans.rs:78-161."""

    def __init__(self, n_clusters, dtype="f64"):
        self.n_clusters = int(n_clusters)
        self.batch_size = 1024
        self.max_iter = 100
        self.tol = 0.0
        self.n_init = 3
        self.random_state = None
        self.init = "kmeans++"
        self.init_centers = None
        self.dtype = dtype
        _dtypes(dtype)

    @classmethod
    def new(cls, n_clusters, dtype="f64"):
        return cls(n_clusters, dtype)

    def with_batch_size(self, batch_size):
        self.batch_size = int(batch_size)
        return self

    def with_max_iter(self, max_iter):
        self.max_iter = int(max_iter)
        return self

    def with_tol(self, tol):
        self.tol = float(tol)
        return self

    def with_n_init(self, n_init):
        self.n_init = int(n_init)
        return self

    def with_random_state(self, seed):
        self.random_state = int(seed)
        return self

    def with_init(self, init):
        """MiniBatchKMeansInit: "kmeans++" or "random"."""
        key = str(init).lower()
        if key not in _INITS:
            raise InvalidParameter(f"Invalid parameter `init`: {init!r}")
        self.init = key
        return self

    def with_init_centers(self, centers):
        """Explicit initial centres: (k, d) for every run, or (n_init, k, d)."""
        self.init_centers = centers
        return self

    def _params(self):
        p = _native.MiniBatchParams()
        _native.lib().fk_minibatch_params_default(C.byref(p), self.n_clusters)
        p.batch_size = self.batch_size
        p.max_iter = self.max_iter
        p.tol = self.tol
        p.n_init = self.n_init
        if self.random_state is not None:
            p.random_state = self.random_state
            p.has_random_state = 1
        p.init = _INITS[self.init]
        return p

    def fit(self, x, y=None, ctx=None, out=None):
        """Fit::fit (mini_batch_kmeans.rs:492-591). out: optional (centres,
        labels) buffers (k x d of the dtype, n of int64/uint64) that receive
        the results in place of new host arrays."""
        ct, suf = _dtypes(self.dtype)
        ctx = ctx or default_context()
        x = _as_matrix(x, ct, ctx)
        n, d = int(x.shape[0]), int(x.shape[1])
        k = self.n_clusters
        init = None
        if self.init_centers is not None:
            ini = np.asarray(self.init_centers, dtype=ct)
            if ini.ndim == 2:
                ini = np.broadcast_to(ini, (max(self.n_init, 1),) + ini.shape)
            ini = np.ascontiguousarray(ini)
            if ini.shape[1:] != (k, d) or ini.shape[0] < max(self.n_init, 1):
                raise ShapeMismatch(f"init centres shape {ini.shape} does not match (n_init, {k}, {d})")
            init = ini
        if out is not None:
            centers, labels = out
            _check_out(centers, ct, (max(k, 0), d), "centres out", ctx)
            _check_out(labels, np.uint64, (n,), "labels out", ctx)
        else:
            centers = np.empty((max(k, 0), d), dtype=ct)
            labels = np.empty(n, dtype=np.uint64)
        inertia = (C.c_double if ct == np.float64 else C.c_float)()
        n_iter, best = C.c_int64(), C.c_int64()
        rep = _native.FitReport()
        params = self._params()
        fn = getattr(_native.lib(), f"fk_minibatch_fit_{suf}")
        _check(fn(ctx.handle, _ptr(x), n, d, C.byref(params), _ptr(init), _ptr(centers), _ptr(labels),
                  C.byref(inertia), C.byref(n_iter), C.byref(best), C.byref(rep)))
        lab = labels if out is not None else labels.view(np.int64)  # labels < 2^63: the same bits, no copy
        report = rep.as_dict()
        report["best_run"] = best.value
        return FittedMiniBatchKMeans(centers, lab, inertia.value, n_iter.value, self.dtype, report)

    def fit_predict(self, x, ctx=None):
        """mini_batch_kmeans.rs:601-604: fit, then predict on the same rows."""
        return self.fit(x, ctx=ctx).predict(x, ctx=ctx)


def minibatch_batch_indices(seed, pos, n, batch_size, iters):
    """The batch rows MiniBatchKMeans draws (sample_batch_indices,
    mini_batch_kmeans.rs:451-472) for `iters` iterations from position pos of
    the library's uniform stream: (iters, min(batch_size, n)) int64."""
    m = min(int(batch_size), int(n))
    out = np.empty((max(int(iters), 0), max(m, 0)), dtype=np.int64)
    _check(_native.lib().fk_minibatch_batch_indices(seed, pos, n, batch_size, iters, _ptr(out)))
    return out

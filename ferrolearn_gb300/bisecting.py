"""Host-side mirror of ferrolearn-cluster's BisectingKMeans over the C ABI.

Mirrors ferrolearn-cluster/src/bisecting_kmeans.rs:
  BisectingKMeans<F>      builder (:72-131): new / with_max_iter /
                          with_n_init / with_random_state /
                          with_bisecting_strategy
  BisectingStrategy       "largest_cluster" or "largest_sse"
  Fit::fit                :326-505 -> FittedBisectingKMeans
  FittedBisectingKMeans   cluster_centers / labels / inertia / n_clusters
                          (:138-171); predict (:521-566) and transform
                          (:568-605) are KMeans's (nearest centre, lowest
                          index on ties; Euclidean distances)
  fit_predict             :508-519

Run r of split s draws the library's uniform stream seeded with
random_state + s * 1000 + r (the reference's seeds on rand's StdRng, which
cannot be reproduced here; the oracle restates the same stream).

F is chosen with dtype: "f64" (BisectingKMeans<f64>) or "f32".
"""
import ctypes as C

import numpy as np

from . import _native
from .kmeans import FittedKMeans, InvalidParameter, _as_matrix, _check, _ptr, default_context

_STRATEGIES = {"largest_cluster": 0, "largest_sse": 1}


def _dtypes(kind):
    if kind == "f64":
        return np.float64, "f64"
    if kind == "f32":
        return np.float32, "f32"
    raise ValueError(f"dtype must be 'f64' or 'f32', got {kind!r}")


class FittedBisectingKMeans(FittedKMeans):
    """FittedBisectingKMeans<F> (bisecting_kmeans.rs:138-171)."""

    def __init__(self, centers, labels, inertia, dtype):
        super().__init__(centers, labels, inertia, 0, dtype)

    def n_clusters(self):
        return int(self._centers.shape[0])

    def predict(self, x, ctx=None, precision=None):
        """Predict (bisecting_kmeans.rs:521-566): nearest centre (isize labels)."""
        return super().predict(x, ctx=ctx)


class BisectingKMeans:
    """BisectingKMeans<F> configuration (unfitted); bisecting_kmeans.rs:72-131."""

    def __init__(self, n_clusters, dtype="f64"):
        self.n_clusters = int(n_clusters)
        self.max_iter = 300
        self.n_init = 10
        self.random_state = None
        self.strategy = "largest_cluster"
        self.dtype = dtype
        _dtypes(dtype)

    @classmethod
    def new(cls, n_clusters, dtype="f64"):
        return cls(n_clusters, dtype)

    def with_max_iter(self, max_iter):
        self.max_iter = int(max_iter)
        return self

    def with_n_init(self, n_init):
        self.n_init = int(n_init)
        return self

    def with_random_state(self, seed):
        self.random_state = int(seed)
        return self

    def with_bisecting_strategy(self, strategy):
        key = str(strategy).lower()
        if key not in _STRATEGIES:
            raise InvalidParameter(f"Invalid parameter `bisecting_strategy`: {strategy!r}")
        self.strategy = key
        return self

    def fit(self, x, y=None, ctx=None):
        """Fit::fit (bisecting_kmeans.rs:326-505)."""
        ct, suf = _dtypes(self.dtype)
        ctx = ctx or default_context()
        x = _as_matrix(x, ct, ctx)
        n, d = int(x.shape[0]), int(x.shape[1])
        p = _native.BisectingParams()
        _native.lib().fk_bisecting_params_default(C.byref(p), self.n_clusters)
        p.max_iter = self.max_iter
        p.n_init = self.n_init
        if self.random_state is not None:
            p.random_state = self.random_state
            p.has_random_state = 1
        p.strategy = _STRATEGIES[self.strategy]
        centers = np.zeros((max(self.n_clusters, 0), d), dtype=ct)
        labels = np.empty(n, dtype=np.int64)
        inertia = (C.c_double if ct == np.float64 else C.c_float)()
        nc = C.c_int64()
        fn = getattr(_native.lib(), f"fk_bisecting_fit_{suf}")
        _check(fn(ctx.handle, _ptr(x), n, d, C.byref(p), _ptr(centers), _ptr(labels), C.byref(inertia),
                  C.byref(nc)))
        return FittedBisectingKMeans(np.ascontiguousarray(centers[:nc.value]), labels, inertia.value, self.dtype)

    def fit_predict(self, x, ctx=None):
        """bisecting_kmeans.rs:508-519: fit, then predict on the same rows."""
        return self.fit(x, ctx=ctx).predict(x, ctx=ctx)

"""sklearn-style KMeans on the GB300 library: the drop-in for ferrolearn-python's
wrapper (ferrolearn-python/python/ferrolearn/_clusterers.py:15-84).

Same constructor keywords (n_clusters=8, max_iter=300, tol=1e-4, n_init=10,
random_state=None), the same fitted attributes (cluster_centers_, labels_,
inertia_, n_iter_) and the same methods (fit, predict, transform,
fit_predict), backed by ferrolearn_gb300.KMeans instead of the PyO3 class
_RsKMeans. Two keywords are added: `precision` ("plain": the reference's FP64
arithmetic; "bf16" / "fp8": the tensor-core forms, which read X as float32
and whose labels equal the FP64 ones on those rows) and `device` (the GPU
index). A tensor-core fit of data that float32 does not hold exactly warns.

With scikit-learn installed the class derives from its BaseEstimator,
ClusterMixin and TransformerMixin (get_params / set_params / clone work like
the reference's); without it the same class stands alone.

MiniBatchKMeans below is the drop-in for the reference's mini-batch wrapper
(_extras.py:396-420), backed by ferrolearn_gb300.MiniBatchKMeans.
"""
import warnings

import numpy as np

from .kmeans import PLAIN, _prec
from .kmeans import KMeans as _KMeans
from .kmeans import default_context

try:  # the wrapper's base classes when scikit-learn is present
    from sklearn.base import BaseEstimator, ClusterMixin, TransformerMixin
    _BASES = (TransformerMixin, ClusterMixin, BaseEstimator)
    _CLUSTER_BASES = (ClusterMixin, BaseEstimator)
except ImportError:  # pragma: no cover - exercised where scikit-learn is absent
    _BASES = _CLUSTER_BASES = (object,)


def _as_f64(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    if x.ndim != 2:
        raise ValueError(f"Expected 2D array, got {x.ndim}D array instead")
    return x


class KMeans(*_BASES):
    """K-Means clustering on one GB300 (kmeans.rs Fit / Predict / Transform)."""

    def __init__(self, *, n_clusters=8, max_iter=300, tol=1e-4, n_init=10, random_state=None, precision="plain",
                 device=0):
        self.n_clusters = n_clusters
        self.max_iter = max_iter
        self.tol = tol
        self.n_init = n_init
        self.random_state = random_state
        self.precision = precision
        self.device = device

    def _plain(self):
        return _prec(self.precision) == PLAIN

    def _model(self):
        dtype = "f64" if self._plain() else "f32x64"
        m = _KMeans(self.n_clusters, dtype=dtype).with_max_iter(self.max_iter).with_tol(self.tol) \
            .with_n_init(self.n_init).with_precision(self.precision)
        if self.random_state is not None:
            m = m.with_random_state(self.random_state)
        return m

    def _rows(self, X):
        x = _as_f64(X)
        if self._plain():
            return x
        # the mixed precisions read X as f32 (KMeans<f64> semantics on f32 storage)
        x32 = np.ascontiguousarray(x, dtype=np.float32)
        if not np.array_equal(x32, x, equal_nan=True):
            warnings.warn(f"precision={self.precision!r} reads X as float32 and X holds values that float32 "
                          "rounds: the results are those of the rounded rows (use precision='plain' for the "
                          "float64 rows)", stacklevel=3)
        return x32

    def fit(self, X, y=None):
        x = self._rows(X)
        self.n_features_in_ = x.shape[1]
        self._fitted = self._model().fit(x, ctx=default_context(self.device))
        self.cluster_centers_ = np.array(self._fitted.cluster_centers())
        self.labels_ = np.asarray(self._fitted.labels())
        self.inertia_ = float(self._fitted.inertia())
        self.n_iter_ = int(self._fitted.n_iter())
        return self

    def _check_fitted(self):
        if not hasattr(self, "_fitted"):
            raise AttributeError("This KMeans instance is not fitted yet. Call 'fit' first.")

    def predict(self, X):
        self._check_fitted()
        return np.asarray(self._fitted.predict(self._rows(X), ctx=default_context(self.device)))

    def transform(self, X):
        self._check_fitted()
        return np.array(self._fitted.transform(_as_f64(X), ctx=default_context(self.device)))

    def fit_predict(self, X, y=None):
        return self.fit(X).labels_

    def fit_transform(self, X, y=None):
        return self.fit(X).transform(X)

    def __getstate__(self):
        state = self.__dict__.copy()
        fitted = state.pop("_fitted", None)
        if fitted is not None:  # keep what predict / transform need
            state["_fitted_state"] = (np.asarray(fitted.cluster_centers()), fitted.dtype, fitted.precision)
        return state

    def __setstate__(self, state):
        saved = state.pop("_fitted_state", None)
        self.__dict__.update(state)
        if saved is not None:
            from .kmeans import FittedKMeans
            centres, dtype, precision = saved
            self._fitted = FittedKMeans(centres, np.asarray(self.labels_), self.inertia_, self.n_iter_, dtype,
                                        precision=precision)


class MiniBatchKMeans(*_CLUSTER_BASES):
    """Mini-batch K-Means on one GB300: the drop-in for ferrolearn-python's
    MiniBatchKMeans wrapper (ferrolearn-python/python/ferrolearn/_extras.py:
    396-420, the PyO3 class _RsMiniBatchKMeans of src/extras.rs:693-735).

    Same keywords and defaults (n_clusters=8, max_iter=100,
    random_state=None; the other hyper-parameters are MiniBatchKMeans::new's),
    the fitted labels_ and n_features_in_, fit / predict / fit_predict; also
    cluster_centers_, inertia_, n_iter_ and the `device` keyword."""

    def __init__(self, *, n_clusters=8, max_iter=100, random_state=None, device=0):
        self.n_clusters = n_clusters
        self.max_iter = max_iter
        self.random_state = random_state
        self.device = device

    def fit(self, X, y=None):
        from .minibatch import MiniBatchKMeans as _MiniBatch
        x = _as_f64(X)
        m = _MiniBatch(self.n_clusters).with_max_iter(self.max_iter)
        if self.random_state is not None:
            m = m.with_random_state(self.random_state)
        self._fitted = m.fit(x, ctx=default_context(self.device))
        self.n_features_in_ = x.shape[1]
        self.labels_ = np.asarray(self._fitted.labels())
        self.cluster_centers_ = np.array(self._fitted.cluster_centers())
        self.inertia_ = float(self._fitted.inertia())
        self.n_iter_ = int(self._fitted.n_iter())
        return self

    def predict(self, X):
        if not hasattr(self, "_fitted"):
            raise AttributeError("This MiniBatchKMeans instance is not fitted yet. Call 'fit' first.")
        return np.asarray(self._fitted.predict(_as_f64(X), ctx=default_context(self.device)))

    def fit_predict(self, X, y=None):
        return self.fit(X).labels_

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

from .kmeans import PLAIN, FittedKMeans, _prec
from .kmeans import KMeans as _KMeans
from .kmeans import default_context

try:  # the wrapper's base classes and input validation when scikit-learn is present
    from sklearn.base import BaseEstimator, ClusterMixin, TransformerMixin
    from sklearn.exceptions import NotFittedError
    from sklearn.utils.validation import check_is_fitted as _sk_check_is_fitted
    from sklearn.utils.validation import validate_data as _sk_validate_data
    _BASES = (TransformerMixin, ClusterMixin, BaseEstimator)
    _CLUSTER_BASES = (ClusterMixin, BaseEstimator)
except ImportError:  # pragma: no cover - exercised where scikit-learn is absent
    _BASES = _CLUSTER_BASES = (object,)
    _sk_validate_data = _sk_check_is_fitted = None

    class NotFittedError(ValueError, AttributeError):
        """An estimator used before fit (scikit-learn's class of the same name)."""


def _as_f64(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    if x.ndim != 2:
        raise ValueError(f"Expected 2D array, got {x.ndim}D array instead")
    return x


def _check_rows(est, X, reset):
    """The checks of scikit-learn's validate_data(est, X, reset=reset,
    dtype="float64") that the reference wrapper relies on, with the same
    messages, for machines without scikit-learn: dense, real, 2-D, at least
    one row and one feature, finite; reset records n_features_in_, otherwise
    the feature count must match it."""
    if hasattr(X, "toarray"):
        raise TypeError("Sparse data was passed, but dense data is required. Use '.toarray()' to convert to a "
                        "dense numpy array.")
    x = np.asarray(X)
    if x.dtype.kind == "c":
        raise ValueError("Complex data not supported")
    if x.ndim != 2:
        kind = "scalar" if x.ndim == 0 else f"{x.ndim}D"
        raise ValueError(f"Expected 2D array, got {kind} array instead")
    x = np.ascontiguousarray(x, dtype=np.float64)
    name = type(est).__name__
    if x.shape[0] < 1:
        raise ValueError(f"Found array with 0 sample(s) (shape={x.shape}) while a minimum of 1 is required by "
                         f"{name}.")
    if x.shape[1] < 1:
        raise ValueError(f"Found array with 0 feature(s) (shape={x.shape}) while a minimum of 1 is required by "
                         f"{name}.")
    if not np.isfinite(x).all():
        raise ValueError("Input X contains NaN." if np.isnan(x).any() else "Input X contains infinity.")
    if reset:
        est.n_features_in_ = x.shape[1]
    elif x.shape[1] != est.n_features_in_:
        raise ValueError(f"X has {x.shape[1]} features, but {name} is expecting {est.n_features_in_} features as "
                         "input.")
    return x


def _validate(est, X, reset):
    """validate_data(est, X, reset=reset, dtype="float64"), as the reference
    wrapper calls it in fit, predict and transform (_clusterers.py:44, 58, 66)."""
    if _sk_validate_data is not None:
        return np.ascontiguousarray(_sk_validate_data(est, X, reset=reset, dtype="float64"))
    return _check_rows(est, X, reset)


def _check_fitted(est):
    if _sk_check_is_fitted is not None:
        _sk_check_is_fitted(est)
    elif not hasattr(est, "cluster_centers_"):
        raise NotFittedError(f"This {type(est).__name__} instance is not fitted yet. Call 'fit' with appropriate "
                             "arguments before using this estimator.")


# The GPU work of the wrapper, in three functions of the module.
def _fit(x, est):
    """Fit::fit on the GPU -> (centres, labels, inertia, n_iter)."""
    dtype = "f64" if est._plain() else "f32x64"
    m = _KMeans(est.n_clusters, dtype=dtype).with_max_iter(est.max_iter).with_tol(est.tol) \
        .with_n_init(est.n_init).with_precision(est.precision)
    if est.random_state is not None:
        m = m.with_random_state(est.random_state)
    f = m.fit(x, ctx=default_context(est.device))
    return np.array(f.cluster_centers()), np.asarray(f.labels()), float(f.inertia()), int(f.n_iter())


def _predict(centres, x, est):
    """Predict::predict on the GPU with the fitted centres (the fit's precision)."""
    dtype = "f64" if est._plain() else "f32x64"
    f = FittedKMeans(centres, None, 0.0, 0, dtype, precision=_prec(est.precision))
    return np.asarray(f.predict(x, ctx=default_context(est.device)))


def _transform(centres, x, est):
    """Transform::transform on the GPU (FP64 direct form)."""
    f = FittedKMeans(centres, None, 0.0, 0, "f64")
    return np.array(f.transform(x, ctx=default_context(est.device)))


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

    def _rows(self, x):
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
        x = _validate(self, X, reset=True)
        c, labels, inertia, n_iter = _fit(self._rows(x), self)
        self.cluster_centers_ = c
        self.labels_ = labels
        self.inertia_ = inertia
        self.n_iter_ = n_iter
        return self

    def predict(self, X):
        _check_fitted(self)
        x = _validate(self, X, reset=False)
        return _predict(self.cluster_centers_, self._rows(x), self)

    def transform(self, X):
        _check_fitted(self)
        x = _validate(self, X, reset=False)
        return _transform(self.cluster_centers_, x, self)

    def fit_predict(self, X, y=None):
        return self.fit(X).labels_

    def fit_transform(self, X, y=None):
        return self.fit(X).transform(X)


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

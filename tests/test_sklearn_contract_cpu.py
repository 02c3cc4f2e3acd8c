"""scikit-learn's estimator contract for the sklearn-style wrapper, as the
reference runs it on its own wrapper (ferrolearn-python/tests/
test_check_estimator.py:33: parametrize_with_checks on KMeans(n_clusters=3,
random_state=42, n_init=2)).

The contract tests what the wrapper itself does -- parameters, cloning,
input validation and its messages, fitted attributes, n_features_in_,
idempotent fits, pickling, pipelines. No machine of this build has both
scikit-learn and a GPU (the GPU machines have no scikit-learn), so here the
wrapper's three GPU calls (ferrolearn_gb300.sklearn._fit / _predict /
_transform) are replaced, for this test only, by the oracle's restatement of
the same Fit / Predict / Transform. The GPU results themselves are compared
with the oracle in tests/test_sklearn_wrapper.py."""
import numpy as np
import pytest

import ferrolearn_gb300.sklearn as S
from oracle import oracle as O

try:  # a module-level skip would count as a skipped test in every selection
    from sklearn.utils.estimator_checks import parametrize_with_checks
except ImportError:
    parametrize_with_checks = None


def _oracle_fit(x, est):
    o = O.fit(np.ascontiguousarray(x, dtype=np.float64), est.n_clusters, max_iter=est.max_iter, tol=est.tol,
              n_init=est.n_init, seed=est.random_state or 0)
    return o["centers"], o["labels"], float(o["inertia"]), int(o["n_iter"])


def _oracle_predict(centres, x, est):
    return O.predict(centres, np.ascontiguousarray(x, dtype=np.float64))


def _oracle_transform(centres, x, est):
    return O.transform(centres, np.ascontiguousarray(x, dtype=np.float64))


@pytest.fixture(autouse=True)
def _oracle_in_place_of_the_gpu(monkeypatch):
    monkeypatch.setattr(S, "_fit", _oracle_fit)
    monkeypatch.setattr(S, "_predict", _oracle_predict)
    monkeypatch.setattr(S, "_transform", _oracle_transform)


if parametrize_with_checks is not None:
    @parametrize_with_checks([S.KMeans(n_clusters=3, random_state=42, n_init=2)])
    def test_estimator_contract(estimator, check):
        check(estimator)
else:
    def test_estimator_contract():
        pytest.skip("scikit-learn is not installed")

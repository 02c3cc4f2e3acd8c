"""BisectingKMeans on the GPU against the oracle's restatement of
bisecting_kmeans.rs, both drawing the library's uniform stream: the same
picks per run and split, so centres, labels, the cluster count and the
inertia (folded in the reference's order) must be identical."""
import numpy as np
import pytest

import ferrolearn_gb300 as F
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _blobs(n, d, k, seed, dtype):
    rng = np.random.default_rng(seed)
    cen = rng.uniform(-10, 10, size=(k, d))
    x = cen[rng.integers(0, k, n)] + rng.normal(0, 1.5, size=(n, d))
    return np.ascontiguousarray(x, dtype=dtype)


def _compare(g, o):
    assert g.n_clusters() == o["n_clusters"]
    assert np.array_equal(g.labels(), o["labels"])
    assert np.array_equal(g.cluster_centers(), o["centers"])
    assert g.inertia() == o["inertia"]


@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("strategy", ["largest_cluster", "largest_sse"])
@pytest.mark.parametrize("n,d,k,n_init", [(3000, 8, 6, 3), (20000, 32, 12, 10), (777, 3, 9, 1)])
def test_bisecting_fit_matches_oracle(dtype, strategy, n, d, k, n_init):
    npdt = np.float64 if dtype == "f64" else np.float32
    x = _blobs(n, d, k, seed=n + d + k, dtype=npdt)
    g = F.BisectingKMeans(k, dtype=dtype).with_n_init(n_init).with_random_state(5) \
        .with_bisecting_strategy(strategy).fit(x)
    o = O.bisecting_fit(x, k, n_init=n_init, seed=5, strategy=strategy)
    _compare(g, o)


def test_bisecting_reference_unit_cases_on_gpu():
    blobs = np.array([0.0, 0.0, 0.1, 0.1, -0.1, 0.1, 10.0, 10.0, 10.1, 10.1, 9.9, 10.1,
                      0.0, 10.0, 0.1, 10.1, -0.1, 9.9]).reshape(9, 2)
    g = F.BisectingKMeans(3).with_random_state(42).fit(blobs)
    _compare(g, O.bisecting_fit(blobs, 3, seed=42))
    assert np.array_equal(g.predict(blobs), g.labels())
    assert np.array_equal(g.transform(blobs), O.transform(g.cluster_centers(), blobs))
    one = F.BisectingKMeans(1).with_random_state(42).fit(np.array([[5.0, 5.0]]))
    assert list(one.labels()) == [0] and one.n_clusters() == 1
    x = np.array([[0.0, 0.0], [5.0, 5.0], [10.0, 10.0]])
    _compare(F.BisectingKMeans(3).with_random_state(42).fit(x), O.bisecting_fit(x, 3, seed=42))


def test_bisecting_unseparable_cluster_is_reported():
    with pytest.raises(F.NumericalInstability):
        F.BisectingKMeans(2).with_n_init(1).with_random_state(1).fit(np.ones((4, 2)))

"""The sklearn-style wrapper (ferrolearn_gb300.sklearn.KMeans), the drop-in for
ferrolearn-python's KMeans (_clusterers.py:15-84): constructor keywords and
defaults, parameter handling, validation on the CPU; fit / predict /
transform / pickling against the library's own API on the GPU."""
import pickle

import numpy as np
import pytest

import ferrolearn_gb300 as F
from ferrolearn_gb300.sklearn import KMeans
from oracle import oracle as O


def test_defaults_match_the_reference_wrapper():
    km = KMeans()
    assert (km.n_clusters, km.max_iter, km.tol, km.n_init, km.random_state) == (8, 300, 1e-4, 10, None)


def test_sklearn_parameter_protocol():
    pytest.importorskip("sklearn")
    from sklearn.base import clone
    km = KMeans(n_clusters=3, random_state=7, precision="bf16")
    p = km.get_params()
    assert p["n_clusters"] == 3 and p["random_state"] == 7 and p["precision"] == "bf16"
    c = clone(km).set_params(n_init=2)
    assert c.n_init == 2 and c.n_clusters == 3


def test_validation_errors_before_any_device_work():
    x = np.ones((5, 2))
    with pytest.raises(F.InvalidParameter):
        KMeans(n_clusters=0).fit(x)
    with pytest.raises(F.InsufficientSamples):
        KMeans(n_clusters=9).fit(x)
    with pytest.raises(ValueError):
        KMeans().fit(np.ones(5))
    with pytest.raises(AttributeError):
        KMeans().predict(x)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["plain", "bf16"])
def test_wrapper_fit_predict_transform_on_gpu(precision):
    # against the FP64 oracle (the same k-means++ stream: run r seeded with
    # random_state + r); bf16 reads X as f32, so X is made f32-exact first
    rng = np.random.default_rng(4)
    cen = rng.uniform(-10, 10, size=(5, 6))
    x = cen[rng.integers(0, 5, 1500)] + rng.normal(0, 1, size=(1500, 6))
    if precision != "plain":
        x = x.astype(np.float32).astype(np.float64)
    km = KMeans(n_clusters=5, n_init=3, random_state=11, precision=precision).fit(x)
    o = O.fit(x, 5, n_init=3, seed=11)
    assert np.array_equal(km.labels_, o["labels"])
    assert np.allclose(km.cluster_centers_, o["centers"], rtol=1e-13, atol=0)
    assert km.n_iter_ == o["n_iter"]
    assert abs(km.inertia_ - o["inertia"]) <= 1e-6 * o["inertia"]
    assert np.array_equal(km.predict(x), O.predict(km.cluster_centers_, x))
    assert np.allclose(km.transform(x[:20]), O.transform(km.cluster_centers_, x[:20]), rtol=1e-12, atol=1e-12)
    assert np.array_equal(km.fit_predict(x), km.labels_)
    km2 = pickle.loads(pickle.dumps(km))
    assert np.array_equal(km2.predict(x), km.predict(x))
    # predict / transform validate like the reference wrapper (validate_data(reset=False))
    with pytest.raises(ValueError, match="features"):
        km.predict(x[:, :4])
    with pytest.raises(ValueError):
        km.transform(np.full((2, 6), np.nan))


@pytest.mark.gpu
def test_fit_predict_is_fit_then_predict_on_gpu():
    # kmeans.rs:522-525: fit, then predict the same rows with the final
    # centres; labels() is the assignment before the last update, so the two
    # can differ when the run stops at max_iter
    rng = np.random.default_rng(9)
    x = rng.normal(size=(4000, 5)) * 3 + rng.integers(0, 7, size=(4000, 1))
    km = F.KMeans(7).with_max_iter(2).with_tol(0.0).with_n_init(2).with_random_state(3)
    got = km.fit_predict(x)
    o = O.fit(x, 7, max_iter=2, tol=0.0, n_init=2, seed=3)
    assert np.array_equal(got, O.predict(o["centers"], x))
    assert not np.array_equal(got, o["labels"])  # the case where they differ



def test_tensor_core_forms_read_float32_rows():
    # exact float32 rows pass silently; rounded ones warn before any device work
    km = KMeans(n_clusters=2, precision="bf16")
    exact = np.array([[0.5, 1.0], [2.0, -3.25]])
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        assert km._rows(exact).dtype == np.float32
    with pytest.warns(UserWarning, match="float32"):
        km._rows(np.array([[0.1, 1.0], [2.0, 3.0]]))
    assert KMeans(n_clusters=2)._rows(np.array([[0.1, 1.0]])).dtype == np.float64
    assert KMeans(n_clusters=2, precision=0)._plain()


def test_tensor_core_forms_need_float32_storage():
    # the library's f64 entry points refuse the mixed forms
    for prec in ("bf16", "fp8"):
        with pytest.raises(F.Unsupported, match="f32x64"):
            F.KMeans(2, dtype="f64").with_precision(prec).fit(np.ones((4, 2)))


def test_minibatch_wrapper_defaults_and_validation():
    from ferrolearn_gb300.sklearn import MiniBatchKMeans
    km = MiniBatchKMeans()
    # ferrolearn-python/python/ferrolearn/_extras.py:408-417
    assert (km.n_clusters, km.max_iter, km.random_state) == (8, 100, None)
    with pytest.raises(F.InvalidParameter):
        MiniBatchKMeans(n_clusters=0).fit(np.ones((5, 2)))
    with pytest.raises(F.InsufficientSamples):
        MiniBatchKMeans(n_clusters=9).fit(np.ones((5, 2)))
    with pytest.raises(AttributeError):
        MiniBatchKMeans().predict(np.ones((5, 2)))
    pytest.importorskip("sklearn")
    from sklearn.base import clone
    c = clone(MiniBatchKMeans(n_clusters=3, random_state=4)).set_params(max_iter=7)
    assert (c.n_clusters, c.random_state, c.max_iter) == (3, 4, 7)


def test_pickled_wrapper_keeps_what_predict_needs():
    # host-side state only: a fitted wrapper survives pickling with its centres,
    # labels and the precision its predict uses
    km = KMeans(n_clusters=2, precision="bf16")
    km.cluster_centers_ = np.array([[0.0, 1.0], [2.0, 3.0]])
    km.labels_ = np.array([0, 1, 1])
    km.inertia_, km.n_iter_, km.n_features_in_ = 1.5, 4, 2
    km._fitted = F.FittedKMeans(km.cluster_centers_.copy(), km.labels_.copy(), 1.5, 4, "f32x64", precision=F.MIXED_BF16)
    km2 = pickle.loads(pickle.dumps(km))
    assert np.array_equal(km2._fitted.cluster_centers(), km.cluster_centers_)
    assert km2._fitted.dtype == "f32x64" and km2._fitted.precision == F.MIXED_BF16
    assert (km2.inertia_, km2.n_iter_, km2.precision) == (1.5, 4, "bf16")
    assert np.array_equal(km2._fitted.labels(), km.labels_)

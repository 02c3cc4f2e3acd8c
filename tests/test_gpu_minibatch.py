"""MiniBatchKMeans on the GPU against the oracle's restatement of
mini_batch_kmeans.rs, both drawing the library's uniform stream: per run the
same initial centres and batches, so labels, centres and n_iter must be
identical and the inertia equal to the last bits of its summation order."""
import numpy as np
import pytest

import ferrolearn_gb300 as F
from oracle import oracle as O

pytestmark = pytest.mark.gpu

INERTIA_RTOL = {"f64": 1e-12, "f32": 1e-5}


def _blobs(n, d, k, seed, dtype):
    rng = np.random.default_rng(seed)
    cen = rng.uniform(-10, 10, size=(k, d))
    x = cen[rng.integers(0, k, n)] + rng.normal(0, 1.5, size=(n, d))
    return np.ascontiguousarray(x, dtype=dtype)


def _compare(g, o, dtype):
    assert np.array_equal(g.labels(), o["labels"])
    assert np.array_equal(g.cluster_centers(), o["centers"])
    assert g.n_iter() == o["n_iter"]
    assert g.report["best_run"] == o["best_run"]
    assert abs(g.inertia() - o["inertia"]) <= INERTIA_RTOL[dtype] * abs(o["inertia"])


@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("init", ["kmeans++", "random"])
@pytest.mark.parametrize("n,d,k,batch", [(5000, 16, 12, 256), (3001, 7, 40, 1024), (20000, 64, 100, 2048)])
def test_minibatch_fit_matches_oracle(dtype, init, n, d, k, batch):
    npdt = np.float64 if dtype == "f64" else np.float32
    x = _blobs(n, d, k, seed=n + d + k, dtype=npdt)
    g = F.MiniBatchKMeans(k, dtype=dtype).with_batch_size(batch).with_max_iter(25).with_n_init(3) \
        .with_random_state(11).with_init(init).fit(x)
    o = O.minibatch_fit(x, k, batch_size=batch, max_iter=25, n_init=3, seed=11, init=init)
    _compare(g, o, dtype)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_minibatch_explicit_init_full_batches_and_tolerance(dtype):
    npdt = np.float64 if dtype == "f64" else np.float32
    x = _blobs(900, 5, 6, seed=3, dtype=npdt)
    rng = np.random.default_rng(4)
    inits = np.stack([x[rng.choice(900, 6, replace=False)] for _ in range(2)])
    # batch_size >= n: every row each iteration, in a random order
    g = F.MiniBatchKMeans(6, dtype=dtype).with_batch_size(5000).with_max_iter(10).with_n_init(2) \
        .with_init_centers(inits).fit(x)
    o = O.minibatch_fit(x, 6, batch_size=5000, max_iter=10, n_init=2, init_centers=inits)
    _compare(g, o, dtype)
    # tol > 0: the runs stop at the first shift below it
    g = F.MiniBatchKMeans(6, dtype=dtype).with_batch_size(64).with_max_iter(400).with_tol(0.05) \
        .with_n_init(2).with_random_state(8).fit(x)
    o = O.minibatch_fit(x, 6, batch_size=64, max_iter=400, tol=0.05, n_init=2, seed=8)
    _compare(g, o, dtype)
    assert g.n_iter() < 400


def test_minibatch_reference_unit_cases_on_gpu():
    blobs = np.array([0.0, 0.0, 0.1, 0.1, -0.1, 0.1, 10.0, 10.0, 10.1, 10.1, 9.9, 10.1,
                      0.0, 10.0, 0.1, 10.1, -0.1, 9.9]).reshape(9, 2)
    g = F.MiniBatchKMeans(3).with_random_state(42).with_n_init(5).with_batch_size(9).fit(blobs)
    o = O.minibatch_fit(blobs, 3, batch_size=9, n_init=5, seed=42)
    _compare(g, o, "f64")
    new = np.array([[0.05, 0.05], [10.05, 10.05], [0.05, 10.05]])
    assert np.array_equal(g.predict(new), O.predict(g.cluster_centers(), new))
    assert np.array_equal(g.transform(blobs), O.transform(g.cluster_centers(), blobs))
    same = np.ones((4, 2))
    assert F.MiniBatchKMeans(1).with_random_state(42).with_batch_size(4).fit(same).inertia() == 0.0


def test_minibatch_device_resident_inputs_and_outputs():
    torch = pytest.importorskip("torch")
    x = _blobs(4000, 8, 10, seed=5, dtype=np.float64)
    m = F.MiniBatchKMeans(10).with_batch_size(500).with_max_iter(20).with_random_state(2)
    host = m.fit(x)
    c_out = torch.empty((10, 8), dtype=torch.float64, device="cuda")
    l_out = torch.empty(4000, dtype=torch.int64, device="cuda")
    m.fit(torch.from_numpy(x).cuda(), out=(c_out, l_out))
    assert np.array_equal(c_out.cpu().numpy(), host.cluster_centers())
    assert np.array_equal(l_out.cpu().numpy(), host.labels())


def test_minibatch_sklearn_wrapper():
    from ferrolearn_gb300.sklearn import MiniBatchKMeans
    x = _blobs(3000, 6, 5, seed=9, dtype=np.float64)
    km = MiniBatchKMeans(n_clusters=5, random_state=3).fit(x)
    o = O.minibatch_fit(x, 5, max_iter=100, n_init=3, seed=3)
    assert np.array_equal(km.labels_, o["labels"])
    assert np.array_equal(km.cluster_centers_, o["centers"])
    assert np.array_equal(km.predict(x), O.predict(km.cluster_centers_, x))
    assert np.array_equal(km.fit_predict(x), km.labels_)

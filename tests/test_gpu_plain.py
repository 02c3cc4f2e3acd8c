"""GPU parity of the plain (direct-form) path against the CPU oracle.

The plain path reproduces kmeans.rs's arithmetic exactly: direct-form
distances with no FMA, strict-< argmin with the lowest index on ties, and
row-order centroid sums. So labels, centres, shifts and n_iter must be
bit-identical to the oracle's for F = f64 and F = f32; only the inertia,
a sum whose order the reference itself leaves to Rayon, is compared with a
relative tolerance (1e-12 for f64, 1e-5 for f32).
"""
import numpy as np
import pytest

import ferrolearn_gb300 as F
from ferrolearn_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

INERTIA_RTOL = {"f64": 1e-12, "f32": 1e-5, "f32x64": 1e-12}


def _blobs(n, d, k, seed, spread=10.0, std=1.0, dtype=np.float64):
    rng = np.random.default_rng(seed)
    cen = rng.uniform(-spread, spread, size=(k, d))
    lab = rng.integers(0, k, size=n)
    x = cen[lab] + rng.normal(0, std, size=(n, d))
    return np.ascontiguousarray(x, dtype=dtype)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("n,d,k", [(1, 1, 1), (7, 3, 2), (200, 5, 3), (1000, 17, 9), (4096, 64, 70),
                                   (3000, 2, 300), (20000, 33, 40)])
def test_lloyd_steps_bit_identical(dtype, n, d, k):
    npdt = np.float64 if dtype == "f64" else np.float32
    x = _blobs(n, d, min(k, n), seed=n + d + k, dtype=npdt)
    rng = np.random.default_rng(1)
    c = x[rng.choice(n, size=k, replace=n < k)].copy()
    for _ in range(4):
        gl, gc, gi, gs, _ = F.lloyd_step(x, c, dtype=dtype)
        ol, oc, oi, os_ = O.lloyd_step(x, c)
        assert np.array_equal(gl, ol)
        assert np.array_equal(gc, oc)
        assert gs == os_
        assert abs(gi - oi) <= INERTIA_RTOL[dtype] * abs(oi) + 1e-300
        c = oc


def test_f32x64_matches_oracle_on_widened_rows():
    x32 = _blobs(5000, 24, 12, seed=3, dtype=np.float32)
    x64 = x32.astype(np.float64)
    c = x64[:12].copy()
    for _ in range(3):
        gl, gc, gi, gs, _ = F.lloyd_step(x32, c, dtype="f32x64")
        ol, oc, oi, os_ = O.lloyd_step(x64, c)
        assert np.array_equal(gl, ol) and np.array_equal(gc, oc) and gs == os_
        c = oc


def test_isotropic_8x16_full_fit():
    w = W.isotropic_8x16()
    x, k = w["x"], w["k"]
    g = F.KMeans(k).with_max_iter(w["max_iter"]).with_tol(w["tol"]).with_n_init(1) \
        .with_init_centers(w["init"]).fit(x)
    o = O.fit(x, k, max_iter=w["max_iter"], tol=w["tol"], n_init=1, init=w["init"][None])
    assert np.array_equal(g.labels(), o["labels"])
    assert np.array_equal(g.cluster_centers(), o["centers"])
    assert g.n_iter() == o["n_iter"]
    assert abs(g.inertia() - o["inertia"]) <= 1e-12 * o["inertia"]


def test_fit_n_init_best_run_and_kmeanspp():
    x = _blobs(3000, 6, 5, seed=11)
    g = F.KMeans(5).with_n_init(4).with_random_state(42).fit(x)
    o = O.fit(x, 5, n_init=4, seed=42)
    assert g.report["best_run"] == o["best_run"]
    assert np.array_equal(g.labels(), o["labels"])
    assert np.array_equal(g.cluster_centers(), o["centers"])
    assert g.n_iter() == o["n_iter"]


def _kpp_draws(seed, k):
    return F.draws(seed, 1 + (k - 1) * (2 + int(np.floor(np.log(k)))))


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_kmeanspp_matches_oracle(dtype):
    npdt = np.float64 if dtype == "f64" else np.float32
    for seed, (n, d, k) in enumerate([(50, 2, 3), (2000, 8, 16), (9000, 16, 40), (70001, 5, 30)]):
        x = _blobs(n, d, k, seed=seed, dtype=npdt)
        dr = _kpp_draws(seed + 100, k)
        gc, gu = F.kmeans_plus_plus(x, k, dr, dtype=dtype)
        oc, ou = O.kmeanspp(x, k, dr)
        assert gu == ou
        assert np.array_equal(gc, oc)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_kmeanspp_edge_cases_match_oracle(dtype):
    npdt = np.float64 if dtype == "f64" else np.float32
    rng = np.random.default_rng(7)
    cases = [
        np.ones((40, 3)),                                         # total 0 after the first centre: random rows
        np.repeat(rng.normal(size=(3, 4)), [500, 1, 2000], 0),    # fewer distinct rows than centres
        rng.integers(-3, 4, size=(30000, 2)).astype(np.float64),  # integer grid: many exact halves and ties
        np.array([[1.5, -2.0]]),                                  # one row
        np.concatenate([rng.normal(size=(5000, 3)) * 1e-20, rng.normal(size=(5000, 3)) * 1e15]),
    ]
    for i, x in enumerate(cases):
        x = np.ascontiguousarray(x, dtype=npdt)
        for k in sorted({1, 2, min(len(x), 9)}):
            dr = _kpp_draws(300 + 10 * i + k, k)
            gc, gu = F.kmeans_plus_plus(x, k, dr, dtype=dtype)
            oc, ou = O.kmeanspp(x, k, dr)
            assert gu == ou, (i, k)
            assert np.array_equal(gc, oc), (i, k)


@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_kmeanspp_at_full_dirichlet_size_matches_oracle(dtype):
    # n = 1,000,000 rows, d = 64, k = 256: every sum of kmeans.rs:201, 215-223
    # and 225-237 is a million-term left fold in F, so a fold in any other
    # order would pick other candidates here
    npdt = np.float64 if dtype == "f64" else np.float32
    w = W.dirichlet_256x64(scale=1.0, seed=3, dtype=npdt)
    x, k = w["x"], w["k"]
    dr = _kpp_draws(5, k)
    gc, gu = F.kmeans_plus_plus(x, k, dr, dtype=dtype)
    oc, ou = O.kmeanspp(x, k, dr)
    assert gu == ou
    assert np.array_equal(gc, oc)


def test_reference_unit_cases_on_gpu():
    x = np.array([[0.0, 0.0], [0.1, 0.1], [-0.1, 0.1], [10.0, 10.0], [10.1, 10.1], [9.9, 10.1],
                  [0.0, 10.0], [0.1, 10.1], [-0.1, 9.9]])
    f = F.KMeans(3).with_random_state(42).with_n_init(5).fit(x)
    lab = f.labels()
    assert lab[0] == lab[1] == lab[2] and lab[3] == lab[4] == lab[5] and lab[6] == lab[7] == lab[8]
    assert len({lab[0], lab[3], lab[6]}) == 3
    new = np.array([[0.05, 0.05], [10.05, 10.05], [0.05, 10.05]])  # kmeans.rs:713-733
    p = f.predict(new)
    assert p[0] == lab[0] and p[1] == lab[3] and p[2] == lab[6]
    f1 = F.KMeans(1).with_random_state(42).fit(np.array([[1.0, 1.0], [2, 2], [3, 3], [4, 4]]))
    assert np.allclose(f1.cluster_centers()[0], [2.5, 2.5], atol=1e-10)
    assert F.KMeans(1).fit(np.ones((4, 2))).inertia() == 0.0
    fk = F.KMeans(3).with_random_state(42).fit(np.array([[0.0, 0.0], [5, 5], [10, 10]]))
    assert fk.inertia() == 0.0 and len(set(fk.labels())) == 3
    with pytest.raises(F.ShapeMismatch):
        f.predict(np.ones((2, 3)))


def test_transform_and_predict_parity():
    x = _blobs(3000, 10, 7, seed=5)
    c = x[:7].copy()
    fitted = F.FittedKMeans(c, np.zeros(len(x), dtype=np.int64), 0.0, 0, "f64")
    assert np.array_equal(fitted.transform(x), O.transform(c, x))
    assert np.array_equal(fitted.predict(x), O.predict(c, x))
    x32 = x.astype(np.float32)
    f32 = F.FittedKMeans(c.astype(np.float32), np.zeros(len(x), dtype=np.int64), 0.0, 0, "f32")
    assert np.array_equal(f32.transform(x32), O.transform(c.astype(np.float32), x32))


def test_ties_nan_and_empty_clusters():
    # duplicate centres -> lowest index; a centre far away stays empty and keeps its value
    x = np.array([[0.0, 0.0], [1.0, 1.0], [2.0, 2.0], [np.nan, 1.0]])
    c = np.array([[1.0, 1.0], [1.0, 1.0], [500.0, 500.0]])
    gl, gc, gi, gs, _ = F.lloyd_step(x, c)
    ol, oc, oi, os_ = O.lloyd_step(x, c)
    assert np.array_equal(gl, ol) and gl.tolist() == [0, 0, 0, 0]
    assert np.array_equal(gc, oc, equal_nan=True)
    assert gi == oi == np.finfo(np.float64).max
    assert (gs == os_) or (np.isnan(gs) and np.isnan(os_))


def test_max_iter_zero_reports_max_inertia():
    x = _blobs(100, 3, 4, seed=2)
    g = F.KMeans(4).with_max_iter(0).with_n_init(1).with_init_centers(x[:4]).fit(x)
    assert g.n_iter() == 0 and g.inertia() == np.finfo(np.float64).max
    assert (g.labels() == 0).all() and np.array_equal(g.cluster_centers(), x[:4])


def test_device_resident_inputs():
    torch = pytest.importorskip("torch")
    x = _blobs(5000, 16, 8, seed=9)
    c = x[:8].copy()
    xd = torch.from_numpy(x).cuda()
    gl, gc, _, _, _ = F.lloyd_step(xd, c)
    ol, oc, _, _ = O.lloyd_step(x, c)
    assert np.array_equal(gl, ol) and np.array_equal(gc, oc)


def test_dirichlet_scale_sampled_rows():
    # Full-size-shaped data at 1/10 scale; the oracle checks a seeded sample of
    # rows exactly (assignment is independent per row) and the update in f64.
    w = W.dirichlet_256x64(scale=0.1)
    x, k = w["x"], w["k"]
    rng = np.random.default_rng(0)
    c = x[rng.choice(len(x), k, replace=False)].copy()
    gl, gc, gi, gs, _ = F.lloyd_step(x, c)
    idx = rng.choice(len(x), 5000, replace=False)
    ol, _ = O.assign(x[idx], c)
    assert np.array_equal(gl[idx], ol)
    # update: row-order sums equal the oracle's own update on the GPU labels
    oc = np.empty_like(c)
    for q in range(k):
        rows = x[gl == q]
        oc[q] = rows.sum(0) / len(rows) if len(rows) else c[q]
    assert np.abs(gc - oc).max() <= 1e-12 * np.abs(oc).max()


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_fit_with_injected_draws_matches_oracle(dtype):
    # one caller-supplied uniform stream shared by the n_init runs' k-means++
    # (each run continues where the previous one stopped)
    npdt = np.float64 if dtype == "f64" else np.float32
    x = _blobs(2500, 5, 7, seed=21, dtype=npdt)
    k, n_init = 7, 3
    dr = F.draws(99, n_init * (1 + (k - 1) * (2 + int(np.floor(np.log(k))))))
    g = F.KMeans(k, dtype=dtype).with_n_init(n_init).with_draws(dr).fit(x)
    o = O.fit(x, k, n_init=n_init, draws_arr=dr)
    assert g.report["best_run"] == o["best_run"]
    assert np.array_equal(g.labels(), o["labels"])
    assert np.array_equal(g.cluster_centers(), o["centers"])
    assert g.n_iter() == o["n_iter"]

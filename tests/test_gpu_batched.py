"""GPU parity of the batched KMeans<f32> fits (fk_kmeans_fit_batched_f32).

Every (problem, run) is checked against the oracle's own fit of that run
(oracle.fit_runs: Fit::fit, kmeans.rs:417-512, with F = f32 and run r
seeded with random_state + r): n_iter equal, the inertia within a relative
tolerance (the reference leaves its summation order to Rayon), and for the
best run the labels and centres bit-identical. The reference reduction is
the reference's own f32 arithmetic; the f64 reduction is checked against
the oracle's f64-sum variant. k-means++ is checked directly through
max_iter = 0 fits, whose centres are the initial ones.
"""
import numpy as np
import pytest

import ferrolearn_gb300 as F
from ferrolearn_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _problems(seed, shapes, n_init=3, max_iter=60, tol=1e-4):
    rng = np.random.default_rng(seed)
    probs = []
    for i, (n, d, k) in enumerate(shapes):
        cen = rng.uniform(-10, 10, size=(k, d)).astype(np.float32)
        x = cen[rng.integers(0, k, size=n)] + rng.standard_normal(size=(n, d), dtype=np.float32)
        probs.append(dict(x=np.ascontiguousarray(x), k=k, n_init=n_init, max_iter=max_iter, tol=tol,
                          random_state=1000 * seed + i))
    return probs


SHAPES = [(1500, 8, 5), (900, 16, 30), (2500, 32, 12), (700, 64, 40), (1200, 5, 7), (600, 64, 64),
          (3000, 16, 70), (400, 8, 4), (2000, 32, 33)]


def _check_against_oracle(probs, fitted, rep, wide):
    f0 = 0
    for p, g in zip(probs, fitted):
        o = O.fit_runs(p["x"], p["k"], max_iter=p["max_iter"], tol=p["tol"], n_init=p["n_init"],
                       seed=p["random_state"], wide_sums=wide)
        runs = p["n_init"]
        assert np.array_equal(rep["fit_n_iter"][f0:f0 + runs], o["n_iter"])
        rtol = 1e-12 if wide else 1e-5
        assert np.allclose(rep["fit_inertia"][f0:f0 + runs], o["inertia"], rtol=rtol, atol=0)
        b = g.report["best_run"]
        # best run: strictly lowest inertia, first on ties (within the inertia tolerance)
        ob = int(np.argmin(o["inertia"]))
        assert b == ob or abs(o["inertia"][b] - o["inertia"][ob]) <= rtol * o["inertia"][ob]
        assert np.array_equal(g.labels(), o["labels"][b])
        assert np.array_equal(g.cluster_centers(), o["centers"][b])
        assert g.n_iter() == o["n_iter"][b]
        f0 += runs


@pytest.mark.parametrize("reduction", ["reference", "f64"])
def test_batched_fits_match_oracle_per_run(reduction):
    probs = _problems(3, SHAPES)
    fitted, rep = F.fit_batched(probs, reduction=reduction)
    assert rep["fits"] == sum(p["n_init"] for p in probs)
    assert rep["iterations_total"] == int(rep["fit_n_iter"].sum())
    assert rep["graph_launches"] >= int(rep["fit_n_iter"].max())
    assert len(rep["tiles"]) >= 5
    _check_against_oracle(probs, fitted, rep, wide=reduction == "f64")


def test_batched_kmeanspp_matches_oracle():
    probs = _problems(5, SHAPES, n_init=2, max_iter=0)
    fitted, rep = F.fit_batched(probs)
    for p, g in zip(probs, fitted):
        c, _ = O.kmeanspp(p["x"], p["k"], seed=p["random_state"])  # run 0 is the best (all FLT_MAX)
        assert np.array_equal(g.cluster_centers(), c)
        assert g.n_iter() == 0 and g.inertia() == np.finfo(np.float32).max
        assert not g.labels().any()


def test_batched_injected_init_and_reference_unit_cases():
    rng = np.random.default_rng(9)
    x1 = rng.normal(size=(50, 3)).astype(np.float32)
    same = np.ones((20, 4), dtype=np.float32)
    probs = [
        dict(x=x1, k=50, n_init=1, init=x1[None].copy()),           # k = n: inertia 0 (kmeans.rs:784-798)
        dict(x=same, k=3, n_init=2),                                 # identical points: inertia 0
        dict(x=x1[:1].copy(), k=1, n_init=1),                        # n = 1: label 0
        dict(x=x1, k=4, n_init=3, init=x1[rng.choice(50, size=(3, 4))], max_iter=7, tol=0.0),
    ]
    fitted, rep = F.fit_batched(probs)
    assert fitted[0].inertia() == 0.0
    assert fitted[1].inertia() == 0.0
    assert fitted[2].labels().tolist() == [0]
    o = O.fit_runs(x1, 4, max_iter=7, tol=0.0, n_init=3, init=probs[3]["init"])
    b = fitted[3].report["best_run"]
    assert np.array_equal(fitted[3].labels(), o["labels"][b])
    assert np.array_equal(fitted[3].cluster_centers(), o["centers"][b])
    assert fitted[3].n_iter() == 7


def test_batched_workload_sample_and_device_inputs():
    torch = pytest.importorskip("torch")
    probs = W.batched_512(scale=0.02, n_problems=24, n_init=2, max_iter=40)
    for p in probs[::3]:
        p["x"] = torch.from_numpy(p["x"]).cuda()  # device-resident rows
    fitted, rep = F.fit_batched(probs)
    host = [dict(p, x=p["x"].cpu().numpy() if hasattr(p["x"], "cpu") else p["x"]) for p in probs]
    _check_against_oracle(host, fitted, rep, wide=False)
    # a second call reuses the tuned tile shapes
    _, rep2 = F.fit_batched(probs[:4])
    assert rep2["tuned_buckets"] == 0

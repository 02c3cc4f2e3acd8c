"""Pins the CPU oracle against the reference's golden data and known answers.

The oracle (oracle/kmeans_oracle.c) is what every GPU parity test compares against,
so it is validated first against:
  * the reference's KMeans fixture (fixtures/kmeans.json, used by
    ferrolearn-cluster/tests/oracle_tests.rs:66-117), both exactly (starting
    from the fixture's converged centres) and with the reference's own loose
    criteria (k-means++ start);
  * the reference's statistical-equivalence fixture
    (sklearn_equivalence.rs:34-117);
  * scikit-learn Lloyd trajectories from explicit initial centres;
  * the known answers of the reference's unit tests (kmeans.rs:620-927) and
    its property invariants (proptest_invariants.rs:37-129).
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def _pairwise_agreement(a, b):
    # oracle_tests.rs: pairs (i, j), j in i+1..min(i+10, n): same-cluster relation agrees
    n = len(a)
    agree = total = 0
    for i in range(n):
        for j in range(i + 1, min(i + 10, n)):
            total += 1
            agree += (a[i] == a[j]) == (b[i] == b[j])
    return agree / total


def _min_centroid_dist(target, centers):
    return np.sqrt(((centers - target) ** 2).sum(1)).min()


def test_reference_fixture_exact_from_converged_centres():
    g = _load("ref_kmeans_blobs150.json")
    x = np.array(g["X"])
    c = np.array(g["cluster_centers"])
    r = O.fit(x, 3, n_init=1, init=c[None])
    assert r["n_iter"] == 1
    assert np.array_equal(r["labels"], np.array(g["labels"]))
    assert abs(r["inertia"] - g["inertia"]) <= 1e-12 * g["inertia"]
    assert np.abs(r["centers"] - c).max() <= 1e-12 * np.abs(c).max()


def test_reference_fixture_oracle_criteria():
    g = _load("ref_kmeans_blobs150.json")
    x = np.array(g["X"])
    r = O.fit(x, 3, n_init=10, seed=42)
    ratio = r["inertia"] / g["inertia"]
    assert 0.95 <= ratio < 1.05
    for row in np.array(g["cluster_centers"]):
        assert _min_centroid_dist(row, r["centers"]) < 0.5
    assert _pairwise_agreement(r["labels"], g["labels"]) >= 0.99


def test_reference_sklearn_equivalence_fixture():
    g = _load("ref_sklearn_kmeans50.json")
    x = np.array(g["X"])
    r = O.fit(x, 3, n_init=10, seed=42)
    ratio = r["inertia"] / g["inertia"]
    assert 0.5 <= ratio < 2.0
    for row in np.array(g["cluster_centers"]):
        assert _min_centroid_dist(row, r["centers"]) < 3.0
    assert _pairwise_agreement(r["labels"], g["labels"]) >= 0.90
    # From sklearn's converged centres the oracle reproduces its labels exactly.
    r2 = O.fit(x, 3, n_init=1, init=np.array(g["cluster_centers"])[None])
    assert np.array_equal(r2["labels"], np.array(g["labels"]))
    assert abs(r2["inertia"] - g["inertia"]) <= 1e-12 * g["inertia"]


def test_sklearn_lloyd_trajectories():
    g = _load("sklearn_lloyd_steps.json")
    for case in g["cases"]:
        x = np.array(case["X"])
        c = np.array(case["init"])
        for step in case["steps"]:
            _, c, _, _ = O.lloyd_step(x, c)
            ref = np.array(step["centers"])
            assert np.abs(c - ref).max() <= 1e-12 * np.abs(ref).max()
            lab, _ = O.assign(x, c)
            assert np.array_equal(lab, np.array(step["labels"]))


BLOBS9 = np.array([[0.0, 0.0], [0.1, 0.1], [-0.1, 0.1], [10.0, 10.0], [10.1, 10.1], [9.9, 10.1],
                   [0.0, 10.0], [0.1, 10.1], [-0.1, 9.9]])


def test_unit_well_separated_blobs():  # kmeans.rs:640-659
    lab = O.fit(BLOBS9, 3, n_init=5, seed=42)["labels"]
    assert lab[0] == lab[1] == lab[2] and lab[3] == lab[4] == lab[5] and lab[6] == lab[7] == lab[8]
    assert len({lab[0], lab[3], lab[6]}) == 3


def test_unit_convergence_and_n_init():  # kmeans.rs:660-686
    assert O.fit(BLOBS9, 3, max_iter=1000, n_init=1, seed=42)["n_iter"] < 100
    r1 = O.fit(BLOBS9, 3, n_init=1, seed=42)
    r10 = O.fit(BLOBS9, 3, n_init=10, seed=42)
    assert r10["inertia"] <= r1["inertia"] + 1e-10


def test_unit_known_answers():
    x = np.array([[0.0, 0.0], [5.0, 5.0], [10.0, 10.0]])  # k = n (kmeans.rs:784-798)
    r = O.fit(x, 3, seed=42)
    assert abs(r["inertia"]) <= 1e-10 and len(set(r["labels"])) == 3
    x = np.array([[1.0, 1.0], [2.0, 2.0], [3.0, 3.0], [4.0, 4.0]])  # k = 1 (kmeans.rs:801-817)
    r = O.fit(x, 1, seed=42)
    assert (r["labels"] == 0).all() and np.allclose(r["centers"][0], [2.5, 2.5], atol=1e-10)
    r = O.fit(np.array([[5.0, 5.0]]), 1, seed=42)  # n = 1 (kmeans.rs:820-828)
    assert r["labels"].tolist() == [0] and abs(r["inertia"]) <= 1e-10
    r = O.fit(np.ones((4, 2)), 1, seed=42)  # identical points (kmeans.rs:919-926)
    assert abs(r["inertia"]) <= 1e-10
    line = np.array([[0.0], [0.1], [-0.1], [100.0], [100.1], [99.9]])  # kmeans.rs:900-916
    lab = O.fit(line, 2, seed=42)["labels"]
    assert lab[0] == lab[1] == lab[2] and lab[3] == lab[4] == lab[5] and lab[0] != lab[3]


def test_unit_errors():  # kmeans.rs:831-879
    with pytest.raises(O.OracleError) as e:
        O.fit(np.array([[1.0, 1.0], [2.0, 2.0]]), 5)
    assert e.value.code == 2
    with pytest.raises(O.OracleError) as e:
        O.fit(np.ones((3, 2)), 0)
    assert e.value.code == 1
    with pytest.raises(O.OracleError) as e:
        O.fit(np.zeros((0, 2)), 3)
    assert e.value.code == 2
    c = np.ones((2, 2))
    with pytest.raises(O.OracleError) as e:
        O.predict(c, np.ones((2, 3)))
    assert e.value.code == 3
    with pytest.raises(O.OracleError):
        O.transform(c, np.ones((2, 3)))


def test_unit_f32_and_transform():  # kmeans.rs:736-763, 882-897
    x = np.array([[0, 0], [0.1, 0.1], [-0.1, 0.1], [10, 10], [10.1, 10.1], [9.9, 10.1]], dtype=np.float32)
    r = O.fit(x, 2, seed=42)
    assert r["labels"].shape == (6,)
    assert O.predict(r["centers"], x).shape == (6,)
    x4 = np.array([[0.0, 0.0], [10.0, 0.0], [0.0, 10.0], [10.0, 10.0]])
    r = O.fit(x4, 2, seed=42)
    dist = O.transform(r["centers"], x4)
    assert dist.shape == (4, 2)
    for i in range(4):
        own = r["labels"][i]
        assert dist[i, own] < dist[i, 1 - own]


def test_property_invariants():  # proptest_invariants.rs:37-129 (128 cases)
    rng = np.random.default_rng(7)
    for _ in range(128):
        k = int(rng.integers(2, 5))
        d = int(rng.integers(2, 4))
        n = int(rng.integers(k, k + 9))
        x = rng.uniform(-10, 10, size=(n, d))
        r = O.fit(x, k, n_init=2, max_iter=50, seed=42)
        assert (r["labels"] < k).all() and r["centers"].shape == (k, d) and r["inertia"] >= 0
        p = O.predict(r["centers"], x)
        assert p.shape == (n,) and (p < k).all()


def test_tie_rule_lowest_index():
    # Two identical centres: every row goes to the lower index (strict <).
    x = np.array([[0.0, 0.0], [1.0, 1.0], [2.0, 2.0]])
    c = np.array([[1.0, 1.0], [1.0, 1.0], [5.0, 5.0]])
    lab, _ = O.assign(x, c)
    assert (lab == 0).all()


def test_nan_rows_follow_strict_less():
    # NaN distances are never < F::MAX: label 0, and the inertia becomes MAX-dominated.
    x = np.array([[np.nan, 0.0], [1.0, 1.0]])
    c = np.array([[5.0, 5.0], [1.0, 1.0]])
    lab, inertia = O.assign(x, c)
    assert lab.tolist() == [0, 1]
    assert inertia == np.finfo(np.float64).max


def test_wide_sum_update_is_the_rounded_exact_mean():
    # the f64-reduction variant of the oracle (the batched entry point's
    # FK_REDUCE_F64): each centre is (f32)(round_f64(exact cluster sum) / count),
    # restated here with exact rational sums
    from fractions import Fraction
    rng = np.random.default_rng(44)
    n, d, k = 300, 3, 5
    x = (rng.normal(size=(n, d)) * rng.choice([1e-3, 1.0, 1e3], size=(n, 1))).astype(np.float32)
    init = x[rng.choice(n, k, replace=False)][None]
    o = O.fit_runs(x, k, max_iter=1, tol=0.0, n_init=1, init=init, wide_sums=True)
    lab = o["labels"][0]
    for c in range(k):
        rows = x[lab == c]
        for j in range(d):
            if len(rows) == 0:
                want = init[0, c, j]
            else:
                s = sum((Fraction(float(v)) for v in rows[:, j]), Fraction(0))
                want = np.float32(float(s) / len(rows))
            assert o["centers"][0, c, j] == want, (c, j)


def test_fit_runs_agrees_with_fit_per_run():
    # the per-run entry point and Fit::fit with one run give the same run
    rng = np.random.default_rng(45)
    x = (rng.normal(size=(400, 4)) + rng.integers(0, 3, size=(400, 1)) * 5).astype(np.float32)
    inits = np.stack([x[rng.choice(400, 3, replace=False)] for _ in range(2)])
    runs = O.fit_runs(x, 3, max_iter=20, tol=1e-4, n_init=2, init=inits)
    for r in range(2):
        one = O.fit(x, 3, max_iter=20, tol=1e-4, n_init=1, init=inits[r][None])
        assert np.array_equal(runs["labels"][r], one["labels"])
        assert np.array_equal(runs["centers"][r], one["centers"])
        assert runs["n_iter"][r] == one["n_iter"]


def test_update_given_labels_is_the_reference_update():
    # the full-size parity checks' update: recompute_centroids_into on f32
    # rows widened to f64, threads split by feature -- the same centres as the
    # oracle's own Lloyd step, bit for bit, and its inertia folded in row order
    rng = np.random.default_rng(11)
    x = (rng.normal(size=(40000, 9)) * 3).astype(np.float32)
    c = x[rng.choice(40000, 12, replace=False)].astype(np.float64)
    c[3] = 1e6  # an empty cluster keeps its centre
    lab, nc, _, _ = O.lloyd_step(x.astype(np.float64), c)
    nc2, inertia = O.update_given_labels(x, lab, c)
    assert np.array_equal(nc, nc2)
    d = ((x.astype(np.float64) - c[lab]) ** 2).sum(1)
    assert abs(inertia - d.sum()) <= 1e-12 * d.sum()


def test_update_split_into_row_ranges_is_the_single_loop():
    # the reference arm of the benchmark runs one Lloyd iteration as K row
    # ranges; the split update must equal the oracle's one-pass update
    rng = np.random.default_rng(12)
    x = rng.normal(size=(10007, 6)) * 5
    c = x[rng.choice(10007, 9, replace=False)].copy()
    c[4] = 1e9
    lab, nc, _, shift = O.lloyd_step(x, c)
    sums, counts = np.zeros((9, 6)), np.zeros(9)
    for lo in range(0, 10007, 777):
        O.update_rows(x[lo:lo + 777], lab[lo:lo + 777], sums, counts)
    nc2, shift2 = O.update_finish(sums, counts, c)
    assert np.array_equal(nc, nc2) and shift == shift2

"""BisectingKMeans oracle (test infrastructure for the next rows of the
path): the restatement of bisecting_kmeans.rs pinned against the reference's
own unit tests (bisecting_kmeans.rs:612-884, on the library's uniform stream
in place of StdRng) and against a literal Python restatement."""
import math

import numpy as np
import pytest

from oracle import oracle as O

BLOBS = np.array([0.0, 0.0, 0.1, 0.1, -0.1, 0.1, 10.0, 10.0, 10.1, 10.1, 9.9, 10.1,
                  0.0, 10.0, 0.1, 10.1, -0.1, 9.9]).reshape(9, 2)  # make_blobs, :612-622


def _grouped3(lab):
    return (lab[0] == lab[1] == lab[2] and lab[3] == lab[4] == lab[5] and lab[6] == lab[7] == lab[8]
            and len({lab[0], lab[3], lab[6]}) == 3)


def test_well_separated_blobs_predict_and_shapes():  # :626-644, :685-711, :724-739
    r = O.bisecting_fit(BLOBS, 3, seed=42)
    assert _grouped3(r["labels"]) and r["n_clusters"] == 3
    assert r["centers"].shape == (3, 2) and r["inertia"] >= 0.0
    assert np.array_equal(O.predict(r["centers"], BLOBS), r["labels"])
    new = np.array([[0.05, 0.05], [10.05, 10.05], [0.05, 10.05]])
    assert list(O.predict(r["centers"], new)) == [r["labels"][0], r["labels"][3], r["labels"][6]]


def test_two_clusters_single_cluster_largest_sse():  # :646-683, :741-758
    x = np.array([[0.0, 0.0], [0.5, 0.0], [0.0, 0.5], [0.5, 0.5], [10.0, 10.0], [10.5, 10.0], [10.0, 10.5],
                  [10.5, 10.5]])
    lab = O.bisecting_fit(x, 2, seed=42)["labels"]
    assert len(set(lab[:4])) == 1 and len(set(lab[4:])) == 1 and lab[0] != lab[4]
    x1 = np.array([[1.0, 1.0], [2.0, 2.0], [3.0, 3.0], [4.0, 4.0]])
    r = O.bisecting_fit(x1, 1, seed=42)
    assert (r["labels"] == 0).all() and r["n_clusters"] == 1
    r = O.bisecting_fit(BLOBS, 3, seed=42, strategy="largest_sse")
    assert r["n_clusters"] == 3 and _grouped3(r["labels"])


def test_reproducible_errors_and_edge_cases():  # :760-839
    a, b = O.bisecting_fit(BLOBS, 3, seed=123), O.bisecting_fit(BLOBS, 3, seed=123)
    assert np.array_equal(a["labels"], b["labels"])
    for x, k, kw, code in [(BLOBS, 0, {}, 1), (np.array([[1.0, 1.0], [2.0, 2.0]]), 5, {}, 2),
                           (np.zeros((0, 2)), 3, {}, 2), (BLOBS, 3, dict(n_init=0), 1)]:
        with pytest.raises(O.OracleError) as e:
            O.bisecting_fit(x, k, **kw)
        assert e.value.code == code
    r = O.bisecting_fit(np.array([[5.0, 5.0]]), 1, seed=42)
    assert list(r["labels"]) == [0] and r["n_clusters"] == 1
    r = O.bisecting_fit(BLOBS[:6].astype(np.float32), 2, seed=42)
    assert r["labels"].shape == (6,) and r["n_clusters"] == 2 and r["centers"].dtype == np.float32
    assert O.bisecting_fit(np.ones((4, 2)), 1, seed=42)["n_clusters"] == 1


def test_labels_in_range_n_init_and_k_equals_n():  # :841-884
    r = O.bisecting_fit(BLOBS, 3, seed=42)
    assert (r["labels"] >= 0).all() and (r["labels"] < r["n_clusters"]).all()
    one = O.bisecting_fit(BLOBS, 3, seed=42, n_init=1)
    ten = O.bisecting_fit(BLOBS, 3, seed=42, n_init=10)
    assert ten["inertia"] <= one["inertia"] + 1e-6
    x = np.array([[0.0, 0.0], [5.0, 5.0], [10.0, 10.0]])
    lab = O.bisecting_fit(x, 3, seed=42)["labels"]
    assert len(set(lab.tolist())) == 3


def test_a_split_that_never_separates_stops_instead_of_looping():
    # identical rows: every 2-means puts all rows on one side, the reference
    # would select the same cluster forever; the restatement reports it
    with pytest.raises(O.OracleError) as e:
        O.bisecting_fit(np.ones((4, 2)), 2, seed=1, n_init=1)
    assert e.value.code == 5


# A literal restatement in Python floats for small inputs.
def _stream(seed):
    st = [seed & (2**64 - 1)]
    M = 2**64 - 1

    def rng(n):
        st[0] = (st[0] + 0x9E3779B97F4A7C15) & M
        z = st[0]
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        z ^= z >> 31
        u = (z >> 11) * (1.0 / 9007199254740992.0)
        return min(max(int(math.floor(u * n)), 0), n - 1)
    return rng


def _sq(a, b):
    acc = 0.0
    for u, v in zip(a, b):
        t = u - v
        acc = acc + t * t
    return acc


def _two_means(x, idx, max_iter, rng):
    m = len(idx)
    i0 = rng(m)
    i1 = rng(m)
    if m > 1:
        while i1 == i0:
            i1 = rng(m)
    c0, c1 = list(x[idx[i0]]), list(x[idx[i1]])
    lab = [0] * m
    for _ in range(max_iter):
        changed = False
        for li, r in enumerate(idx):
            nl = 0 if _sq(x[r], c0) <= _sq(x[r], c1) else 1
            if nl != lab[li]:
                lab[li], changed = nl, True
        if not changed:
            break
        s0, s1, n0, n1 = [0.0] * len(c0), [0.0] * len(c0), 0.0, 0.0
        for li, r in enumerate(idx):
            if lab[li] == 0:
                n0 = n0 + 1.0
                s0 = [a + b for a, b in zip(s0, x[r])]
            else:
                n1 = n1 + 1.0
                s1 = [a + b for a, b in zip(s1, x[r])]
        if n0 > 0.0:
            c0 = [v / n0 for v in s0]
        if n1 > 0.0:
            c1 = [v / n1 for v in s1]
    sse = 0.0
    for li, r in enumerate(idx):
        sse = sse + _sq(x[r], c1 if lab[li] else c0)
    return lab, c0, c1, sse


def _py_bisecting(x, k, max_iter, n_init, seed, strategy):
    x = [list(map(float, r)) for r in x]
    n = len(x)
    c = [0.0] * len(x[0])
    for r in x:
        c = [a + b for a, b in zip(c, r)]
    c = [v / float(n) for v in c]
    sse = 0.0
    for r in x:
        sse = sse + _sq(r, c)
    clusters = [(list(range(n)), c, sse)]
    split = 0
    while len(clusters) < k:
        t = None
        for ci, cl in enumerate(clusters):
            if len(cl[0]) < 2:
                continue
            key = len(cl[0]) if strategy == "largest_cluster" else cl[2]
            if t is None or not (tkey > key):
                t, tkey = ci, key
        if t is None:
            break
        idx = clusters[t][0]
        best = None
        for run in range(n_init):
            lab, c0, c1, s = _two_means(x, idx, max_iter, _stream(seed + split * 1000 + run))
            if s < (best[3] if best else 1.7976931348623157e308):
                best = (lab, c0, c1, s)
        split += 1
        lab, c0, c1, _ = best
        i0 = [r for r, lb in zip(idx, lab) if lb == 0]
        i1 = [r for r, lb in zip(idx, lab) if lb == 1]
        s0 = 0.0
        for r in i0:
            s0 = s0 + _sq(x[r], c0)
        s1 = 0.0
        for r in i1:
            s1 = s1 + _sq(x[r], c1)
        del clusters[t]
        if i0:
            clusters.append((i0, c0, s0))
        if i1:
            clusters.append((i1, c1, s1))
    labels = [0] * n
    inertia = 0.0
    for ci, cl in enumerate(clusters):
        for r in cl[0]:
            labels[r] = ci
        inertia = inertia + cl[2]
    return np.array([cl[1] for cl in clusters]), np.array(labels), inertia


@pytest.mark.parametrize("strategy", ["largest_cluster", "largest_sse"])
@pytest.mark.parametrize("n,d,k", [(40, 2, 4), (60, 3, 6), (25, 5, 3)])
def test_oracle_matches_a_literal_python_restatement(strategy, n, d, k):
    rng = np.random.default_rng(n * d + k)
    x = rng.normal(size=(n, d)) * 2 + rng.integers(0, 4, size=(n, 1)) * 5
    want_c, want_l, want_i = _py_bisecting(x, k, 30, 3, 9, strategy)
    got = O.bisecting_fit(x, k, max_iter=30, n_init=3, seed=9, strategy=strategy)
    assert np.array_equal(got["labels"], want_l)
    assert np.array_equal(got["centers"], want_c)
    assert got["inertia"] == want_i


# The library's side without a GPU: defaults and argument errors in the
# reference's validation order (bisecting_kmeans.rs:333-358).
def test_library_defaults_match_the_builder():
    import ctypes as C
    import ferrolearn_gb300 as F
    from ferrolearn_gb300 import _native
    p = _native.BisectingParams()
    _native.lib().fk_bisecting_params_default(C.byref(p), 5)
    assert (p.n_clusters, p.max_iter, p.n_init, p.has_random_state, p.strategy) == (5, 300, 10, 0, 0)  # :93-102
    m = F.BisectingKMeans(5)
    assert (m.max_iter, m.n_init, m.random_state, m.strategy) == (300, 10, None, "largest_cluster")


@pytest.mark.parametrize("k,x,kw,exc,needle", [
    (0, np.ones((3, 2)), {}, "InvalidParameter", "n_clusters"),
    (3, np.ones((9, 2)), dict(n_init=0), "InvalidParameter", "n_init"),
    (3, np.zeros((0, 2)), {}, "InsufficientSamples", "Insufficient"),
    (5, np.ones((2, 2)), {}, "InsufficientSamples", "Insufficient"),
    (0, np.zeros((0, 2)), dict(n_init=0), "InvalidParameter", "n_clusters"),
    (2, np.ones((4, 1025)), {}, "Unsupported", "d <= 1024"),
])
def test_library_validation_order(k, x, kw, exc, needle):
    import ferrolearn_gb300 as F
    for dtype in ("f64", "f32"):
        m = F.BisectingKMeans(k, dtype=dtype)
        if "n_init" in kw:
            m.with_n_init(kw["n_init"])
        with pytest.raises(getattr(F, exc), match=needle):
            m.fit(x)


def test_library_rejects_unknown_strategy():
    import ferrolearn_gb300 as F
    with pytest.raises(F.InvalidParameter):
        F.BisectingKMeans(2).with_bisecting_strategy("smallest")

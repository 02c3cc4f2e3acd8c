"""MiniBatchKMeans without a GPU: the oracle's restatement of
mini_batch_kmeans.rs pinned against the reference's own unit tests
(mini_batch_kmeans.rs:693-951, run on the library's uniform stream in place
of StdRng), the library's batch-index generator against the oracle's, and
the C ABI's argument errors in the reference's validation order (:495-526)."""
import numpy as np
import pytest

import ferrolearn_gb300 as F
from oracle import oracle as O

BLOBS = np.array([0.0, 0.0, 0.1, 0.1, -0.1, 0.1,
                  10.0, 10.0, 10.1, 10.1, 9.9, 10.1,
                  0.0, 10.0, 0.1, 10.1, -0.1, 9.9]).reshape(9, 2)  # make_blobs, :694-704


def _grouped(labels):
    return (labels[0] == labels[1] == labels[2] and labels[3] == labels[4] == labels[5]
            and labels[6] == labels[7] == labels[8] and len({labels[0], labels[3], labels[6]}) == 3)


def test_oracle_well_separated_blobs_and_predict():  # :707-727, :762-780
    r = O.minibatch_fit(BLOBS, 3, batch_size=9, n_init=5, seed=42)
    assert _grouped(r["labels"])
    new = np.array([[0.05, 0.05], [10.05, 10.05], [0.05, 10.05]])
    p = O.predict(r["centers"], new)
    assert list(p) == [r["labels"][0], r["labels"][3], r["labels"][6]]


def test_oracle_shapes_inertia_and_n_iter():  # :730-760, :782-789
    r = O.minibatch_fit(BLOBS, 3, seed=42)
    assert r["centers"].shape == (3, 2) and r["labels"].shape == (9,)
    assert r["inertia"] >= 0.0
    assert r["n_iter"] == 100  # tol 0: every one of max_iter batches runs
    assert O.transform(r["centers"], BLOBS).shape == (9, 3)


def test_oracle_transform_structure():  # :791-811
    x = np.array([[0.0, 0.0], [10.0, 0.0], [0.0, 10.0], [10.0, 10.0]])
    r = O.minibatch_fit(x, 2, batch_size=4, n_init=5, seed=42)
    dist = O.transform(r["centers"], x)
    for i in range(4):
        own = r["labels"][i]
        assert dist[i, own] <= dist[i, 1 - own] + 1e-10


def test_oracle_reproducible_random_init_single_cluster():  # :813-852
    a = O.minibatch_fit(BLOBS, 3, batch_size=9, seed=99)
    b = O.minibatch_fit(BLOBS, 3, batch_size=9, seed=99)
    assert np.array_equal(a["labels"], b["labels"]) and a["inertia"] == b["inertia"]
    r = O.minibatch_fit(BLOBS, 3, batch_size=9, n_init=5, seed=42, init="random")
    assert r["centers"].shape == (3, 2) and r["inertia"] >= 0.0
    x = np.array([[1.0, 1.0], [2.0, 2.0], [3.0, 3.0], [4.0, 4.0]])
    assert (O.minibatch_fit(x, 1, batch_size=4, seed=42)["labels"] == 0).all()


def test_oracle_errors():  # :854-877, :935-940
    x = np.array([[1.0, 1.0], [2.0, 2.0], [3.0, 3.0]])
    for kw, code in [(dict(k=0), 1), (dict(k=2, batch_size=0), 1), (dict(k=3, n_init=0), 1)]:
        k = kw.pop("k")
        with pytest.raises(O.OracleError) as e:
            O.minibatch_fit(x, k, **kw)
        assert e.value.code == code
    with pytest.raises(O.OracleError) as e:
        O.minibatch_fit(x[:2], 5)
    assert e.value.code == 2
    with pytest.raises(O.OracleError) as e:
        O.minibatch_fit(np.zeros((0, 2)), 3)
    assert e.value.code == 2


def test_oracle_f32_large_batch_identical_points():  # :905-933, :942-950
    x32 = BLOBS[:6].astype(np.float32)
    r = O.minibatch_fit(x32, 2, batch_size=6, seed=42)
    assert r["labels"].shape == (6,) and r["centers"].dtype == np.float32
    r = O.minibatch_fit(BLOBS, 3, batch_size=1000, seed=7)
    assert r["centers"].shape == (3, 2)
    same = np.ones((4, 2))
    assert abs(O.minibatch_fit(same, 1, batch_size=4, seed=42)["inertia"]) <= 1e-10


def test_oracle_update_is_the_running_mean():
    # one centre, counts starting at 1: after the batch the centre is the mean
    # of the initial centre and the batch rows (c += (x - c) / count)
    x = np.array([[2.0], [4.0], [8.0]])
    r = O.minibatch_fit(x, 1, batch_size=3, max_iter=1, n_init=1, init_centers=np.array([[[0.0]]]))
    assert r["centers"][0, 0] == pytest.approx((0.0 + 2.0 + 4.0 + 8.0) / 4, rel=1e-15)


def test_oracle_tolerance_stops_early():
    x = np.repeat(BLOBS, 3, axis=0)
    r = O.minibatch_fit(x, 3, batch_size=4, max_iter=500, tol=1e-3, n_init=2, seed=5)
    assert 1 <= r["n_iter"] < 500
    assert (r["run_n_iter"] >= 1).all() and r["run_inertia"][r["best_run"]] == r["inertia"]


@pytest.mark.parametrize("seed,pos,n,batch,iters", [(42, 0, 10, 4, 3), (7, 13, 5, 9, 2), (1, 0, 1000, 1000, 2),
                                                     (3, 5, 100_000, 1024, 5), (9, 0, 1, 1, 3), (2**63, 77, 50, 49, 4)])
def test_library_batch_indices_match_the_oracle(seed, pos, n, batch, iters):
    # the library draws its batches from a sparse partial Fisher-Yates pass;
    # the oracle restates sample_batch_indices with the whole pool
    got = F.minibatch_batch_indices(seed, pos, n, batch, iters)
    want = O.minibatch_indices(seed, pos, n, batch, iters)
    assert np.array_equal(got, want)
    for row in got:
        assert len(set(row.tolist())) == len(row) and row.min() >= 0 and row.max() < n


def test_library_defaults_match_the_builder():
    import ctypes as C
    from ferrolearn_gb300 import _native
    p = _native.MiniBatchParams()
    _native.lib().fk_minibatch_params_default(C.byref(p), 4)
    # MiniBatchKMeans::new, mini_batch_kmeans.rs:108-118
    assert (p.n_clusters, p.batch_size, p.max_iter, p.tol, p.n_init, p.has_random_state, p.init) == \
        (4, 1024, 100, 0.0, 3, 0, 0)
    m = F.MiniBatchKMeans(4)
    assert (m.batch_size, m.max_iter, m.tol, m.n_init, m.random_state, m.init) == (1024, 100, 0.0, 3, None, "kmeans++")


@pytest.mark.parametrize("kw,x,exc,needle", [
    (dict(k=0), np.ones((3, 2)), F.InvalidParameter, "n_clusters"),             # :495-500
    (dict(k=2, batch_size=0), np.ones((3, 2)), F.InvalidParameter, "batch_size"),  # :501-506
    (dict(k=3, n_init=0), np.ones((3, 2)), F.InvalidParameter, "n_init"),         # :507-512
    (dict(k=3), np.zeros((0, 2)), F.InsufficientSamples, "Insufficient"),         # :513-519
    (dict(k=5), np.ones((2, 2)), F.InsufficientSamples, "Insufficient"),          # :520-526
    (dict(k=0, batch_size=0), np.zeros((0, 2)), F.InvalidParameter, "n_clusters"),  # order: n_clusters first
])
def test_library_validation_order(kw, x, exc, needle):
    for dtype in ("f64", "f32"):
        m = F.MiniBatchKMeans(kw["k"], dtype=dtype)
        if "batch_size" in kw:
            m.with_batch_size(kw["batch_size"])
        if "n_init" in kw:
            m.with_n_init(kw["n_init"])
        with pytest.raises(exc, match=needle):
            m.fit(x)


def test_library_rejects_unknown_init():
    with pytest.raises(F.InvalidParameter):
        F.MiniBatchKMeans(2).with_init("farthest")


# A second, literal restatement in Python floats (IEEE f64, no fused
# multiply-add) for small inputs: it checks the C oracle statement by
# statement, including the stream positions.
def _py_stream(seed):
    state = [seed & (2**64 - 1)]
    M = 2**64 - 1

    def nxt():
        state[0] = (state[0] + 0x9E3779B97F4A7C15) & M
        z = state[0]
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        z ^= z >> 31
        return (z >> 11) * (1.0 / 9007199254740992.0)

    def rng(n):  # random_range(0..n)
        import math
        return min(max(int(math.floor(nxt() * n)), 0), n - 1)
    return nxt, rng


def _py_sq(a, b):
    acc = 0.0
    for u, v in zip(a, b):
        t = u - v
        acc = acc + t * t
    return acc


def _py_nearest(row, cs):
    best, bd = 0, 1.7976931348623157e308
    for q, c in enumerate(cs):
        v = _py_sq(row, c)
        if v < bd:
            best, bd = q, v
    return best, bd


def _py_kpp(x, k, nxt, rng):
    import math
    n = len(x)
    cs = [list(x[rng(n)])]
    if k == 1:
        return cs
    mind = [_py_sq(r, cs[0]) for r in x]
    trials = max(2 + int(math.floor(math.log(k))), 1)
    for _ in range(1, k):
        total = 0.0
        for v in mind:
            total = total + v
        if total <= 0.0:
            cs.append(list(x[rng(n)]))
            continue
        best = None
        for _t in range(trials):
            thr = nxt() * total
            cum, cand = 0.0, n - 1
            for i, v in enumerate(mind):
                cum = cum + v
                if cum >= thr:
                    cand = i
                    break
            nd = []
            for r, m in zip(x, mind):
                v = _py_sq(r, x[cand])
                nd.append(v if v < m else m)
            pot = 0.0
            for v in nd:
                pot = pot + v
            if best is None or pot < best[0]:
                best = (pot, cand, nd)
        cs.append(list(x[best[1]]))
        mind = best[2]
    return cs


def _py_minibatch(x, k, batch, max_iter, tol, n_init, seed, init):
    x = [list(map(float, r)) for r in x]
    n = len(x)
    best = None
    for run in range(n_init):
        nxt, rng = _py_stream(seed + run * 1000003)
        if init == "random":
            pool = list(range(n))
            cs = []
            for i in range(k):
                j = i + rng(n - i)
                pool[i], pool[j] = pool[j], pool[i]
                cs.append(list(x[pool[i]]))
        else:
            cs = _py_kpp(x, k, nxt, rng)
        counts = [1] * k
        n_iter = 0
        for _ in range(max_iter):
            pool = list(range(n))
            m = min(batch, n)
            idx = []
            for i in range(m):
                j = i + rng(n - i)
                pool[i], pool[j] = pool[j], pool[i]
                idx.append(pool[i])
            labs = [_py_nearest(x[i], cs)[0] for i in idx]
            old = [list(c) for c in cs]
            for i, lab in zip(idx, labs):
                counts[lab] += 1
                lr = 1.0 / float(counts[lab])
                cs[lab] = [c + lr * (v - c) for c, v in zip(cs[lab], x[i])]
            shift = 0.0
            for c, o in zip(cs, old):
                s = _py_sq(c, o) ** 0.5
                if s > shift:
                    shift = s
            n_iter += 1
            if shift < tol:
                break
        labels, inertia = [], 0.0
        for r in x:
            lab, dist = _py_nearest(r, cs)
            labels.append(lab)
            inertia = inertia + dist
        if best is None or inertia < best["inertia"]:
            best = dict(centers=np.array(cs), labels=np.array(labels), inertia=inertia, n_iter=n_iter, best_run=run)
    return best


@pytest.mark.parametrize("init", ["kmeans++", "random"])
@pytest.mark.parametrize("n,d,k,batch,tol", [(60, 3, 4, 16, 0.0), (40, 2, 3, 100, 0.0), (80, 4, 5, 7, 0.05)])
def test_oracle_matches_a_literal_python_restatement(init, n, d, k, batch, tol):
    rng = np.random.default_rng(n + d + k)
    x = rng.normal(size=(n, d)) * 3 + rng.integers(0, 3, size=(n, 1)) * 6
    want = _py_minibatch(x, k, batch, 12, tol, 2, 17, init)
    got = O.minibatch_fit(x, k, batch_size=batch, max_iter=12, tol=tol, n_init=2, seed=17, init=init)
    assert np.array_equal(got["labels"], want["labels"])
    assert np.array_equal(got["centers"], want["centers"])
    assert got["inertia"] == want["inertia"] and got["n_iter"] == want["n_iter"]
    assert got["best_run"] == want["best_run"]

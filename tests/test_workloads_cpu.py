"""CPU checks of the seeded workload generators: shapes, dtypes, seeding, that
each init is made of rows of X, and that the bisector workload holds its 10%
of near-tie rows (equidistant to two centres up to f32 rounding)."""
import numpy as np

from ferrolearn_gb300 import workloads as W


def _rows_of(init, x):
    """True when every row of init is (exactly) some row of x."""
    x64 = np.asarray(x, dtype=np.float64)
    keys = {r.tobytes() for r in x64}
    return all(np.asarray(r, dtype=np.float64).tobytes() in keys for r in init)


def test_isotropic_shapes_seed_and_init():
    a = W.isotropic_8x16()
    assert a["x"].shape == (10_000, 16) and a["x"].dtype == np.float64 and a["k"] == 8
    assert a["init"].shape == (8, 16) and _rows_of(a["init"], a["x"])
    assert (a["max_iter"], a["tol"], a["n_init"]) == (300, 1e-4, 1)
    b = W.isotropic_8x16()
    assert np.array_equal(a["x"], b["x"]) and np.array_equal(a["init"], b["init"])
    c = W.isotropic_8x16(seed=1)
    assert not np.array_equal(a["x"], c["x"])
    assert W.isotropic_8x16(scale=0.1)["x"].shape == (1000, 16)


def test_dirichlet_shapes_and_dtype():
    w = W.dirichlet_256x64(scale=0.004)
    assert w["x"].shape == (4000, 64) and w["x"].dtype == np.float64 and w["x"].flags.c_contiguous
    assert w["k"] == 256 and w["init"] is None and (w["max_iter"], w["tol"]) == (100, 1e-4)
    w32 = W.dirichlet_256x64(scale=0.004, dtype=np.float32)
    assert w32["x"].dtype == np.float32
    np.testing.assert_array_equal(w32["x"], w["x"].astype(np.float32))
    # never fewer rows than clusters
    assert W.dirichlet_256x64(scale=1e-6)["x"].shape[0] == 256


def test_anisotropic_shapes_init_and_blob_spread():
    w = W.anisotropic_1024x128(scale=0.001)
    x = w["x"]
    assert x.shape == (4000, 128) and x.dtype == np.float32 and x.flags.c_contiguous
    assert w["k"] == 1024 and (w["max_iter"], w["tol"]) == (50, 0.0)
    assert w["init"].shape == (1024, 128) and w["init"].dtype == np.float64
    assert _rows_of(w["init"], x)
    assert len({r.tobytes() for r in w["init"]}) == 1024  # k distinct rows
    # centres U[-15,15]: the data stays within the centre box plus a few blob widths
    assert np.abs(x).max() < 15 + 12 * 0.3 * np.sqrt(128)


def _bisector_centres(seed=0, k=4096, d=256):
    rng = np.random.default_rng(seed)
    return rng.uniform(-30.0, 30.0, size=(k, d)).astype(np.float32)


def test_bisector_rows_are_equidistant_to_their_pair():
    cen = _bisector_centres(k=64, d=32)
    rows = W._bisector_rows(cen, 500, np.random.default_rng(7))
    rng = np.random.default_rng(7)
    a = rng.integers(0, 64, size=500)
    b = (a + 1 + rng.integers(0, 63, size=500)) % 64
    assert np.all(a != b)
    da = ((rows - cen[a].astype(np.float64)) ** 2).sum(1)
    db = ((rows - cen[b].astype(np.float64)) ** 2).sum(1)
    np.testing.assert_allclose(da, db, rtol=1e-12)
    r32 = rows.astype(np.float32).astype(np.float64)
    da = ((r32 - cen[a]) ** 2).sum(1)
    db = ((r32 - cen[b]) ** 2).sum(1)
    assert np.all(np.abs(da - db) <= 1e-6 * da)  # f32 storage: a tie up to rounding


def test_bisector_workload_holds_ten_percent_near_ties():
    w = W.bisector_4096x256(scale=0.001)
    x, k = w["x"], w["k"]
    assert x.shape == (8000, 256) and x.dtype == np.float32 and k == 4096
    assert w["x_predict"].shape == (2000, 256) and w["x_predict"].dtype == np.float32
    assert w["init"].shape == (4096, 256) and _rows_of(w["init"], x)
    assert (w["max_iter"], w["tol"]) == (20, 0.0)
    cen = _bisector_centres().astype(np.float64)
    c2 = (cen * cen).sum(1)
    for rows, m_bis in ((x, 800), (w["x_predict"], 200)):
        x64 = rows.astype(np.float64)
        dist = (x64 * x64).sum(1)[:, None] - 2.0 * x64 @ cen.T + c2[None, :]
        two = np.partition(dist, 1, axis=1)[:, :2]
        gap = (two[:, 1] - two[:, 0]) / two[:, 1]
        # bisector rows tie their two nearest centres up to f32 rounding;
        # blob rows (std 1 around centres about 390 apart) are far from a tie
        assert int((gap < 1e-5).sum()) == m_bis
        assert np.sort(gap)[m_bis] > 0.5


def test_batched_problem_ranges():
    probs = W.batched_512(n_problems=64)
    assert len(probs) == 64
    seeds = set()
    for p in probs:
        n, d = p["x"].shape
        assert 2000 <= n <= 200_000 and d in (8, 16, 32, 64) and 4 <= p["k"] <= 64
        assert p["x"].dtype == np.float32 and p["x"].flags.c_contiguous
        assert (p["n_init"], p["max_iter"], p["tol"]) == (10, 300, 1e-4)
        seeds.add(p["random_state"])
    assert len(seeds) == 64
    small = W.batched_512(scale=0.001, n_problems=16)
    assert all(p["x"].shape[0] >= p["k"] for p in small)
    # the same seed gives the same problems
    again = W.batched_512(n_problems=64)
    assert all(np.array_equal(p["x"], q["x"]) for p, q in zip(probs, again))

"""GPU tests of the mixed BF16 tensor-core path (tcgen05 + TMA + TMEM) with the
exact FP64 re-check.

1. The raw FP32 accumulators of one tile equal an exact f64 product of the
   BF16 operands the kernel used (checks the TMA swizzle, the shared-memory
   and instruction descriptors and the TMEM read-out layout).
2. Every top-2 record agrees with the exact scores up to the documented key
   truncation (2^-15 relative) plus the FP32 accumulation error.
3. Lloyd steps and full fits on the f32x64 entry point give labels identical
   to the FP64 oracle at every iteration, centres within 1e-13 relative (they
   are the correctly rounded means of exact fixed-point sums, the oracle's
   sequential f64 sums can differ by a few ulp) and the same n_iter; the
   inertia (compensated f32 partials) within 1e-6 relative.
"""
import ctypes as C

import numpy as np
import pytest

import ferrolearn_gb300 as F
from ferrolearn_gb300 import _native
from ferrolearn_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

INERTIA_RTOL_MIXED = 1e-6
CENTRE_RTOL_MIXED = 1e-13


def _close(a, b):
    scale = np.nanmax(np.abs(b)) if np.isfinite(b).any() else 1.0
    same_nan = np.array_equal(np.isnan(a), np.isnan(b))
    return same_nan and np.nanmax(np.abs(a - b)) <= CENTRE_RTOL_MIXED * scale


def _bf16_to_f32(u16):
    return (u16.astype(np.uint32) << 16).view(np.float32)


def _probe(x32, c64):
    torch = pytest.importorskip("torch")
    ctx = F.default_context()
    n, d = x32.shape
    k = c64.shape[0]
    xd = torch.from_numpy(np.ascontiguousarray(x32)).cuda()
    cd = torch.from_numpy(np.ascontiguousarray(c64)).cuda()
    d_pad = (d + 63) // 64 * 64
    kmax = (k + 255) // 256 * 256 * 2 + 512
    dump = np.zeros(128 * kmax, dtype=np.float32)
    xb = np.zeros(128 * d_pad, dtype=np.uint16)
    cb = np.zeros(kmax * d_pad, dtype=np.uint16)
    aug = np.zeros(kmax * 16, dtype=np.uint16)
    top = np.zeros(n * 8 * 8, dtype=np.float32)
    plan = np.zeros(8, dtype=np.int32)
    st = _native.lib().fk_debug_tc_probe(ctx.handle, C.c_void_p(xd.data_ptr()), n, d, C.c_void_p(cd.data_ptr()), k,
                                         dump.ctypes.data_as(C.c_void_p), xb.ctypes.data_as(C.c_void_p),
                                         cb.ctypes.data_as(C.c_void_p), aug.ctypes.data_as(C.c_void_p),
                                         top.ctypes.data_as(C.c_void_p), plan.ctypes.data_as(C.c_void_p))
    assert st == 0, _native.last_error()
    d_pad, kp, parts, k_pad, grid, err = plan[:6]
    assert err == 0
    rows = min(n, 128)
    xbf = _bf16_to_f32(xb[: rows * d_pad]).reshape(rows, d_pad).astype(np.float64)
    cbf = _bf16_to_f32(cb[: k_pad * d_pad]).reshape(k_pad, d_pad).astype(np.float64)
    augf = _bf16_to_f32(aug[: k_pad * 16]).reshape(k_pad, 16).astype(np.float64)
    acc = dump[: 128 * kp].reshape(128, kp)[:rows]
    recs = top[: parts * n * 8].view(np.uint32).reshape(parts, n, 8)
    return dict(acc=acc, xb=xbf, cb=cbf, aug=augf, kp=kp, parts=parts, k_pad=k_pad, recs=recs)


def _aniso(n, d, k, seed):
    rng = np.random.default_rng(seed)
    cen = rng.uniform(-15, 15, size=(k, d))
    lab = rng.integers(0, k, size=n)
    x = cen[lab] + rng.normal(0, 3.0, size=(n, d))
    return x.astype(np.float32), cen


@pytest.mark.parametrize("n,d,k", [(300, 128, 300), (200, 64, 1024), (150, 16, 40), (260, 128, 1024), (129, 100, 7)])
def test_tc_accumulators_exact(n, d, k):
    x32, cen = _aniso(n, d, k, seed=n + d + k)
    c = x32[np.random.default_rng(0).choice(n, size=min(k, n), replace=False)].astype(np.float64)
    if c.shape[0] < k:
        c = np.concatenate([c, cen[: k - c.shape[0]]])
    r = _probe(x32, c)
    kp = r["kp"]
    ref = r["xb"] @ r["cb"][:kp].T + r["aug"][:kp].sum(1)[None, :]
    big = np.abs(ref).max()
    err = np.abs(r["acc"].astype(np.float64) - ref).max()
    assert err <= 1e-5 * big, (err, big)


@pytest.mark.parametrize("n,d,k", [(1000, 128, 1024), (700, 64, 300), (333, 32, 5)])
def test_tc_top2_records(n, d, k):
    x32, cen = _aniso(n, d, k, seed=7 + d)
    c = cen.astype(np.float64)
    r = _probe(x32, c)
    kp, parts = r["kp"], r["parts"]
    # full exact scores from the device operands (all rows)
    torch = pytest.importorskip("torch")  # noqa: F841
    recs = r["recs"]
    v1 = recs[..., 0].view(np.float32)
    u3 = recs[..., 2].view(np.float32)
    i1 = recs[..., 4].view(np.int32)
    i2 = recs[..., 5].view(np.int32)
    # the best over all slices must be a centre whose exact score is within the
    # truncation + accumulation slack of the true maximum (rows of the first tile)
    rows = r["xb"].shape[0]
    scores = r["xb"] @ r["cb"].T + r["aug"].sum(1)[None, :]
    best = scores[:, :k].max(1)
    for p in range(parts):
        lo, hi = p * kp, min(k, (p + 1) * kp)
        if lo >= k:
            continue
        sl = scores[:, lo:hi]
        m = sl.max(1)
        assert np.all(np.abs(v1[p, :rows] - m) <= 2 ** -14 * np.abs(m) + 1e-5 * best)
        picked = sl[np.arange(rows), i1[p, :rows] - lo]
        assert np.all(m - picked <= 2 ** -14 * np.abs(m) + 1e-5 * best)
        # u3 bounds every score of the slice other than the two kept ones
        rest = sl.copy()
        rest[np.arange(rows), i1[p, :rows] - lo] = -np.inf
        rest[np.arange(rows), i2[p, :rows] - lo] = -np.inf
        assert np.all(rest.max(1) <= u3[p, :rows] + 2 ** -14 * np.abs(m) + 1e-5 * best)


@pytest.mark.parametrize("n,d,k", [(4096, 128, 1024), (5000, 64, 100), (3000, 16, 9), (2500, 100, 300)])
def test_mixed_steps_match_fp64_oracle(n, d, k):
    x32, _ = _aniso(n, d, k, seed=11 * d + k)
    x64 = x32.astype(np.float64)
    c = x64[np.random.default_rng(1).choice(n, size=k, replace=False)].copy()
    for _ in range(3):
        gl, gc, gi, gs, rep = F.lloyd_step(x32, c, dtype="f32x64", precision="bf16")
        ol, oc, oi, os_ = O.lloyd_step(x64, c)
        assert np.array_equal(gl, ol)
        assert _close(gc, oc)
        assert abs(gs - os_) <= 1e-12 * max(os_, 1e-300)
        assert abs(gi - oi) <= INERTIA_RTOL_MIXED * oi
        c = oc


def test_mixed_fit_anisotropic_small():
    w = W.anisotropic_1024x128(scale=0.005)  # 20,000 rows, same distribution
    x32, k = w["x"], w["k"]
    g = F.KMeans(k, dtype="f32x64").with_precision("bf16").with_max_iter(8).with_tol(0.0).with_n_init(1) \
        .with_init_centers(w["init"]).fit(x32)
    o = O.fit(x32.astype(np.float64), k, max_iter=8, tol=0.0, n_init=1, init=w["init"][None])
    assert np.array_equal(g.labels(), o["labels"])
    assert _close(g.cluster_centers(), o["centers"])
    assert g.n_iter() == o["n_iter"] == 8
    assert abs(g.inertia() - o["inertia"]) <= INERTIA_RTOL_MIXED * o["inertia"]


def test_mixed_exact_ties_and_nan_rows_are_rechecked():
    rng = np.random.default_rng(5)
    d, k = 64, 40
    c = rng.uniform(-10, 10, size=(k, d))
    x = c[rng.integers(0, k, 3000)] + rng.normal(0, 1, size=(3000, d))
    # rows exactly on the bisector of centres 3 and 17 (in real arithmetic)
    for t in range(200):
        a, b = c[3], c[17]
        u = rng.normal(size=d)
        u -= (u @ (b - a)) / ((b - a) @ (b - a)) * (b - a)
        x[t] = (a + b) / 2 + 0.1 * u
    x[-1, 5] = np.nan
    x32 = x.astype(np.float32)
    x64 = x32.astype(np.float64)
    gl, gc, gi, gs, rep = F.lloyd_step(x32, c, dtype="f32x64", precision="bf16")
    ol, oc, oi, os_ = O.lloyd_step(x64, c)
    assert np.array_equal(gl, ol)
    assert _close(gc, oc)
    assert rep["rows_rechecked"] >= 200
    assert rep["rows_full_rescan"] >= 1


def test_fixed_point_sums_handle_extremes():
    # tiny, huge, signed zero, infinities: the update must follow IEEE f64
    # summation of the f32 values (here all sums are exact in f64)
    x = np.zeros((8, 4), dtype=np.float32)
    x[:, 0] = [1e-30, -1e-30, 3e-38, 1.0, 2.0, -3.0, 1e20, -1e20]
    x[:, 1] = [np.inf, 1, 2, 3, 4, 5, 6, 7]
    x[:, 2] = [np.inf, -np.inf, 0, 0, 0, 0, 0, 0]
    x[:, 3] = -0.0
    c = np.zeros((1, 4))
    gl, gc, gi, gs, rep = F.lloyd_step(x, c, dtype="f32x64", precision="bf16")
    ol, oc, oi, os_ = O.lloyd_step(x.astype(np.float64), c)
    assert np.array_equal(gl, ol)
    assert np.array_equal(gc, oc, equal_nan=True)


def test_mixed_predict_matches_oracle():
    x32, cen = _aniso(6000, 128, 500, seed=3)
    fitted = F.FittedKMeans(cen.astype(np.float64), np.zeros(6000, dtype=np.int64), 0.0, 0, "f32x64",
                            precision=F.MIXED_BF16)
    assert np.array_equal(fitted.predict(x32), O.predict(cen, x32.astype(np.float64)))


def _equidistant_rows(c, ids, count, rng, spread=0.5):
    """Rows at equal (real) distance from the centres ids: the circumcentre of
    their affine hull plus offsets orthogonal to it."""
    base = c[ids[0]]
    dirs = np.stack([c[i] - base for i in ids[1:]])  # (m-1, d)
    gram = dirs @ dirs.T
    rhs = 0.5 * np.array([dv @ dv for dv in dirs])
    coef = np.linalg.solve(gram, rhs)
    centre = base + coef @ dirs
    q, _ = np.linalg.qr(dirs.T)
    rows = []
    for _ in range(count):
        u = rng.normal(size=c.shape[1])
        u -= q @ (q.T @ u)
        rows.append(centre + spread * u)
    return np.array(rows)


def test_mixed_multiway_ties_use_the_second_pass():
    # rows equidistant from three and from six centres: the first pass cannot
    # separate them, the top-4 second pass (or the exhaustive path for six)
    # must, and the labels must still be the FP64 oracle's
    rng = np.random.default_rng(8)
    d, k = 64, 300
    c = rng.uniform(-10, 10, size=(k, d))
    c[[1, 2, 3, 4, 6, 7]] = c[1] + rng.normal(0, 0.5, size=(6, d))  # six close centres
    x = c[rng.integers(0, k, 6000)] + rng.normal(0, 1, size=(6000, d))
    x[:300] = _equidistant_rows(c, [5, 40, 77], 300, rng)
    x[300:360] = _equidistant_rows(c, [1, 2, 3, 4, 6, 7], 60, rng)
    x32 = x.astype(np.float32)
    x64 = x32.astype(np.float64)
    gl, gc, gi, gs, rep = F.lloyd_step(x32, c, dtype="f32x64", precision="bf16")
    ol, oc, oi, os_ = O.lloyd_step(x64, c)
    assert np.array_equal(gl, ol)
    assert _close(gc, oc)
    assert rep["rows_full_rescan"] >= 300
    assert rep["rows_fp64"] >= 100

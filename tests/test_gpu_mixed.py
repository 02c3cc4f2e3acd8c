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
4. Fits update the exact sums from the rows whose label changed; their
   centres equal, bit for bit, full recomputations step by step.
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


def _e4m3_to_f64(u8):
    """E4M3 (1 sign, 4 exponent bits with bias 7, 3 mantissa bits; no
    infinities, S.1111.111 is NaN) decoded exactly."""
    u = u8.astype(np.int64)
    e = (u >> 3) & 15
    m = (u & 7).astype(np.float64)
    v = np.where(e == 0, m / 8.0 * 2.0 ** -6, (1.0 + m / 8.0) * np.exp2(e.astype(np.float64) - 7.0))
    v = np.where((e == 15) & ((u & 7) == 7), np.nan, v)
    return np.where(u & 0x80, -v, v)


def _probe(x32, c64, precision="bf16"):
    torch = pytest.importorskip("torch")
    ctx = F.default_context()
    n, d = x32.shape
    k = c64.shape[0]
    fp8 = precision == "fp8"
    xd = torch.from_numpy(np.ascontiguousarray(x32)).cuda()
    cd = torch.from_numpy(np.ascontiguousarray(c64)).cuda()
    per_atom = 128 if fp8 else 64
    d_pad = (d + per_atom - 1) // per_atom * per_atom
    kmax = (k + 255) // 256 * 256 * 2 + 512
    et = np.uint8 if fp8 else np.uint16
    dump = np.zeros(128 * kmax, dtype=np.float32)
    xq = np.zeros(128 * d_pad, dtype=et)
    cq = np.zeros(kmax * d_pad, dtype=et)
    aug = np.zeros(kmax * 16, dtype=np.uint16)
    xaug = np.zeros(128 * 16, dtype=np.uint16)
    top = np.zeros(n * 8 * 8, dtype=np.float32)
    plan = np.zeros(8, dtype=np.int32)
    vp = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    st = _native.lib().fk_debug_tc_probe(ctx.handle, C.c_void_p(xd.data_ptr()), n, d, C.c_void_p(cd.data_ptr()), k,
                                         F.MIXED_FP8 if fp8 else F.MIXED_BF16, vp(dump), vp(xq), vp(cq), vp(aug),
                                         vp(xaug), vp(top), vp(plan))
    assert st == 0, _native.last_error()
    d_pad_dev, kp, parts, k_pad, grid, err = plan[:6]
    assert err == 0 and d_pad_dev == d_pad
    rows = min(n, 128)
    dec = _e4m3_to_f64 if fp8 else (lambda u: _bf16_to_f32(u).astype(np.float64))
    xqf = dec(xq[: rows * d_pad]).reshape(rows, d_pad)
    cqf = dec(cq[: k_pad * d_pad]).reshape(k_pad, d_pad)
    augf = _bf16_to_f32(aug[: k_pad * 16]).reshape(k_pad, 16).astype(np.float64)
    if fp8:
        xaugf = _bf16_to_f32(xaug[: rows * 16]).reshape(rows, 16).astype(np.float64)
    else:
        xaugf = np.zeros((rows, 16))
        xaugf[:, :3] = 1.0
    acc = dump[: 128 * kp].reshape(128, kp)[:rows]
    recs = top[: parts * n * 8].view(np.uint32).reshape(parts, n, 8)
    scores = xqf @ cqf.T + xaugf @ augf.T  # exact in f64: the accumulator units of each row
    return dict(acc=acc, xq=xqf, cq=cqf, aug=augf, xaug=xaugf, scores=scores, kp=kp, parts=parts, k_pad=k_pad,
                recs=recs)


def _aniso(n, d, k, seed):
    rng = np.random.default_rng(seed)
    cen = rng.uniform(-15, 15, size=(k, d))
    lab = rng.integers(0, k, size=n)
    x = cen[lab] + rng.normal(0, 3.0, size=(n, d))
    return x.astype(np.float32), cen


PRECISIONS = ["bf16", "fp8"]


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("n,d,k", [(300, 128, 300), (200, 64, 1024), (150, 16, 40), (260, 128, 1024), (129, 100, 7),
                                   (140, 256, 600)])
def test_tc_accumulators_exact(n, d, k, precision):
    x32, cen = _aniso(n, d, k, seed=n + d + k)
    c = x32[np.random.default_rng(0).choice(n, size=min(k, n), replace=False)].astype(np.float64)
    if c.shape[0] < k:
        c = np.concatenate([c, cen[: k - c.shape[0]]])
    r = _probe(x32, c, precision)
    kp = r["kp"]
    ref = r["scores"][:, :kp]
    big = np.abs(ref).max()
    err = np.abs(r["acc"].astype(np.float64) - ref)
    assert err.max() <= 1e-5 * big, (err.max(), big)
    # the accumulation-error model of the re-check bound: (d_pad + 32) 2^-22
    # times (||xq|| max ||cq|| + the augmentation term), row by row
    d_pad = r["xq"].shape[1]
    xn = np.linalg.norm(r["xq"], axis=1)[:, None]
    chn = np.linalg.norm(r["cq"][:kp], axis=1).max()
    augv = np.abs(r["xaug"]) @ np.abs(r["aug"][:kp]).T
    bound = (d_pad + 32) * 2.0 ** -22 * (xn * chn + augv)
    assert np.all(err <= bound), (err / bound).max()


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("n,d,k", [(1000, 128, 1024), (700, 64, 300), (333, 32, 5)])
def test_tc_top2_records(n, d, k, precision):
    x32, cen = _aniso(n, d, k, seed=7 + d)
    c = cen.astype(np.float64)
    r = _probe(x32, c, precision)
    kp, parts = r["kp"], r["parts"]
    recs = r["recs"]
    v1 = recs[..., 0].view(np.float32)
    u3 = recs[..., 2].view(np.float32)
    i1 = recs[..., 4].view(np.int32)
    i2 = recs[..., 5].view(np.int32)
    # the best over all slices must be a centre whose exact score is within the
    # truncation + accumulation slack of the true maximum (rows of the first tile)
    scores = r["scores"]
    rows = scores.shape[0]
    best = scores[:, :k].max(1)
    for p in range(parts):
        lo, hi = p * kp, min(k, (p + 1) * kp)
        if lo >= k:
            continue
        sl = scores[:, lo:hi]
        m = sl.max(1)
        tol = 2 ** -14 * np.abs(m) + 1e-5 * best
        assert np.all(np.abs(v1[p, :rows] - m) <= tol)
        picked = sl[np.arange(rows), i1[p, :rows] - lo]
        assert np.all(m - picked <= tol)
        # u3 bounds every score of the slice other than the two kept ones
        rest = sl.copy()
        rest[np.arange(rows), i1[p, :rows] - lo] = -np.inf
        rest[np.arange(rows), i2[p, :rows] - lo] = -np.inf
        assert np.all(rest.max(1) <= u3[p, :rows] + tol)


def test_fp8_operands_are_scaled_roundings():
    # each row's E4M3 values times its power-of-two scale approximate x - mu
    # within E4M3's relative rounding (2^-4) or its subnormal step
    x32, cen = _aniso(256, 256, 64, seed=2)
    r = _probe(x32, cen.astype(np.float64), "fp8")
    xq, xaug = r["xq"], r["xaug"]
    s = 1.0 / xaug[:, 0]  # the augmentation row holds 2^-sh
    assert np.all(np.log2(s) == np.round(np.log2(s)))
    deq = xq[:, :256] * s[:, None]
    mu = x32.astype(np.float64).mean(0)  # the device centres by the f32 mean of the same rows
    t = x32[:128].astype(np.float64) - mu
    assert np.all(np.abs(xq).max(1) <= 256) and np.all(np.abs(xq).max(1) >= 128)
    # half an E4M3 ulp in the row's top binade is 1/16 of the row's max |t|
    assert np.all(np.abs(deq - t) <= np.abs(t).max(1, keepdims=True) / 16 * 1.001 + 1e-4)


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("n,d,k", [(4096, 128, 1024), (5000, 64, 100), (3000, 16, 9), (2500, 100, 300),
                                   (3000, 256, 700)])
def test_mixed_steps_match_fp64_oracle(n, d, k, precision):
    x32, _ = _aniso(n, d, k, seed=11 * d + k)
    x64 = x32.astype(np.float64)
    c = x64[np.random.default_rng(1).choice(n, size=k, replace=False)].copy()
    for _ in range(3):
        gl, gc, gi, gs, rep = F.lloyd_step(x32, c, dtype="f32x64", precision=precision)
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


@pytest.mark.parametrize("precision", PRECISIONS)
def test_mixed_exact_ties_and_nan_rows_are_rechecked(precision):
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
    gl, gc, gi, gs, rep = F.lloyd_step(x32, c, dtype="f32x64", precision=precision)
    ol, oc, oi, os_ = O.lloyd_step(x64, c)
    assert np.array_equal(gl, ol)
    assert _close(gc, oc)
    assert rep["rows_rechecked"] >= 200
    assert rep["rows_full_rescan"] >= 1


@pytest.mark.parametrize("precision", PRECISIONS)
def test_fixed_point_sums_handle_extremes(precision):
    # tiny, huge, signed zero, infinities: the update must follow IEEE f64
    # summation of the f32 values (here all sums are exact in f64)
    x = np.zeros((8, 4), dtype=np.float32)
    x[:, 0] = [1e-30, -1e-30, 3e-38, 1.0, 2.0, -3.0, 1e20, -1e20]
    x[:, 1] = [np.inf, 1, 2, 3, 4, 5, 6, 7]
    x[:, 2] = [np.inf, -np.inf, 0, 0, 0, 0, 0, 0]
    x[:, 3] = -0.0
    c = np.zeros((1, 4))
    gl, gc, gi, gs, rep = F.lloyd_step(x, c, dtype="f32x64", precision=precision)
    ol, oc, oi, os_ = O.lloyd_step(x.astype(np.float64), c)
    assert np.array_equal(gl, ol)
    assert np.array_equal(gc, oc, equal_nan=True)


@pytest.mark.parametrize("precision", [F.MIXED_BF16, F.MIXED_FP8])
@pytest.mark.parametrize("n,d,k", [(6000, 128, 500), (40000, 256, 600)])
def test_mixed_predict_matches_oracle(precision, n, d, k):
    # (40000, 256, 600): BF16 at d = 256 runs its one X stage as a ring of four
    # atom slots; 313 tiles over 50 CTAs a centre slice take every slot through
    # both barrier phases several times
    x32, cen = _aniso(n, d, k, seed=3)
    fitted = F.FittedKMeans(cen.astype(np.float64), np.zeros(n, dtype=np.int64), 0.0, 0, "f32x64",
                            precision=precision)
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


@pytest.mark.parametrize("precision", PRECISIONS)
def test_mixed_multiway_ties_use_the_second_pass(precision):
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
    gl, gc, gi, gs, rep = F.lloyd_step(x32, c, dtype="f32x64", precision=precision)
    ol, oc, oi, os_ = O.lloyd_step(x64, c)
    assert np.array_equal(gl, ol)
    assert _close(gc, oc)
    assert rep["rows_full_rescan"] >= 300
    assert rep["rows_fp64"] >= 100


def test_fp8_bisector_fit_and_predict_match_fp64_oracle():
    # the large-k FP8 workload's distribution at a size the oracle finishes
    # quickly: 10% of the rows on bisectors of two centres
    w = W.bisector_4096x256(scale=0.003, k=512)  # 24,000 rows, 6,000 to predict
    x32, k = w["x"], w["k"]
    g = F.KMeans(k, dtype="f32x64").with_precision("fp8").with_max_iter(3).with_tol(0.0).with_n_init(1) \
        .with_init_centers(w["init"]).fit(x32)
    o = O.fit(x32.astype(np.float64), k, max_iter=3, tol=0.0, n_init=1, init=w["init"][None])
    assert np.array_equal(g.labels(), o["labels"])
    assert _close(g.cluster_centers(), o["centers"])
    assert g.n_iter() == o["n_iter"] == 3
    assert abs(g.inertia() - o["inertia"]) <= INERTIA_RTOL_MIXED * o["inertia"]
    assert g.report["rows_rechecked"] >= int(0.1 * x32.shape[0])  # every bisector row at least
    xp = w["x_predict"]
    assert np.array_equal(g.predict(xp), O.predict(g.cluster_centers(), xp.astype(np.float64)))


def _plan(n, d, k, precision, topk, sms=152):
    out = (C.c_int64 * 10)()
    st = _native.lib().fk_debug_tc_plan(n, d, k, precision, topk, sms, out)
    assert st == 0
    return dict(zip(["d_pad", "kp", "parts", "k_pad", "nblocks", "xst", "smem", "grid", "ctas", "tiles"], out))


def test_fp8_bisector_at_full_k_and_d_matches_fp64_oracle():
    # the large-k FP8 workload at its own k = 4096 and d = 256 (200,000 rows,
    # 10% on bisectors): the E4M3 main pass runs 8 slices of 512 resident
    # centres and the BF16 second pass (count pass, then mask pass) 16 slices
    # of 256, the plans the full-size workload runs; labels of every
    # iteration, centres, n_iter and predict on fresh rows must be the FP64
    # oracle's
    w = W.bisector_4096x256(scale=0.025, predict_scale=0.01)
    x32, k = w["x"], w["k"]
    n = x32.shape[0]
    assert x32.shape == (200000, 256) and k == 4096
    torch = pytest.importorskip("torch")
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert _plan(n, 256, k, F.MIXED_FP8, 2, sms)["parts"] == 8
    assert _plan(n // 4, 256, k, F.MIXED_BF16, 3, sms)["parts"] == 16
    x64 = x32.astype(np.float64)
    c = w["init"].copy()
    second = 0
    for _ in range(2):
        gl, gc, gi, gs, rep = F.lloyd_step(x32, c, dtype="f32x64", precision="fp8")
        ol, oc, oi, os_ = O.lloyd_step(x64, c)
        assert np.array_equal(gl, ol)
        assert _close(gc, oc)
        assert abs(gi - oi) <= INERTIA_RTOL_MIXED * oi
        second += rep["rows_second_pass"]
        c = gc  # the GPU's own trajectory, which the fit below follows
    assert second > 0
    g = F.KMeans(k, dtype="f32x64").with_precision("fp8").with_max_iter(2).with_tol(0.0).with_n_init(1) \
        .with_init_centers(w["init"]).fit(x32)
    assert np.array_equal(g.cluster_centers(), gc) and g.n_iter() == 2
    xp = w["x_predict"]
    assert np.array_equal(g.predict(xp), O.predict(g.cluster_centers(), xp.astype(np.float64)))


def test_bf16_mask_pass_at_full_k_and_d_matches_fp64_oracle():
    # the BF16 form at k = 4096, d = 256 (200,000 rows of the bisector
    # workload): the main pass and the mask pass both run many centre slices,
    # so every slice writes its own words of a row's candidate mask; rows
    # equidistant from three centres of far-apart slices are in the mask
    # pass for sure; labels, centres and inertia against the FP64 oracle
    w = W.bisector_4096x256(scale=0.025, predict_scale=0.01)
    x32, k = w["x"].copy(), w["k"]
    n = x32.shape[0]
    torch = pytest.importorskip("torch")
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert _plan(n, 256, k, F.MIXED_BF16, 2, sms)["parts"] > 1
    c = w["init"]
    rng = np.random.default_rng(23)
    x32[:400] = _equidistant_rows(c, [7, 2100, 4090], 400, rng).astype(np.float32)
    x32[400:460] = _equidistant_rows(c, [300, 1300, 2300, 3300, 4000, 4095], 60, rng).astype(np.float32)
    gl, gc, gi, gs, rep = F.lloyd_step(x32, c, dtype="f32x64", precision="bf16")
    ol, oc, oi, os_ = O.lloyd_step(x32.astype(np.float64), c)
    assert np.array_equal(gl, ol)
    assert _close(gc, oc)
    assert abs(gi - oi) <= INERTIA_RTOL_MIXED * oi
    assert rep["rows_second_pass"] >= 400


def test_bf16_count_pass_fit_matches_fp64_oracle_and_single_steps():
    # from the fourth iteration of a fit on, the BF16 main pass is the count
    # pass (thresholds carried from the previous iteration); the fit's labels,
    # centres and n_iter must be the FP64 oracle's, and its centres bit for
    # bit those of single steps, which always rank a top-2
    w = W.anisotropic_1024x128(scale=0.01)  # 40,000 rows, d = 128, k = 1024
    x32, k = w["x"].copy(), w["k"]
    rng = np.random.default_rng(24)
    x32[:300] = _equidistant_rows(w["init"], [3, 500, 1000], 300, rng).astype(np.float32)
    iters = 12
    g = F.KMeans(k, dtype="f32x64").with_precision("bf16").with_max_iter(iters).with_tol(0.0).with_n_init(1) \
        .with_init_centers(w["init"]).fit(x32)
    o = O.fit(x32.astype(np.float64), k, max_iter=iters, tol=0.0, n_init=1, init=w["init"][None])
    assert np.array_equal(g.labels(), o["labels"])
    assert _close(g.cluster_centers(), o["centers"])
    assert g.n_iter() == o["n_iter"] == iters
    assert g.report["count_iterations"] >= 3
    c = w["init"]
    for _ in range(iters):
        gl, c, gi, gs, rep = F.lloyd_step(x32, c, dtype="f32x64", precision="bf16")
    assert np.array_equal(g.cluster_centers(), c)


def test_fp8_count_pass_fit_matches_fp64_oracle_and_single_steps():
    # the FP8 form's count pass: E4M3 accumulators are the row's scores times
    # a power of two, so the marks and the carried floors scale exactly; the
    # fit must equal the FP64 oracle and the single (top-2) steps
    w = W.anisotropic_1024x128(scale=0.01)  # 40,000 rows, d = 128, k = 1024
    x32, k = w["x"], w["k"]
    iters = 10
    g = F.KMeans(k, dtype="f32x64").with_precision("fp8").with_max_iter(iters).with_tol(0.0).with_n_init(1) \
        .with_init_centers(w["init"]).fit(x32)
    o = O.fit(x32.astype(np.float64), k, max_iter=iters, tol=0.0, n_init=1, init=w["init"][None])
    assert np.array_equal(g.labels(), o["labels"])
    assert _close(g.cluster_centers(), o["centers"])
    assert g.n_iter() == o["n_iter"] == iters
    assert g.report["count_iterations"] >= 2
    c = w["init"]
    for _ in range(iters):
        gl, c, gi, gs, rep = F.lloyd_step(x32, c, dtype="f32x64", precision="fp8")
    assert np.array_equal(g.cluster_centers(), c)


def test_bf16_mask_pass_sends_wide_ties_to_the_exhaustive_rescore():
    # forty copies of one centre: a row near it has forty exactly tied
    # candidates, more than the mask pass re-scores (32), so it is re-scored
    # against every centre; six-way near-ties stay in the mask pass. Labels
    # are the FP64 oracle's (the lowest index among exact ties).
    rng = np.random.default_rng(21)
    d, k = 64, 300
    c = rng.uniform(-10, 10, size=(k, d))
    c[10:50] = c[10]
    c[[101, 102, 103, 104, 106, 107]] = c[101] + rng.normal(0, 0.5, size=(6, d))
    x = c[rng.integers(0, k, 6000)] + rng.normal(0, 1, size=(6000, d))
    x[:200] = c[10] + rng.normal(0, 1, size=(200, d))
    x[200:260] = _equidistant_rows(c, [101, 102, 103, 104, 106, 107], 60, rng)
    x32 = x.astype(np.float32)
    gl, gc, gi, gs, rep = F.lloyd_step(x32, c, dtype="f32x64", precision="bf16")
    ol, oc, oi, os_ = O.lloyd_step(x32.astype(np.float64), c)
    assert np.array_equal(gl, ol)
    assert _close(gc, oc)
    assert rep["rows_exhaustive"] >= 200


def test_bf16_rows_not_16_byte_aligned_match_the_oracle():
    # X on the device one float past a 16-byte boundary: every kernel that
    # reads the f32 rows in 16-byte pieces must take its one-float path
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(22)
    n, d, k = 20000, 64, 256
    c = rng.uniform(-5, 5, size=(k, d))
    x32 = (c[rng.integers(0, k, n)] + rng.normal(0, 2.0, size=(n, d))).astype(np.float32)
    buf = torch.empty(n * d + 1, dtype=torch.float32, device="cuda")
    xd = buf[1:].view(n, d)
    xd.copy_(torch.from_numpy(x32))
    assert xd.data_ptr() % 16 == 4
    x64 = x32.astype(np.float64)
    gl, gc, gi, gs, rep = F.lloyd_step(xd, c, dtype="f32x64", precision="bf16")
    ol, oc, oi, os_ = O.lloyd_step(x64, c)
    assert np.array_equal(gl, ol)
    assert _close(gc, oc)
    g = F.KMeans(k, dtype="f32x64").with_precision("bf16").with_max_iter(4).with_tol(0.0).with_n_init(1) \
        .with_init_centers(c).fit(xd)
    o = O.fit(x64, k, max_iter=4, tol=0.0, n_init=1, init=c[None])
    assert np.array_equal(g.labels(), o["labels"])
    assert _close(g.cluster_centers(), o["centers"])


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("scale", [1e-35, 1e-20, 1e15, 1e18])
def test_mixed_extreme_scales_fall_back_exactly(precision, scale):
    # scores that leave the f32 range of the keys (or underflow) must send the
    # rows to the exact re-score, never to a wrong label
    rng = np.random.default_rng(12)
    d, k = 16, 9
    cen = rng.uniform(-10, 10, size=(k, d))
    x = (cen[rng.integers(0, k, 3000)] + rng.normal(0, 1, size=(3000, d))) * scale
    x32 = x.astype(np.float32)
    x64 = x32.astype(np.float64)
    c = x64[rng.choice(3000, size=k, replace=False)].copy()
    for _ in range(2):
        gl, gc, gi, gs, rep = F.lloyd_step(x32, c, dtype="f32x64", precision=precision)
        ol, oc, oi, os_ = O.lloyd_step(x64, c)
        assert np.array_equal(gl, ol)
        assert _close(gc, oc)
        c = oc


def test_fit_into_device_outputs_matches_host_outputs():
    torch = pytest.importorskip("torch")
    w = W.anisotropic_1024x128(scale=0.002)
    x32, k = w["x"], w["k"]
    m = F.KMeans(k, dtype="f32x64").with_precision("bf16").with_max_iter(3).with_tol(0.0).with_n_init(1) \
        .with_init_centers(w["init"])
    host = m.fit(x32)
    c_out = torch.empty((k, x32.shape[1]), dtype=torch.float64, device="cuda")
    l_out = torch.empty(x32.shape[0], dtype=torch.int64, device="cuda")
    dev = m.fit(torch.from_numpy(x32).cuda(), out=(c_out, l_out))
    assert np.array_equal(c_out.cpu().numpy(), host.cluster_centers())
    assert np.array_equal(l_out.cpu().numpy(), host.labels())
    assert dev.n_iter() == host.n_iter() == 3
    assert np.array_equal(dev.predict(x32), host.predict(x32))


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("n,k", [(6001, 24), (20000, 5)])  # 6001: label buffers not 16-byte aligned
def test_incremental_exact_sums_equal_full_recompute(precision, n, k):
    # after its first iteration a fit adds and removes only the rows whose
    # label changed; tiny values (remainders below both grids, more than the
    # per-block list holds when k is small) take the 128-bit path both ways
    rng = np.random.default_rng(21 + k)
    d = 32
    cen = rng.uniform(-20, 20, size=(k, d))
    x = cen[rng.integers(0, k, n)] + rng.normal(0, 4, size=(n, d))  # overlapping blobs: many moves
    x[:, 3] = rng.normal(0, 1e-6, n)
    x[::7, 5] *= 1e-7
    x32 = x.astype(np.float32)
    init = x32[rng.choice(n, k, replace=False)].astype(np.float64)
    iters = 12
    g = F.KMeans(k, dtype="f32x64").with_precision(precision).with_max_iter(iters).with_tol(0.0).with_n_init(1) \
        .with_init_centers(init).fit(x32)
    c = init
    for _ in range(iters):
        gl, c_next, gi, gs, rep = F.lloyd_step(x32, c, dtype="f32x64", precision=precision)
        c = c_next
    assert np.array_equal(g.cluster_centers(), c)
    assert np.array_equal(g.labels(), gl)
    assert abs(g.inertia() - gi) <= INERTIA_RTOL_MIXED * gi


@pytest.mark.parametrize("precision", PRECISIONS)
def test_incremental_fit_with_tolerance_and_runs_matches_oracle(precision):
    # n_init runs, each converging at its own iteration (the queued successor
    # of the converged iteration is discarded), against the FP64 oracle
    rng = np.random.default_rng(8)
    n, d, k = 8000, 16, 12
    cen = rng.uniform(-10, 10, size=(k, d))
    x32 = (cen[rng.integers(0, k, n)] + rng.normal(0, 2, size=(n, d))).astype(np.float32)
    inits = np.stack([x32[rng.choice(n, k, replace=False)] for _ in range(3)]).astype(np.float64)
    g = F.KMeans(k, dtype="f32x64").with_precision(precision).with_max_iter(60).with_tol(1e-3).with_n_init(3) \
        .with_init_centers(inits).fit(x32)
    o = O.fit(x32.astype(np.float64), k, max_iter=60, tol=1e-3, n_init=3, init=inits)
    assert np.array_equal(g.labels(), o["labels"])
    assert _close(g.cluster_centers(), o["centers"])
    assert g.n_iter() == o["n_iter"]
    assert abs(g.inertia() - o["inertia"]) <= INERTIA_RTOL_MIXED * o["inertia"]


@pytest.mark.parametrize("precision", PRECISIONS)
def test_mixed_fit_reference_edge_cases(precision):
    # the reference's known answers (kmeans.rs:784-860) on the mixed forms:
    # k = n from the rows themselves, identical rows, a single row
    rng = np.random.default_rng(31)
    x1 = rng.normal(size=(50, 8)).astype(np.float32)
    g = F.KMeans(50, dtype="f32x64").with_precision(precision).with_n_init(1) \
        .with_init_centers(x1.astype(np.float64)[None]).fit(x1)
    assert g.inertia() == 0.0
    assert np.array_equal(g.labels(), np.arange(50))
    same = np.ones((20, 4), dtype=np.float32)
    g = F.KMeans(3, dtype="f32x64").with_precision(precision).with_n_init(2).with_random_state(5).fit(same)
    assert g.inertia() == 0.0
    assert not g.labels().any()
    g = F.KMeans(1, dtype="f32x64").with_precision(precision).with_n_init(1).fit(x1[:1])
    assert g.labels().tolist() == [0] and g.inertia() == 0.0
    assert np.array_equal(g.cluster_centers(), x1[:1].astype(np.float64))

"""C-ABI checks that need no GPU: the library builds and loads, exports every
symbol include/ferrokmeans.h declares, maps argument errors onto the
FerroError variants in the reference's validation order (kmeans.rs:421-449,
542-548, 572-578), and its host-side uniform stream equals the oracle's."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import ferrolearn_gb300 as F
from ferrolearn_gb300 import _native
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            text = open(os.path.join(ROOT, "include", name)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            syms |= set(re.findall(r"\b(fk_[a-z0-9_]+)\s*\(", text))
    return syms


def test_library_exports_every_declared_symbol():
    lib = _native.lib()
    syms = _header_symbols()
    assert len(syms) >= 19
    missing = [s for s in sorted(syms) if not hasattr(lib, s)]
    assert not missing, missing
    assert set(_native.EXPORTS) <= syms


def test_version_and_defaults():
    lib = _native.lib()
    assert b"sm_103a" in lib.fk_version()
    p = _native.KMeansParams()
    lib.fk_kmeans_params_default(C.byref(p), 7)
    # KMeans::new defaults, kmeans.rs:76-84
    assert (p.n_clusters, p.max_iter, p.tol, p.n_init, p.has_random_state) == (7, 300, 1e-4, 10, 0)


def test_draw_stream_matches_oracle():
    assert np.array_equal(F.draws(123, 1000), O.draws(123, 1000))
    u = F.draws(0, 10000)
    assert (u >= 0).all() and (u < 1).all()


@pytest.mark.parametrize("k,x,exc", [
    (0, np.ones((3, 2)), F.InvalidParameter),              # kmeans.rs:421-426
    (3, np.zeros((0, 2)), F.InsufficientSamples),          # kmeans.rs:428-434
    (5, np.ones((2, 2)), F.InsufficientSamples),           # kmeans.rs:436-442
])
def test_fit_validation_errors(k, x, exc):
    for dtype in ("f64", "f32", "f32x64"):
        with pytest.raises(exc):
            F.KMeans(k, dtype=dtype).fit(x)


def test_fit_n_init_zero():
    with pytest.raises(F.InvalidParameter):  # kmeans.rs:444-449
        F.KMeans(2).with_n_init(0).fit(np.ones((4, 2)))


def test_zero_clusters_checked_before_samples():
    # n_clusters is validated first even when the data is also empty.
    with pytest.raises(F.InvalidParameter):
        F.KMeans(0).fit(np.zeros((0, 2)))


def test_predict_transform_shape_mismatch():
    fitted = F.FittedKMeans(np.ones((2, 2)), np.zeros(4, dtype=np.int64), 0.0, 1, "f64")
    with pytest.raises(F.ShapeMismatch):
        fitted.predict(np.ones((2, 3)))
    with pytest.raises(F.ShapeMismatch):
        fitted.transform(np.ones((2, 3)))


def test_mixed_precision_rejected_for_f32_semantics():
    with pytest.raises(F.Unsupported):
        F.KMeans(2, dtype="f32").with_precision("bf16").fit(np.ones((4, 2), dtype=np.float32))


@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_fp8_needs_f32_storage_with_f64_semantics(dtype):
    x = np.ones((4, 2), dtype=np.float32 if dtype == "f32" else np.float64)
    with pytest.raises(F.Unsupported):
        F.KMeans(2, dtype=dtype).with_precision("fp8").fit(x)
    with pytest.raises(F.Unsupported):
        F.lloyd_step(x, np.ones((2, 2)), dtype=dtype, precision="fp8")


def test_unknown_precision_code_rejected():
    with pytest.raises(F.Unsupported):
        F.KMeans(2, dtype="f32x64").with_precision(3).fit(np.ones((4, 2), dtype=np.float32))


def _bp(n=10, d=2, k=2, **kw):
    p = dict(x=np.ones((n, d), dtype=np.float32), k=k, n_init=2)
    p.update(kw)
    return p


@pytest.mark.parametrize("prob,exc,needle", [
    (_bp(k=0), F.InvalidParameter, "problem 1: Invalid parameter `n_clusters`"),
    (_bp(n=3, k=5), F.InsufficientSamples, "problem 1: Insufficient samples"),
    (_bp(n_init=0), F.InvalidParameter, "problem 1: Invalid parameter `n_init`"),
    (_bp(n=2000, d=64, k=1000), F.Unsupported, "k*d <= 32768"),
])
def test_batched_validation_names_the_problem(prob, exc, needle):
    with pytest.raises(exc) as e:
        F.fit_batched([_bp(), prob])
    assert needle in str(e.value)


def test_batched_empty_and_bad_reduction():
    fitted, rep = F.fit_batched([])
    assert fitted == [] and rep["fits"] == 0
    with pytest.raises(F.InvalidParameter):
        F.fit_batched([_bp()], reduction=7)


def _plan(n, d, k, precision, topk, sms=152):
    import ctypes as C
    out = (C.c_int64 * 10)()
    st = _native.lib().fk_debug_tc_plan(n, d, k, precision, topk, sms, out)
    return st, dict(zip(["d_pad", "kp", "parts", "k_pad", "nblocks", "xst", "smem", "grid", "ctas", "tiles"], out))


def test_tensor_core_plans_of_the_workloads():
    # host-only planning of the resident-slice kernel: the shapes the bench
    # workloads run (a plan that loses resident centres slows every launch)
    st, p = _plan(4_000_000, 128, 1024, F.MIXED_BF16, 2)
    assert st == 0 and (p["d_pad"], p["kp"], p["parts"], p["xst"], p["nblocks"]) == (128, 512, 2, 2, 2)
    assert p["grid"] == 152 and p["tiles"] == 31250 and p["smem"] <= 227 * 1024
    st, p = _plan(8_000_000, 256, 4096, F.MIXED_FP8, 2)
    assert st == 0 and (p["d_pad"], p["kp"], p["parts"], p["xst"]) == (256, 512, 8, 2)
    assert p["grid"] == 152 and p["smem"] <= 227 * 1024
    st, p = _plan(2_000_000, 256, 4096, F.MIXED_BF16, 3)  # the second pass of the FP8 form (count pass): BF16
    # rows of 512 bytes leave room for one X stage and 256 resident centres
    assert st == 0 and (p["kp"], p["parts"], p["xst"], p["grid"]) == (256, 16, 1, 144) and p["smem"] <= 227 * 1024
    st, p = _plan(2_000_000, 256, 4096, F.MIXED_FP8, 3)  # the FP8 count pass: the FP8 top-2 pass's slices
    assert st == 0 and (p["kp"], p["parts"], p["xst"]) == (512, 8, 2) and p["smem"] <= 227 * 1024
    for topk in (1, 3):  # the BF16 mask and count passes fit the main pass's slices at cfg3
        st, p = _plan(100_000, 128, 1024, F.MIXED_BF16, topk)
        assert st == 0 and (p["kp"], p["xst"]) == (512, 2)
    # small shapes: one padded slice, grid no larger than the tiles
    st, p = _plan(1, 1, 1, F.MIXED_BF16, 2)
    assert st == 0 and (p["d_pad"], p["kp"], p["parts"], p["k_pad"], p["grid"], p["tiles"]) == (64, 256, 1, 256, 1, 1)


def test_tensor_core_plan_rejects_what_the_kernel_cannot_hold():
    st, _ = _plan(1000, 512, 64, F.MIXED_BF16, 2)  # d beyond the resident-slice kernel's BF16 limit
    assert st == 13  # FK_ERR_UNSUPPORTED
    assert "supports d <=" in _native.last_error()
    st, _ = _plan(1000, 64, 64, 0, 2)  # the plain precision has no tensor-core plan
    assert st != 0


def test_out_of_range_arguments_are_refused_before_any_device_work():
    # every entry point checks the ranges its kernels index (int32 labels,
    # 32-bit feature and cluster indices) before CUDA is touched: the
    # pointers below are never read
    lib = _native.lib()
    ctx = C.c_void_p()
    assert lib.fk_ctx_create(C.byref(ctx), 0, None) == 0
    buf = np.zeros(64)
    p = buf.ctypes.data
    big_n, big_d, big_k = 2**31, 2**16 + 1, 2**20 + 1
    try:
        assert lib.fk_kmeans_predict_f64(ctx, p, 2, 2, p, big_n, 2, 0, p) == 13
        assert lib.fk_kmeans_predict_f32(ctx, p, big_k, 2, p, 4, 2, 0, p) == 13
        assert lib.fk_kmeans_predict_f64(ctx, p, 2, -1, p, 4, -1, 0, p) == 1
        assert lib.fk_kmeans_transform_f64(ctx, p, big_k, 2, p, 4, 2, p) == 13
        assert lib.fk_kmeans_transform_f32(ctx, p, 2, big_d, p, 4, big_d, p) == 13
        assert lib.fk_kmeans_plus_plus_f64(ctx, p, 4, 2, 2, p, -1, 0, p, None) == 1
        assert "n_draws" in _native.last_error()
        assert lib.fk_kmeans_plus_plus_f32(ctx, p, 4, big_d, 2, None, 0, 0, p, None) == 13
        rep = _native.FitReport()
        assert lib.fk_lloyd_step_f64(ctx, p, big_n, 2, p, 2, 0, p, p, p, p, C.byref(rep)) == 13
        assert lib.fk_lloyd_step_f32x64(ctx, p, 4, -2, p, 2, 1, p, p, p, p, None) == 1
        params = _native.KMeansParams()
        lib.fk_kmeans_params_default(C.byref(params), 2)
        params.draws = p
        params.n_draws = -1
        assert lib.fk_kmeans_fit_f64(ctx, p, 4, 2, C.byref(params), None, p, p, p, p, None) == 1
        assert "n_draws" in _native.last_error()
        params.n_draws = 8
        assert lib.fk_kmeans_fit_f64(ctx, p, big_n, 2, C.byref(params), None, p, p, p, p, None) == 13
        assert "supported range" in _native.last_error()
    finally:
        lib.fk_ctx_destroy(ctx)


def test_tensors_and_output_buffers_are_checked_before_the_call():
    # a tensor is used as raw memory: a wrong dtype, shape or layout would make
    # the kernels read or write past it, so the host layer refuses it first
    torch = pytest.importorskip("torch")
    x32 = torch.ones((8, 4), dtype=torch.float32)
    with pytest.raises(F.InvalidParameter, match="torch.float64"):
        F.KMeans(2, dtype="f64").fit(x32)  # f64 entry point reads 8-byte values
    with pytest.raises(F.InvalidParameter, match="contiguous"):
        F.KMeans(2, dtype="f32").fit(torch.ones((4, 8), dtype=torch.float32).t())
    with pytest.raises(F.ShapeMismatch):
        F.KMeans(2, dtype="f32").fit(torch.ones(8, dtype=torch.float32))
    m = F.KMeans(2, dtype="f32x64").with_n_init(1)
    with pytest.raises(F.ShapeMismatch, match="centres out"):
        m.fit(x32, out=(torch.empty((3, 4), dtype=torch.float64), torch.empty(8, dtype=torch.int64)))
    with pytest.raises(F.InvalidParameter, match="centres out"):
        m.fit(x32, out=(torch.empty((2, 4), dtype=torch.float32), torch.empty(8, dtype=torch.int64)))
    with pytest.raises(F.ShapeMismatch, match="labels out"):
        m.fit(x32, out=(torch.empty((2, 4), dtype=torch.float64), torch.empty(7, dtype=torch.int64)))
    with pytest.raises(F.InvalidParameter, match="labels out"):
        m.fit(x32, out=(np.empty((2, 4)), np.empty(8, dtype=np.int32)))
    with pytest.raises(F.InvalidParameter, match="writeable"):
        ro = np.empty((2, 4))
        ro.flags.writeable = False
        m.fit(x32, out=(ro, np.empty(8, dtype=np.uint64)))
    with pytest.raises(F.InvalidParameter):
        F.lloyd_step(torch.ones((8, 4), dtype=torch.float64), np.ones((2, 4)), dtype="f32")
    with pytest.raises(F.InvalidParameter):
        F.fit_batched([dict(x=torch.ones((8, 4), dtype=torch.float64), k=2)])
    with pytest.raises(F.InvalidParameter):
        F.kmeans_plus_plus(torch.ones((8, 4), dtype=torch.float32), 2, dtype="f64")
    fitted = F.FittedKMeans(np.ones((2, 4)), np.zeros(8, dtype=np.int64), 0.0, 1, "f64")
    with pytest.raises(F.InvalidParameter):
        fitted.predict(x32)
    with pytest.raises(F.InvalidParameter):
        fitted.transform(x32)

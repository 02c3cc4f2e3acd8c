"""Host-side mirror of ferrolearn-cluster's KMeans API over the C ABI.

Mirrors ferrolearn-cluster/src/kmeans.rs:
  KMeans<F>            builder (kmeans.rs:55-113): new / with_max_iter /
                       with_tol / with_n_init / with_random_state
  Fit::fit             kmeans.rs:417-512 -> FittedKMeans
  FittedKMeans<F>      getters cluster_centers / labels / inertia / n_iter
                       (kmeans.rs:121-156)
  Predict::predict     kmeans.rs:538-552
  Transform::transform kmeans.rs:568-617
  fit_predict          kmeans.rs:522-525
and FerroError (ferrolearn-core/src/error.rs:30-91) as exceptions.

Two builder methods have no reference counterpart: with_init_centers (the
reference always seeds with k-means++ from rand's StdRng, which cannot be
reproduced here, so parity runs inject the initial centres) and
with_precision (the mixed BF16 / FP8 tensor-core contractions with exact
re-check).

F is chosen with dtype: "f64" (KMeans<f64>), "f32" (KMeans<f32>) or
"f32x64" (KMeans<f64> semantics on X stored as f32, each value widened
exactly; the entry point of the mixed precisions).
"""
import atexit
import ctypes as C
import threading
import weakref

import numpy as np

from . import _native

PLAIN = 0
MIXED_BF16 = 1
MIXED_FP8 = 2

_PREC_NAMES = {"plain": PLAIN, "bf16": MIXED_BF16, "mixed_bf16": MIXED_BF16, "fp8": MIXED_FP8,
               "mixed_fp8": MIXED_FP8}


class FerroError(Exception):
    """Base of the errors returned by the library (FerroError)."""

    code = -1


class InvalidParameter(FerroError, ValueError):
    code = 1


class InsufficientSamples(FerroError, ValueError):
    code = 2


class ShapeMismatch(FerroError, ValueError):
    code = 3


class NumericalInstability(FerroError):
    code = 4


class CudaError(FerroError, RuntimeError):
    code = 10


class DeviceOutOfMemory(CudaError):
    code = 11


class DeviceTimeout(CudaError):
    code = 12


class Unsupported(FerroError, NotImplementedError):
    code = 13


class NullPointer(FerroError, ValueError):
    code = 14


_BY_CODE = {c.code: c for c in (InvalidParameter, InsufficientSamples, ShapeMismatch, NumericalInstability,
                                CudaError, DeviceOutOfMemory, DeviceTimeout, Unsupported, NullPointer)}


def _check(status):
    if status != 0:
        cls = _BY_CODE.get(status, FerroError)
        raise cls(_native.last_error() or f"status {status}")


def _ptr(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):  # torch tensor on the device (or host)
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(C.c_void_p)


class Context:
    """A GPU + CUDA stream binding (fk_ctx). stream: a cudaStream_t as int, or None."""

    def __init__(self, device=0, stream=None):
        self._lib = _native.lib()
        h = C.c_void_p()
        _check(self._lib.fk_ctx_create(C.byref(h), int(device), C.c_void_p(stream) if stream else None))
        self.handle = h
        self.device = device
        _live.add(self)

    def close(self):
        if self.handle:
            self._lib.fk_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# Contexts still open at interpreter exit are closed by an exit handler, while
# the CUDA runtime and the streams they use are intact (a context released
# later, during module teardown, would free device memory in arbitrary order).
_live = weakref.WeakSet()


@atexit.register
def _close_live_contexts():
    for ctx in list(_live):
        try:
            ctx.close()
        except Exception:
            pass


_tls = threading.local()


def default_context(device=0):
    ctxs = getattr(_tls, "ctxs", None)
    if ctxs is None:
        ctxs = _tls.ctxs = {}
    if device not in ctxs:
        ctxs[device] = Context(device)
    return ctxs[device]


def _dtypes(kind):
    if kind == "f64":
        return np.float64, np.float64, "f64"
    if kind == "f32":
        return np.float32, np.float32, "f32"
    if kind == "f32x64":
        return np.float32, np.float64, "f32x64"
    raise ValueError(f"dtype must be 'f64', 'f32' or 'f32x64', got {kind!r}")


def _prec(p):
    if isinstance(p, str):
        return _PREC_NAMES[p.lower()]
    return int(p)


_TORCH_NAMES = {np.dtype(np.float32): ("torch.float32",), np.dtype(np.float64): ("torch.float64",),
                np.dtype(np.uint64): ("torch.int64", "torch.uint64")}


def _check_tensor(t, dt, what, ctx, shape=None, ndim=None):
    """A torch tensor is handed to the library as raw memory, so its dtype,
    shape and layout must be exactly what the entry point reads or writes,
    and a device tensor must live on the context's GPU (the kernels use it in
    place). Labels are written as uint64; int64 tensors hold the same bits."""
    names = _TORCH_NAMES[np.dtype(dt)]
    if str(t.dtype) not in names:
        raise InvalidParameter(f"{what}: a {t.dtype} tensor where {' or '.join(names)} is expected")
    if ndim is not None and t.dim() != ndim:
        raise ShapeMismatch(f"{what}: expected a {ndim}-D tensor, got shape {tuple(t.shape)}")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ShapeMismatch(f"{what}: expected shape {tuple(shape)}, got {tuple(t.shape)}")
    if not t.is_contiguous():
        raise InvalidParameter(f"{what}: the tensor must be contiguous (row-major)")
    dev = t.device
    if dev.type == "cuda":
        if ctx is not None and dev.index != int(ctx.device):
            raise InvalidParameter(f"{what}: tensor on cuda:{dev.index}, context on cuda:{ctx.device}")
    elif dev.type != "cpu":
        raise InvalidParameter(f"{what}: tensors on {dev.type} are not supported")
    return t


def _as_matrix(x, dt, ctx=None):
    if hasattr(x, "data_ptr"):
        return _check_tensor(x, dt, "x", ctx, ndim=2)
    a = np.ascontiguousarray(x, dtype=dt)
    if a.ndim != 2:
        raise ShapeMismatch(f"expected a 2-D array, got shape {a.shape}")
    return a


def _check_out(a, dt, shape, what, ctx):
    """An output buffer the library writes in place (numpy array or tensor)."""
    if hasattr(a, "data_ptr"):
        return _check_tensor(a, dt, what, ctx, shape=shape)
    if not isinstance(a, np.ndarray):
        raise InvalidParameter(f"{what}: expected a numpy array or a tensor")
    ok = (a.dtype == np.dtype(dt)) or (dt == np.uint64 and a.dtype == np.int64)
    if not ok:
        raise InvalidParameter(f"{what}: dtype {a.dtype} where {np.dtype(dt)} is written")
    if a.shape != tuple(shape):
        raise ShapeMismatch(f"{what}: expected shape {tuple(shape)}, got {a.shape}")
    if not (a.flags.c_contiguous and a.flags.writeable):
        raise InvalidParameter(f"{what}: the array must be C-contiguous and writeable")
    return a


def draws(seed, count):
    """The library's uniform stream (splitmix64), as consumed by k-means++."""
    out = np.empty(count, dtype=np.float64)
    _check(_native.lib().fk_draws_f64(seed, count, _ptr(out)))
    return out


class KMeans:
    """KMeans<F> configuration (unfitted); kmeans.rs:55-113."""

    def __init__(self, n_clusters, dtype="f64"):
        self.n_clusters = int(n_clusters)
        self.max_iter = 300
        self.tol = 1e-4
        self.n_init = 10
        self.random_state = None
        self.dtype = dtype
        self.precision = PLAIN
        self.init_centers = None
        self.draws = None
        self.collect_timing = False
        _dtypes(dtype)

    @classmethod
    def new(cls, n_clusters, dtype="f64"):
        return cls(n_clusters, dtype)

    def with_max_iter(self, max_iter):
        self.max_iter = int(max_iter)
        return self

    def with_tol(self, tol):
        self.tol = float(tol)
        return self

    def with_n_init(self, n_init):
        self.n_init = int(n_init)
        return self

    def with_random_state(self, seed):
        self.random_state = int(seed)
        return self

    def with_init_centers(self, centers):
        """Explicit initial centres: (k, d) for every run, or (n_init, k, d)."""
        self.init_centers = centers
        return self

    def with_draws(self, uniform_stream):
        """Uniform [0,1) stream for k-means++ in place of the seeded generator."""
        self.draws = np.ascontiguousarray(uniform_stream, dtype=np.float64)
        return self

    def with_precision(self, precision):
        self.precision = _prec(precision)
        return self

    def with_timing(self, on=True):
        self.collect_timing = bool(on)
        return self

    def _params(self):
        p = _native.KMeansParams()
        _native.lib().fk_kmeans_params_default(C.byref(p), self.n_clusters)
        p.max_iter = self.max_iter
        p.tol = self.tol
        p.n_init = self.n_init
        if self.random_state is not None:
            p.random_state = self.random_state
            p.has_random_state = 1
        p.precision = self.precision
        if self.draws is not None:
            p.draws = self.draws.ctypes.data
            p.n_draws = self.draws.size
        p.collect_timing = 1 if self.collect_timing else 0
        return p

    def fit(self, x, y=None, ctx=None, out=None):
        """Fit::fit (kmeans.rs:417-512). out: optional (centres, labels) device
        tensors (k x d of the centre dtype, n of int64) that receive the
        results in place of new host arrays."""
        xt, ct, suf = _dtypes(self.dtype)
        ctx = ctx or default_context()
        x = _as_matrix(x, xt, ctx)
        n, d = int(x.shape[0]), int(x.shape[1])
        k = self.n_clusters
        init = None
        if self.init_centers is not None:
            ini = np.asarray(self.init_centers, dtype=ct)
            if ini.ndim == 2:
                ini = np.broadcast_to(ini, (max(self.n_init, 1),) + ini.shape)
            ini = np.ascontiguousarray(ini)
            if ini.shape[1:] != (k, d) or ini.shape[0] < max(self.n_init, 1):
                raise ShapeMismatch(f"init centres shape {ini.shape} does not match (n_init, {k}, {d})")
            init = ini
        if out is not None:
            centers, labels = out
            _check_out(centers, ct, (max(k, 0), d), "centres out", ctx)
            _check_out(labels, np.uint64, (n,), "labels out", ctx)
        else:
            centers = np.empty((max(k, 0), d), dtype=ct)
            labels = np.empty(n, dtype=np.uint64)
        inertia = (C.c_double if ct == np.float64 else C.c_float)()
        n_iter = C.c_int64()
        rep = _native.FitReport()
        params = self._params()
        fn = getattr(_native.lib(), f"fk_kmeans_fit_{suf}")
        _check(fn(ctx.handle, _ptr(x), n, d, C.byref(params), _ptr(init), _ptr(centers), _ptr(labels),
                  C.byref(inertia), C.byref(n_iter), C.byref(rep)))
        lab = labels if out is not None else labels.view(np.int64)  # labels < 2^63: the same bits, no copy
        return FittedKMeans(centers, lab, inertia.value, n_iter.value, self.dtype, rep.as_dict(), self.precision)

    def fit_predict(self, x, ctx=None):
        """kmeans.rs:522-525: fit, then predict on the same rows."""
        return self.fit(x, ctx=ctx).predict(x, ctx=ctx)


class FittedKMeans:
    """FittedKMeans<F> (kmeans.rs:121-156)."""

    def __init__(self, centers, labels, inertia, n_iter, dtype, report=None, precision=PLAIN):
        self._centers = centers
        self._labels = labels
        self._inertia = inertia
        self._n_iter = n_iter
        self.dtype = dtype
        self.report = report or {}
        self.precision = precision

    def cluster_centers(self):
        return self._centers

    def labels(self):
        return self._labels

    def inertia(self):
        return self._inertia

    def n_iter(self):
        return self._n_iter

    def predict(self, x, ctx=None, precision=None):
        """Predict::predict (kmeans.rs:538-552)."""
        xt, ct, suf = _dtypes(self.dtype)
        ctx = ctx or default_context()
        x = _as_matrix(x, xt, ctx)
        n, d = int(x.shape[0]), int(x.shape[1])
        labels = np.empty(n, dtype=np.uint64)
        prec = self.precision if precision is None else _prec(precision)
        fn = getattr(_native.lib(), f"fk_kmeans_predict_{suf}")
        _check(fn(ctx.handle, _ptr(self._centers), self._centers.shape[0], self._centers.shape[1], _ptr(x), n, d,
                  prec, _ptr(labels)))
        return labels.view(np.int64)

    def transform(self, x, ctx=None):
        """Transform::transform (kmeans.rs:568-617)."""
        xt, ct, suf = _dtypes(self.dtype)
        if suf == "f32x64":
            xt, suf = np.float64, "f64"
        ctx = ctx or default_context()
        x = _as_matrix(x, xt, ctx)
        n, d = int(x.shape[0]), int(x.shape[1])
        k = self._centers.shape[0]
        out = np.empty((n, k), dtype=ct)
        fn = getattr(_native.lib(), f"fk_kmeans_transform_{suf}")
        _check(fn(ctx.handle, _ptr(self._centers), k, self._centers.shape[1], _ptr(x), n, d, _ptr(out)))
        return out


def lloyd_step(x, centers, dtype="f64", precision=PLAIN, ctx=None):
    """One Lloyd iteration (kmeans.rs:468-488): (labels, new_centers, inertia, max_shift, report)."""
    xt, ct, suf = _dtypes(dtype)
    ctx = ctx or default_context()
    x = _as_matrix(x, xt, ctx)
    c = np.ascontiguousarray(centers, dtype=ct)
    n, d = x.shape
    k = c.shape[0]
    labels = np.empty(n, dtype=np.uint64)
    nc = np.empty_like(c)
    T = C.c_double if ct == np.float64 else C.c_float
    inertia, shift = T(), T()
    rep = _native.FitReport()
    fn = getattr(_native.lib(), f"fk_lloyd_step_{suf}")
    _check(fn(ctx.handle, _ptr(x), n, d, _ptr(c), k, _prec(precision), _ptr(labels), _ptr(nc), C.byref(inertia),
              C.byref(shift), C.byref(rep)))
    return labels.view(np.int64), nc, inertia.value, shift.value, rep.as_dict()


def kmeans_plus_plus(x, k, draws_arr=None, seed=0, dtype="f64", ctx=None):
    """kmeans_plus_plus (kmeans.rs:169-253) on the GPU -> (centers, draws consumed)."""
    xt, ct, suf = _dtypes(dtype)
    if suf == "f32x64":
        raise Unsupported("k-means++ runs on f64 or f32 matrices")
    ctx = ctx or default_context()
    x = _as_matrix(x, xt, ctx)
    n, d = x.shape
    out = np.empty((max(int(k), 0), d), dtype=ct)
    used = C.c_int64()
    dr = None if draws_arr is None else np.ascontiguousarray(draws_arr, dtype=np.float64)
    fn = getattr(_native.lib(), f"fk_kmeans_plus_plus_{suf}")
    _check(fn(ctx.handle, _ptr(x), n, d, k, _ptr(dr), 0 if dr is None else dr.size, seed, _ptr(out),
              C.byref(used)))
    return out, used.value


REDUCE_REFERENCE = 0
REDUCE_F64 = 1
_REDUCTIONS = {"reference": REDUCE_REFERENCE, "f32": REDUCE_REFERENCE, "f64": REDUCE_F64}

_BUCKET_D = (8, 16, 32, 64, "other")
_BUCKET_K = ("<=16", "<=32", "<=64", ">64")
_VARIANTS = ("1 row x 1 centre", "2 rows x 1 centre", "1 row x 2 centres", "2 rows x 2 centres",
             "4 rows x 1 centre")


def fit_batched(problems, reduction="reference", ctx=None):
    """Many independent KMeans<f32> fits in one call (fk_kmeans_fit_batched_f32).

    problems: a list of dicts with x (n x d f32, numpy or a device tensor), k,
    and optionally n_init (10), max_iter (300), tol (1e-4), random_state (0),
    init ((n_init, k, d) or (k, d) initial centres). Each problem is
    Fit::fit (kmeans.rs:417-512) with F = f32; run r draws k-means++ from the
    stream seeded with random_state + r. reduction: "reference" (f32 row-order
    centroid sums, bit-identical to KMeans<f32>) or "f64" (each cluster sum
    formed exactly and rounded once to f64, the mean rounded once to f32).

    Returns (list of FittedKMeans, report dict with per-fit inertia / n_iter,
    the autotuner's tile choice per (d, k) bucket and phase times).
    """
    ctx = ctx or default_context()
    red = _REDUCTIONS[reduction] if isinstance(reduction, str) else int(reduction)
    n_probs = len(problems)
    arr = (_native.BatchProblem * max(1, n_probs))()
    keep, outs = [], []
    total_fits = 0
    for i, pr in enumerate(problems):
        x = _as_matrix(pr["x"], np.float32, ctx)
        n, d = int(x.shape[0]), int(x.shape[1])
        k = int(pr["k"])
        n_init = int(pr.get("n_init", 10))
        init = pr.get("init")
        if init is not None:
            ini = np.asarray(init, dtype=np.float32)
            if ini.ndim == 2:
                ini = np.broadcast_to(ini, (max(n_init, 1),) + ini.shape)
            init = np.ascontiguousarray(ini)
        c_out = np.empty((max(k, 0), d), dtype=np.float32)
        l_out = np.empty(n, dtype=np.uint64)
        in_out = np.empty(1, dtype=np.float32)
        it_out = np.empty(1, dtype=np.int64)
        br_out = np.empty(1, dtype=np.int64)
        q = arr[i]
        q.x = _ptr(x).value if hasattr(x, "data_ptr") else x.ctypes.data
        q.n, q.d, q.n_clusters = n, d, k
        q.max_iter = int(pr.get("max_iter", 300))
        q.tol = float(pr.get("tol", 1e-4))
        q.n_init = n_init
        q.random_state = int(pr.get("random_state", 0))
        q.init = None if init is None else init.ctypes.data
        q.centers_out = c_out.ctypes.data
        q.labels_out = l_out.ctypes.data
        q.inertia_out = in_out.ctypes.data
        q.n_iter_out = it_out.ctypes.data
        q.best_run_out = br_out.ctypes.data
        keep += [x, init]
        outs.append((c_out, l_out, in_out, it_out, br_out))
        total_fits += max(n_init, 0)
    fit_in = np.empty(max(1, total_fits), dtype=np.float64)
    fit_it = np.empty(max(1, total_fits), dtype=np.int64)
    rep = _native.BatchReport()
    rep.fit_inertia = fit_in.ctypes.data
    rep.fit_n_iter = fit_it.ctypes.data
    _check(_native.lib().fk_kmeans_fit_batched_f32(ctx.handle, arr, n_probs, red, C.byref(rep)))
    fitted = [FittedKMeans(c, l.astype(np.int64), float(inr[0]), int(it[0]), "f32",
                           {"best_run": int(br[0])}) for c, l, inr, it, br in outs]
    tiles = {}
    for b in range(20):
        v = rep.bucket_variant[b]
        if v >= 0:
            tiles[f"d={_BUCKET_D[b // 4]},k{_BUCKET_K[b % 4]}"] = _VARIANTS[v]
    report = dict(fits=rep.fits, iterations_total=rep.iterations_total, graph_launches=rep.graph_launches,
                  tuned_buckets=rep.tuned_buckets, tiles=tiles, ms_upload=rep.ms_upload, ms_init=rep.ms_init,
                  ms_tune=rep.ms_tune, ms_lloyd=rep.ms_lloyd, ms_download=rep.ms_download, ms_total=rep.ms_total,
                  fit_inertia=fit_in[:total_fits].copy(), fit_n_iter=fit_it[:total_fits].copy())
    return fitted, report

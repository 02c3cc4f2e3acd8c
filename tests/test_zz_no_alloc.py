"""The allocation-free scoring entry point, checked against the existing ones.

fk_kmeans_score_f64_noalloc is for callers that cannot allocate device memory
when they need a score (a serving loop that must not synchronise the device
through an allocation, a fixed memory budget, an allocator owned by another
framework). Its scratch is a fixed array inside the library, shared by every
call, so this test makes two calls in a row on the same stream -- the second
must not see anything left by the first -- and compares both with
fk_kmeans_predict_f64 (labels, exactly) and fk_lloyd_step_f64 (inertia, the
1e-12 relative tolerance the other f64 tests use). This file is collected
last so a failure here never hides the other tests' results.
"""
import ctypes as C

import numpy as np
import pytest

import ferrolearn_gb300 as F
from ferrolearn_gb300 import _native

pytestmark = pytest.mark.gpu

MAX_ROWS = 1 << 19


def _p(t):
    return C.c_void_p(t.data_ptr())


def test_score_noalloc_two_calls_match_existing_entry_points():
    torch = pytest.importorskip("torch")
    lib = _native.lib()
    rng = np.random.default_rng(123)
    n, d, k = 20000, 24, 37
    x = rng.normal(size=(n, d)) * 3.0 + rng.integers(0, 6, size=(n, 1)) * 4.0
    xd = torch.from_numpy(x).cuda()
    labels_d = torch.full((n,), -1, dtype=torch.int64, device="cuda")
    inertia_d = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    for call in range(2):
        c = x[rng.choice(n, k, replace=False)].copy()
        cd = torch.from_numpy(c).cuda()
        st = lib.fk_kmeans_score_f64_noalloc(_p(xd), n, d, _p(cd), k, _p(labels_d), _p(inertia_d),
                                             C.c_void_p(stream.cuda_stream))
        assert st == 0, _native.last_error()
        torch.cuda.synchronize()
        got_labels = labels_d.cpu().numpy()
        got_inertia = float(inertia_d.cpu().numpy()[0])
        fitted = F.FittedKMeans(c, np.zeros(n, dtype=np.int64), 0.0, 0, "f64")
        assert np.array_equal(got_labels, fitted.predict(x))
        step_labels, _, step_inertia, _, _ = F.lloyd_step(x, c, dtype="f64")
        assert np.array_equal(got_labels, step_labels)
        assert abs(got_inertia - step_inertia) <= 1e-12 * step_inertia


def test_score_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    lib = _native.lib()
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    st = lib.fk_kmeans_score_f64_noalloc(_p(buf), MAX_ROWS + 1, 1, _p(buf), 1, _p(buf), _p(buf), None)
    assert st == 1
    assert "524288" in _native.last_error()
    host = np.zeros(16)
    st = lib.fk_kmeans_score_f64_noalloc(host.ctypes.data_as(C.c_void_p), 4, 1, _p(buf), 1, _p(buf), _p(buf), None)
    assert st == 1
    assert "`x`" in _native.last_error()

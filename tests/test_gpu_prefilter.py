"""The plain f64 assignment through its FP32 prefilter (fk_prefilter.cu):
labels, centres and inertia must stay those of the FP64 direct form, bit for
bit, where the FP32 pass can decide a row and where it cannot -- values
outside the f32 range or below its normal range, exact and near ties, NaN
and infinite values."""
import numpy as np
import pytest

import ferrolearn_gb300 as F
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _step_equal(x, c):
    gl, gc, gi, gs, _ = F.lloyd_step(x, c)
    ol, oc, oi, os_ = O.lloyd_step(x, c)
    assert np.array_equal(gl, ol)
    assert np.array_equal(gc, oc, equal_nan=True)
    assert (gs == os_) or (np.isnan(gs) and np.isnan(os_))
    if np.isfinite(oi):
        assert abs(gi - oi) <= 1e-12 * abs(oi) + 1e-300
    else:
        assert gi == oi
    return gl


def test_prefilter_values_outside_the_f32_range():
    rng = np.random.default_rng(5)
    x = rng.normal(size=(3000, 12))
    c = rng.normal(size=(17, 12))
    x[:40] *= 1e39   # beyond f32: their f32 copies overflow, the rows go to FP64
    x[40:80] *= 1e-41  # f32 subnormals: large relative rounding errors
    c[3] *= 1e-41
    x[80, 5] = np.inf
    x[81, :] = np.nan
    x[82, 0] = -np.inf
    assert np.array_equal(F.FittedKMeans(c, np.zeros(3000, dtype=np.int64), 0.0, 0, "f64").predict(x),
                          O.predict(c, x))
    _step_equal(x, c)


def test_prefilter_exact_and_near_ties():
    rng = np.random.default_rng(9)
    d = 24
    c = rng.normal(size=(40, d)) * 5
    c[7] = c[21]  # duplicate centres: the lower index wins
    c[30] = c[2]
    x = c[rng.integers(0, 40, 4000)] + rng.normal(size=(4000, d))
    # rows exactly between two centres (the midpoint of 1 and 11, of 5 and 6)
    x[:200] = 0.5 * (c[1] + c[11])
    x[200:400] = 0.5 * (c[5] + c[6])
    # rows a hair off the midpoint
    x[400:600] = 0.5 * (c[3] + c[4]) + 1e-13 * rng.normal(size=(200, d))
    # rows equal to centres
    x[600:700] = c[rng.integers(0, 40, 100)]
    assert np.array_equal(F.FittedKMeans(c, np.zeros(4000, dtype=np.int64), 0.0, 0, "f64").predict(x),
                          O.predict(c, x))
    _step_equal(x, c)


def test_prefilter_dirichlet_shape_steps_and_fit():
    # the plain f64 form at 200,000 rows of the d = 64, k = 256 workload
    from ferrolearn_gb300 import workloads as W
    w = W.dirichlet_256x64(scale=0.2)
    x, k = w["x"], w["k"]
    c = x[np.random.default_rng(2).permutation(x.shape[0])[:k]].copy()
    for _ in range(3):
        gl = _step_equal(x, c)
        c = O.lloyd_step(x, c)[1]
    g = F.KMeans(k).with_init_centers(c).with_max_iter(12).with_tol(0.0).with_n_init(1).fit(x)
    o = O.fit(x, k, max_iter=12, tol=0.0, n_init=1, init=c[None])
    assert np.array_equal(g.labels(), o["labels"])
    assert np.array_equal(g.cluster_centers(), o["centers"])
    assert abs(g.inertia() - o["inertia"]) <= 1e-12 * o["inertia"]
    assert gl.shape[0] == x.shape[0]

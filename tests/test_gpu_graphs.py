"""CUDA-graph replay of a fit's steady-state iterations.

Without phase timers, a fit captures each steady-state iteration (from the
third on) once per key -- the centre and label buffers it rotates through,
its update mode, the main pass kind -- and replays the graph from then on,
within the call and in later calls on the same context. The results must be
those of the same fit run launch by launch (with phase timers), and of the
FP64 / f32 oracle.
"""
import numpy as np
import pytest

import ferrolearn_gb300 as F
from ferrolearn_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert np.array_equal(a.cluster_centers(), b.cluster_centers())
    assert np.array_equal(a.labels(), b.labels())
    assert a.inertia() == b.inertia() and a.n_iter() == b.n_iter()


@pytest.mark.parametrize("dtype,precision", [("f64", "plain"), ("f32", "plain"), ("f32x64", "bf16"),
                                             ("f32x64", "fp8")])
def test_graph_replayed_fits_equal_the_launch_by_launch_fit(dtype, precision):
    if precision == "plain":
        w = W.dirichlet_256x64(scale=0.02, dtype=np.float64 if dtype == "f64" else np.float32)
        x, k = w["x"], w["k"]
        init = x[np.random.default_rng(3).permutation(x.shape[0])[:k]].astype(np.float64)
    else:
        w = W.anisotropic_1024x128(scale=0.005)  # 20,000 rows, d = 128, k = 1024
        x, k, init = w["x"], w["k"], w["init"]
    ctx = F.Context(0)
    iters = 24  # two rounds of the six buffer rotations, then replays

    def model():
        m = F.KMeans(k, dtype=dtype).with_init_centers(init if dtype != "f32" else init.astype(np.float32))
        if precision != "plain":
            m = m.with_precision(precision)
        return m.with_max_iter(iters).with_tol(0.0).with_n_init(1)
    first = model().fit(x, ctx=ctx)          # captures, then replays
    again = model().fit(x, ctx=ctx)          # replays the first call's graphs
    timed = model().with_timing(True).fit(x, ctx=ctx)  # launch by launch
    _same(first, timed)
    _same(again, timed)
    if precision == "plain":
        o = O.fit(x, k, max_iter=iters, tol=0.0, n_init=1, init=(init if dtype != "f32" else init.astype(np.float32))[None])
        assert np.array_equal(first.labels(), o["labels"])
        assert np.array_equal(first.cluster_centers(), o["centers"])
    else:
        o = O.fit(x.astype(np.float64), k, max_iter=iters, tol=0.0, n_init=1, init=init[None])
        assert np.array_equal(first.labels(), o["labels"])
    ctx.close()


def test_graphs_follow_a_new_input_on_the_same_context():
    # a different X (another device buffer) is another key: captured anew,
    # results equal to a fresh context's
    torch = pytest.importorskip("torch")
    w = W.dirichlet_256x64(scale=0.01, dtype=np.float32)
    x, k = w["x"], w["k"]
    init = x[:k].astype(np.float32)
    ctx = F.Context(0)
    m = lambda: F.KMeans(k, dtype="f32").with_init_centers(init).with_max_iter(16).with_tol(0.0).with_n_init(1)
    xa = torch.from_numpy(x).cuda()
    xb = torch.from_numpy(np.ascontiguousarray(x[::-1])).cuda()
    ra = m().fit(xa, ctx=ctx)
    rb = m().fit(xb, ctx=ctx)
    ctx2 = F.Context(0)
    _same(rb, m().fit(xb, ctx=ctx2))
    _same(ra, m().fit(xa, ctx=ctx2))
    ctx.close()
    ctx2.close()

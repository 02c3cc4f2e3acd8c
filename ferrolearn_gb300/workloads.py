"""Seeded synthetic inputs for the KMeans Lloyd workloads.

No public dataset is involved: every workload is a Gaussian blob mixture made
here with numpy's PCG64 generator, with the shapes and value distributions of
the benchmark configurations. Each generator takes a size scale so that tests
can run the same distribution at a size the CPU oracle finishes quickly.

  isotropic_8x16      n=10,000 d=16 k=8: 8 isotropic blobs, centres
                      U[-10,10]^16, std 1.0, equal sizes, seed 0; init = the
                      first 8 rows of a seeded permutation; f64; max_iter 300,
                      tol 1e-4, n_init 1.
  dirichlet_256x64    n=1,000,000 d=64 k=256: 256 blobs, centres
                      U[-20,20]^64, per-blob std U[0.5,3.0], blob sizes from a
                      Dirichlet(alpha=1) multinomial; k-means++ init;
                      max_iter 100, tol 1e-4.
  anisotropic_1024x128 n=4,000,000 d=128 k=1024, X stored f32: blobs with
                      covariance A A^T, A_ij ~ N(0, 0.3^2) (128x128), centres
                      U[-15,15]^128; init = first k rows of a seeded
                      permutation; 50 iterations (tol 0).
  batched_512         512 independent problems: n log-uniform in
                      [2,000, 200,000], d from {8, 16, 32, 64}, k uniform
                      in [4, 64]; each a mixture of k Gaussian blobs with
                      std 1.0 and centres U[-10,10]^d; f32; 10 seeded
                      k-means++ restarts each (5,120 fits), tol 1e-4.
  bisector_4096x256   n=8,000,000 d=256 k=4096, X stored f32: 4096 blobs,
                      std 1.0, centres U[-30,30]^256, plus 10% of the rows
                      placed on the perpendicular bisector of two seeded
                      centres (equidistant in real arithmetic; f32 storage
                      leaves them within rounding of a tie); init = first k
                      rows of a seeded permutation; 20 iterations (tol 0);
                      then predict on 2,000,000 fresh rows of the same
                      mixture.
"""
import numpy as np


def _perm_init(x, k, seed):
    rng = np.random.default_rng(seed)
    idx = rng.permutation(x.shape[0])[:k]
    return np.ascontiguousarray(x[idx])


def isotropic_8x16(scale=1.0, seed=0):
    n_per = max(1, int(round(1250 * scale)))
    k, d = 8, 16
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-10.0, 10.0, size=(k, d))
    x = np.concatenate([centres[b] + rng.normal(0.0, 1.0, size=(n_per, d)) for b in range(k)])
    init = _perm_init(x, k, seed + 1)
    return dict(x=x, k=k, init=init, max_iter=300, tol=1e-4, n_init=1, name="isotropic_8x16",
                desc=f"n={x.shape[0]} d={d} k={k} f64, 8 isotropic blobs, init = first k rows of a seeded permutation")


def dirichlet_256x64(scale=1.0, seed=0, k=256, d=64, dtype=np.float64):
    n = max(k, int(round(1_000_000 * scale)))
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-20.0, 20.0, size=(k, d))
    stds = rng.uniform(0.5, 3.0, size=k)
    w = rng.dirichlet(np.ones(k))
    sizes = rng.multinomial(n, w)
    lab = np.repeat(np.arange(k), sizes)
    rng.shuffle(lab)
    x = centres[lab] + rng.standard_normal(size=(n, d)) * stds[lab][:, None]
    return dict(x=np.ascontiguousarray(x, dtype=dtype), k=k, init=None, max_iter=100, tol=1e-4, n_init=1,
                seed=seed, name="dirichlet_256x64",
                desc=f"n={n} d={d} k={k}, 256 blobs with Dirichlet(1) sizes, k-means++ init")


def anisotropic_1024x128(scale=1.0, seed=0, k=1024, d=128):
    n = max(k, int(round(4_000_000 * scale)))
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-15.0, 15.0, size=(k, d)).astype(np.float32)
    sizes = np.full(k, n // k)
    sizes[: n - sizes.sum()] += 1
    x = np.empty((n, d), dtype=np.float32)
    pos = 0
    for b in range(k):
        a = rng.normal(0.0, 0.3, size=(d, d)).astype(np.float32)
        z = rng.standard_normal(size=(sizes[b], d), dtype=np.float32)
        x[pos:pos + sizes[b]] = centres[b] + z @ a.T
        pos += sizes[b]
    perm = rng.permutation(n)
    x = np.ascontiguousarray(x[perm])
    init = _perm_init(x, k, seed + 1).astype(np.float64)
    return dict(x=x, k=k, init=init, max_iter=50, tol=0.0, n_init=1, name="anisotropic_1024x128",
                desc=f"n={n} d={d} k={k}, X f32, 1024 anisotropic blobs (A A^T, A~N(0,0.3^2)), 50 iterations")


def _bisector_rows(centres, m, rng):
    """m rows on the perpendicular bisector of two seeded centres each:
    (a + b) / 2 + u with u a N(0, 1) vector projected orthogonal to b - a."""
    k, d = centres.shape
    a = rng.integers(0, k, size=m)
    b = (a + 1 + rng.integers(0, k - 1, size=m)) % k
    ca, cb = centres[a].astype(np.float64), centres[b].astype(np.float64)
    w = cb - ca
    u = rng.standard_normal(size=(m, d))
    u -= ((u * w).sum(1) / (w * w).sum(1))[:, None] * w
    return 0.5 * (ca + cb) + u


def _bisector_mixture(n, centres, rng, frac=0.1, chunk=1 << 20):
    k, d = centres.shape
    x = np.empty((n, d), dtype=np.float32)
    m_bis = int(round(frac * n))
    lab = rng.integers(0, k, size=n - m_bis)
    for lo in range(0, n - m_bis, chunk):
        hi = min(n - m_bis, lo + chunk)
        x[lo:hi] = centres[lab[lo:hi]] + rng.standard_normal(size=(hi - lo, d), dtype=np.float32)
    for lo in range(n - m_bis, n, chunk):
        hi = min(n, lo + chunk)
        x[lo:hi] = _bisector_rows(centres, hi - lo, rng)
    return np.ascontiguousarray(x[rng.permutation(n)])


def bisector_4096x256(scale=1.0, seed=0, k=4096, d=256, predict_scale=None):
    n = max(k, int(round(8_000_000 * scale)))
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-30.0, 30.0, size=(k, d)).astype(np.float32)
    x = _bisector_mixture(n, centres, rng)
    init = _perm_init(x, k, seed + 1).astype(np.float64)
    ps = scale if predict_scale is None else predict_scale
    n_pred = max(1, int(round(2_000_000 * ps)))
    x_pred = _bisector_mixture(n_pred, centres, np.random.default_rng(seed + 2))
    return dict(x=x, k=k, init=init, max_iter=20, tol=0.0, n_init=1, x_predict=x_pred, name="bisector_4096x256",
                desc=f"n={n} d={d} k={k}, X f32, 4096 blobs std 1 + 10% bisector rows, 20 iterations, "
                     f"predict on {n_pred} rows")


def batched_512(scale=1.0, seed=0, n_problems=512, n_init=10, max_iter=300, tol=1e-4):
    """The batched workload: a list of problem dicts for fit_batched. scale
    multiplies every n (kept >= k); n_problems trims the list."""
    rng = np.random.default_rng(seed)
    probs = []
    for p in range(n_problems):
        n = int(round(np.exp(rng.uniform(np.log(2000.0), np.log(200000.0))) * scale))
        d = int(rng.choice([8, 16, 32, 64]))
        k = int(rng.integers(4, 65))
        n = max(n, k)
        cen = rng.uniform(-10.0, 10.0, size=(k, d)).astype(np.float32)
        lab = rng.integers(0, k, size=n)
        x = cen[lab] + rng.standard_normal(size=(n, d), dtype=np.float32)
        probs.append(dict(x=np.ascontiguousarray(x, dtype=np.float32), k=k, n_init=n_init, max_iter=max_iter,
                          tol=tol, random_state=int(seed * 100003 + p)))
    return probs

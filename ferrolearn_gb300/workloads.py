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

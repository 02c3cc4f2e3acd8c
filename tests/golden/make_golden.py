"""Regenerate the golden fixtures under tests/golden/.

Run once in a checkout that has the reference tree mounted read-only:

    python tests/golden/make_golden.py /path/to/ferrolearn

Outputs (small JSON files, committed):

* ref_kmeans_blobs150.json -- the reference's own KMeans oracle fixture
  (ferrolearn fixtures/kmeans.json, produced by the reference's
  scripts/generate_fixtures.py with scikit-learn 1.7.2): X 150x2, k=3,
  expected labels / centres / inertia / n_iter. Consumed by
  ferrolearn-cluster/tests/oracle_tests.rs:66-117.
* ref_sklearn_kmeans50.json -- the reference's statistical-equivalence
  fixture (tests/fixtures/sklearn_reference/kmeans.json): X 50x5, k=3.
  Consumed by ferrolearn-cluster/tests/sklearn_equivalence.rs:34-117.
* sklearn_lloyd_steps.json -- Lloyd trajectories computed here with the
  installed scikit-learn (algorithm="lloyd", n_init=1, tol=0) from explicit
  initial centres, for m = 1..4 iterations: the centres after m updates and
  the labels against those centres. These pin the update step and the
  assignment step of the oracle independently of any random init.

Only the data values are copied; nothing here is reference source code.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _dump(name, obj):
    with open(os.path.join(HERE, name), "w") as f:
        json.dump(obj, f, separators=(",", ":"))
        f.write("\n")


def copy_reference_fixtures(ref_root):
    d = json.load(open(os.path.join(ref_root, "fixtures", "kmeans.json")))
    _dump("ref_kmeans_blobs150.json", {
        "source": "ferrolearn fixtures/kmeans.json (scikit-learn %s)" % d["sklearn_version"],
        "params": d["params"],
        "X": d["input"]["X"],
        "labels": d["expected"]["labels"],
        "cluster_centers": d["expected"]["cluster_centers"],
        "inertia": d["expected"]["inertia"],
        "n_iter": d["expected"]["n_iter"],
    })
    d = json.load(open(os.path.join(ref_root, "tests", "fixtures", "sklearn_reference", "kmeans.json")))
    _dump("ref_sklearn_kmeans50.json", {
        "source": "ferrolearn tests/fixtures/sklearn_reference/kmeans.json (scikit-learn %s)"
                  % d["sklearn_version"],
        "params": d["params"],
        "X": d["X_train"],
        "labels": d["labels"],
        "cluster_centers": d["cluster_centers"],
        "inertia": d["inertia"],
        "n_iter": d["n_iter"],
    })


def sklearn_steps():
    from sklearn.cluster import KMeans as SkKMeans
    import sklearn

    cases = []
    rng = np.random.default_rng(20261203)
    for (n, d, k) in [(200, 3, 4), (500, 8, 6), (300, 16, 8)]:
        centres = rng.uniform(-10, 10, size=(k, d))
        lab = rng.integers(0, k, size=n)
        x = centres[lab] + rng.normal(0, 1.5, size=(n, d))
        init = x[rng.permutation(n)[:k]].copy()
        steps = []
        for m in range(1, 5):
            km = SkKMeans(n_clusters=k, init=init, n_init=1, max_iter=m, tol=0.0,
                          algorithm="lloyd").fit(x)
            steps.append({"m": m, "centers": km.cluster_centers_.tolist(),
                          "labels": km.labels_.tolist(), "n_iter": int(km.n_iter_)})
        cases.append({"n": n, "d": d, "k": k, "X": x.tolist(), "init": init.tolist(), "steps": steps})
    _dump("sklearn_lloyd_steps.json", {"sklearn_version": sklearn.__version__, "cases": cases})


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py <reference-root>")
    copy_reference_fixtures(sys.argv[1])
    sklearn_steps()
    print("golden fixtures written to", HERE)

"""Build recipe of the native library: nvcc, sm_103a only, in-tree.

Each translation unit under csrc/ is compiled in parallel, then linked into
ferrolearn_gb300/_build/libferrokmeans.so (static cudart, no torch). The
exactness-critical units (direct-form distances, centroid sums, k-means++)
are compiled with -fmad=false as well as using the _rn intrinsics, so no
multiply-add is ever contracted there.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libferrokmeans.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "--expt-relaxed-constexpr", "-I", INCLUDE]
EXACT_UNITS = {"fk_assign.cu", "fk_update.cu", "fk_kpp.cu", "fk_batched.cu"}


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build ferrolearn_gb300")
    return cand


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _digest():
    h = hashlib.sha256()
    for name in sorted(os.listdir(CSRC)):
        if name.endswith((".cu", ".cuh", ".h")):
            h.update(name.encode())
            h.update(open(os.path.join(CSRC, name), "rb").read())
    h.update(open(os.path.join(INCLUDE, "ferrokmeans.h"), "rb").read())
    h.update(" ".join(ARCH + COMMON).encode())
    return h.hexdigest()


def _compile(nvcc, src, extra=()):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    flags = list(COMMON) + list(extra)
    if src in EXACT_UNITS:
        flags += ["-fmad=false"]
    cmd = [nvcc] + ARCH + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force=False, verbose=False, extra=()):
    """Compile every CUDA unit and link the shared library; returns its path."""
    os.makedirs(OUT, exist_ok=True)
    stamp = os.path.join(OUT, "stamp.txt")
    dig = _digest() + "|" + " ".join(extra)
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == dig:
        return LIB
    nvcc = _nvcc()
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(nvcc, s, extra), srcs))
    if verbose:
        for _, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(dig)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))

"""Benchmark of the KMeans Lloyd hot path on one GB300.

Workload (default): anisotropic_1024x128 -- n=4,000,000 rows x d=128
features, k=1024 clusters, X stored f32 (2.05 GB, larger than L2), 1024
anisotropic Gaussian blobs, init = first k rows of a seeded permutation, tol 0
so every iteration runs. A step is one Lloyd iteration over all n rows
(assignment + centroid update + inertia + shift).

  value   Lloyd iterations/s of the chosen form with X already resident in
          HBM: one fit call running W warm-up iterations, then one fit call
          running exactly K iterations (results into device tensors) timed
          with CUDA events on the stream the library launches on (no phase
          timers in it, so its steady-state iterations replay CUDA graphs;
          the phase breakdown comes from a second, timed run of the same
          fit).
  e2e     the same metric through the public API with host buffers: one fit
          call on a pinned host X (H2D of X, K iterations, D2H of labels and
          centres inside the timed region).
  parity  outside the timed region, the same K iterations replayed one step
          at a time from the same centres, each checked against the FP64
          oracle (oracle/, a restatement of kmeans.rs): label mismatches on a
          seeded sample of rows (the oracle's direct form with the step's
          centres), centre error against the oracle's update over all n rows
          with the step's labels, inertia error, the shift, the near-tie
          count; and the timed fit's own outputs against the replay's.
  forms   bf16  = FK_PRECISION_MIXED_BF16 on the f32x64 entry point
                  (KMeans<f64> semantics, BF16 tcgen05 contraction + FP64
                  re-check); labels identical to the FP64 oracle.
          fp8   = FK_PRECISION_MIXED_FP8, the same with an E4M3 contraction
                  (per-row power-of-two scales).
          fp32  = plain KMeans<f32> (direct-form FP32 on CUDA cores).
          fp64  = plain KMeans<f64> on f64 data (the dirichlet workload drawn
                  in f64; k-means++ in f64).

Other workloads (--workload; parity cases of the same path, measured on
request): bisector = n=8,000,000 d=256 k=4096 with 10% bisector rows, FP8,
20 iterations, then predict on 2,000,000 fresh rows (reported as
predict_rows_per_s); dirichlet = n=1,000,000 d=64 k=256, plain f32 / f64,
k-means++ init on the GPU (timed separately as kpp_ms); batched = 512
independent problems (n log-uniform in [2,000, 200,000], d in {8,16,32,64},
k in [4,64]) x 10 k-means++ restarts, one fit_batched call per step (f32
distances, FP64 centroid sums); value = Lloyd iterations over all 5,120 fits
per second of the call, pt_k_per_s = sum of n * k * iterations per second;
minibatch = MiniBatchKMeans on the dirichlet shape (batch 1024); bisecting =
BisectingKMeans, n=200,000 d=16 k=32, n_init 10; transform = the n x k
distance matrix of the dirichlet shape (f32), rows/s, with the bytes written.

--impl reference times the CPU restatement of the reference (oracle/; the
reference is Rust and cannot be built here) with all host threads: the K
timed steps together are ONE full Lloyd iteration over all n rows (step s
assigns rows [s n / K, (s + 1) n / K) with the chunked parallel assignment
and adds them to the row-order centroid sums; the last step finishes the
update), so value = 1 / (time of that full iteration), measured, not
extrapolated.
"""
import argparse
import ctypes as C
import faulthandler
import json
import os
import platform
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed Lloyd iterations (default: the workload's own count, 50 for anisotropic)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="auto", choices=["auto", "bf16", "fp8", "fp32", "fp64"])
    ap.add_argument("--workload", default="anisotropic",
                    choices=["anisotropic", "bisector", "dirichlet", "batched", "minibatch", "bisecting",
                             "transform"])
    ap.add_argument("--scale", type=float, default=1.0, help="fraction of the full row count")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the per-iteration oracle checks")
    ap.add_argument("--parity-rows", type=int, default=100_000,
                    help="rows per iteration whose labels are checked against the oracle's direct form")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    args = ap.parse_args(argv)
    if args.steps is None:  # the configurations' own iteration counts (anisotropic: 50 Lloyd iterations)
        args.steps = {"anisotropic": 50, "bisector": 20, "dirichlet": 20, "batched": 20, "minibatch": 100,
                      "bisecting": 3, "transform": 20}[args.workload]
    return args


METRIC = "KMeans Lloyd iters/s & pt·k/s: BF16+FP64 recheck vs plain FP32, labels=FP64"

# DRAM traffic of the main pass per row of X (ncu dram__bytes_read.sum +
# dram__bytes_write.sum of one launch, divided by the rows it processed; the
# traffic grows in proportion to the rows: X read once, records written once).
# Source: profiles/tc_count_anisotropic_1024x128_quarter.md, 1,000,000-row
# captures of tc_assign_kernel<3> (count pass: 260.4 MB read + 25.5 MB
# written) and tc_assign_kernel<2> (top-2 pass: 256.4 + 25.1 MB).
TRAFFIC_BYTES_PER_ROW = {("anisotropic_1024x128", "bf16", "count"): (260.4e6 + 25.5e6) / 1e6,
                         ("anisotropic_1024x128", "bf16", "top2"): (256.4e6 + 25.1e6) / 1e6}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm": d.get("hbm_gbs", 6800.0), "bf16": d.get("bf16_tflops", 1900.0),
                "bf16s": d.get("bf16_tflops_sustained", 1700.0), "sm_max": d.get("sm_max_mhz", 2070.0),
                "src": "measured"}
    return {"hbm": 6800.0, "bf16": 1900.0, "bf16s": 1700.0, "sm_max": 2070.0, "src": "fallback"}


def pick_tensor_peak(peaks, clocks):
    """The burst BF16 peak when the SM clock stayed at its maximum through the
    timed region (a short region: the power cap has not pulled the clock
    down), else the sustained one; returns (TFLOP/s, which)."""
    sm = clocks.get("sm_mhz")
    mx = clocks.get("sm_max_mhz") or peaks["sm_max"]
    if sm is not None and mx and sm >= 0.97 * mx:
        return peaks["bf16"], (f"bf16_tflops, burst ({peaks['src']}): the SM clock stayed at {sm:.0f} of "
                               f"{mx:.0f} MHz in the timed region")
    return peaks["bf16s"], (f"bf16_tflops_sustained ({peaks['src']}): the SM clock ran at {sm} of {mx} MHz "
                            "in the timed region")


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else platform)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    return platform.processor() or platform.machine()


def max_over_ranks(value, device):
    """The slowest rank's value (the job ends with it); the value itself on
    one rank or without a process group. device: where the collective's
    tensor lives ("cuda" under NCCL, "cpu" under gloo)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(iters_per_rank, ms_slowest, world):
    """Whole-job Lloyd iterations/s: every replica's iterations over the
    slowest replica's time."""
    return world * iters_per_rank / (ms_slowest / 1e3)


class ClockSampler:
    """nvidia-smi clocks + throttle reasons sampled every 20 ms; summary()
    keeps the samples taken while the timed region ran (mark_start/mark_end,
    host clock, +-0.15 s), or the nearest one when the region was shorter
    than the sampling interval."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            deadline = time.time() + 3.0
            while not self.lines and time.time() < deadline:  # sampling is live before the region starts
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def mark_start(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = list(self.lines)
        if self.t0 is not None and self.t1 is not None and rows:
            inside = [r for r in rows if self.t0 - 0.15 <= r[0] <= self.t1 + 0.15]
            if not inside:
                mid = 0.5 * (self.t0 + self.t1)
                inside = [min(rows, key=lambda r: abs(r[0] - mid))]
            rows = inside
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for _, ln in rows:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(args):
    from ferrolearn_gb300 import workloads as W
    if args.workload == "bisector":
        return W.bisector_4096x256(scale=args.scale)
    if args.workload == "dirichlet":
        return W.dirichlet_256x64(scale=args.scale, dtype=np.float64 if args.form == "fp64" else np.float32)
    return W.anisotropic_1024x128(scale=args.scale)


DEFAULT_FORM = {"anisotropic": "bf16", "bisector": "fp8", "dirichlet": "fp32", "batched": "fp32"}


def workload_config(w):
    """The `config` of both arms' JSON lines (the workload, not the arm)."""
    n, d = w["x"].shape
    return {"workload": w["name"], "n": int(n), "d": int(d), "k": int(w["k"]),
            "X": "f64" if w["x"].dtype == np.float64 else "f32",
            "init": "first k rows of a seeded permutation" if w.get("init") is not None or w["name"] != "dirichlet_256x64"
            else "k-means++ (seeded)",
            "tol": 0.0, "l2": f"inputs larger than L2 (X {w['x'].nbytes / 1e9:.2f} GB)", "parallelism": "replicas"}


def initial_centres(w, xd, ctx):
    """The workload's initial centres, or k-means++ on the GPU (timed) where it
    names none; returns (centres f64, ms of the k-means++ call or None)."""
    if w["init"] is not None:
        return w["init"], None
    import torch

    import ferrolearn_gb300 as F
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    c, _ = F.kmeans_plus_plus(xd, w["k"], seed=w.get("seed", 0),
                              dtype="f64" if w["x"].dtype == np.float64 else "f32", ctx=ctx)
    ms = (time.perf_counter() - t0) * 1e3
    w["init"] = c.astype(np.float64)
    return w["init"], ms


def cpu_baseline(w, seconds, threads):
    """Oracle (CPU restatement of kmeans.rs) on a bounded row sample; iters/s extrapolated to the full n."""
    from oracle import oracle as O
    c = w["init"]
    n = w["x"].shape[0]
    rows = 2048
    while True:
        xs = w["x"][:rows].astype(np.float64)  # only the sampled rows are widened
        t0 = time.perf_counter()
        O.lloyd_step(xs, c, nthreads=threads)
        dt = time.perf_counter() - t0
        if dt >= seconds / 4 or rows >= n:
            break
        rows = min(n, int(rows * max(2.0, (seconds / 4) / max(dt, 1e-3))))
    xs = w["x"][:rows].astype(np.float64)
    reps = max(1, int(seconds / max(dt, 1e-3)))
    t0 = time.perf_counter()
    for _ in range(reps):
        O.lloyd_step(xs, c, nthreads=threads)
    dt = (time.perf_counter() - t0) / reps
    per_iter = dt * n / rows
    return {"value": 1.0 / per_iter, "unit": "iters/s", "cores": threads, "cpu_model": cpu_model(), "kind": "port",
            "sample": f"{rows} of {n} rows, {reps} Lloyd iterations (FP64 direct form, OpenMP chunked like "
                      f"assign_parallel, serial update); per-iteration time extrapolated x{n / rows:.1f}",
            "seconds_per_full_iteration": per_iter}


def run_reference(args):
    """The reference's CPU algorithm (the oracle restatement, kind "port") on
    the machine's host cores: K steps that together are one full Lloyd iteration
    over all n rows, timed step by step."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    w = make_workload(args)
    if w["init"] is None:
        w["init"] = w["x"][np.random.default_rng(1).permutation(w["x"].shape[0])[: w["k"]]].astype(np.float64)
    threads = os.cpu_count() or 1
    x32 = w["x"]
    n, d = x32.shape
    k = w["k"]
    x64 = x32.astype(np.float64)  # KMeans<f64>'s input: X widened exactly, once, before any timing
    c = np.ascontiguousarray(w["init"], dtype=np.float64)
    wrows = min(n, 20000)
    for _ in range(max(1, args.warmup)):  # warm-up: the assignment on a 20,000-row slice
        O.assign(x64[:wrows], c, nthreads=threads)
    K = max(1, args.steps)
    bounds = [n * s // K for s in range(K + 1)]
    sums, counts = np.zeros((k, d)), np.zeros(k)
    step_s = []
    for s in range(K):
        t0 = time.perf_counter()
        lo, hi = bounds[s], bounds[s + 1]
        if hi > lo:
            lab, _ = O.assign(x64[lo:hi], c, nthreads=threads)  # nearest_center over the rows, chunked in parallel
            O.update_rows(x64[lo:hi], lab, sums, counts)           # recompute_centroids_into's row-order sums
        if s == K - 1:
            O.update_finish(sums, counts, c)                       # means, empty clusters, shift
        step_s.append(time.perf_counter() - t0)
    total = float(np.sum(step_s))
    v = 1.0 / total
    sample = (f"one full Lloyd iteration over all {n} rows split into {K} consecutive row ranges, one per step "
              f"(parallel assignment, serial row-order update), measured: {total:.2f} s")
    out = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "iters/s", "n_gpus": args.gpus,
        "steps": K, "warmup": args.warmup, "ms_per_step": total * 1e3 / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(w),
        "step": "1/K of one Lloyd iteration (rows [s n/K, (s+1) n/K))",
        "cpu_baseline": {"value": v, "unit": "iters/s", "cores": threads, "cpu_model": cpu_model(), "kind": "port",
                         "arithmetic": "KMeans<f64> on X widened exactly (FP64 direct form)", "sample": sample},
        "e2e": {"value": v, "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def run_batched(args):
    """The batched workload: one fit_batched call per step."""
    import torch

    import ferrolearn_gb300 as F
    from ferrolearn_gb300 import _native
    from ferrolearn_gb300 import workloads as W

    dev = torch.cuda.current_device()
    probs = W.batched_512(scale=args.scale)
    stream = torch.cuda.Stream()
    ctx = F.Context(dev, stream=stream.cuda_stream)
    dprobs = [dict(p, x=torch.from_numpy(p["x"]).to(dev)) for p in probs]
    torch.cuda.synchronize()
    for _ in range(max(1, args.warmup)):
        F.fit_batched(dprobs, reduction="f64", ctx=ctx)
    l0 = _native.lib().fk_debug_launch_count()
    times, reps = [], []
    with ClockSampler(dev) as clocks:
        clocks.mark_start()
        for _ in range(args.steps):
            torch.cuda.synchronize()
            start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            start.record(stream)
            _, rep = F.fit_batched(dprobs, reduction="f64", ctx=ctx)
            end.record(stream)
            torch.cuda.synchronize()
            times.append(start.elapsed_time(end))
            reps.append(rep)
        clocks.mark_end()
    launches = int(_native.lib().fk_debug_launch_count() - l0)
    ms = float(np.sum(times))
    iters = sum(r["iterations_total"] for r in reps)
    nk, nkd = 0.0, 0.0
    for r in reps:
        f0 = 0
        for p in probs:
            it = float(r["fit_n_iter"][f0:f0 + p["n_init"]].sum())
            nk += float(p["x"].shape[0]) * p["k"] * it
            nkd += float(p["x"].shape[0]) * p["k"] * p["x"].shape[1] * it
            f0 += p["n_init"]
    rep = reps[-1]
    # the Lloyd phase runs on the CUDA cores: its peak is measured in this run
    pk = (C.c_double * 8)()
    _native.lib().fk_debug_measure_peaks(ctx.handle, pk)
    fp32 = pk[0] / 1e12
    lloyd_ms = float(np.sum([r["ms_lloyd"] for r in reps]))
    achieved = 2.0 * nkd / (lloyd_ms / 1e3) / 1e12
    out = {
        "metric": METRIC, "value": iters / (ms / 1e3), "unit": "iters/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (f64 centroid sums)", "data": "synthetic", "form": "batched",
        "config": {"workload": "batched_512", "problems": len(probs), "fits": rep["fits"],
                   "rows_total": int(sum(p["x"].shape[0] for p in probs)), "n_init": 10,
                   "init": "k-means++ per restart (seeded)", "tol": 1e-4, "reduction": "f64",
                   "l2": "inputs larger than L2", "parallelism": "replicas"},
        "pt_k_per_s": nk / (ms / 1e3),
        "iterations_per_step": iters / args.steps,
        "phase_ms": {k: rep[k] for k in ("ms_upload", "ms_init", "ms_tune", "ms_lloyd", "ms_download", "ms_total")},
        "graph_launches": rep["graph_launches"], "tiles": rep["tiles"],
        "gpu_launches": launches, "clocks": clocks.summary(),
        "roofline": {"bound": "fp32-simt", "achieved": achieved, "peak": fp32, "unit": "TFLOP/s",
                     "frac": achieved / fp32, "traffic": None,
                     "kernel": "the graph-replayed Lloyd phase (batch_assign + batch_update), all fits",
                     "ms_per_launch": lloyd_ms / len(reps),
                     "peak_source": "FP32 FMA peak measured in this run (fk_debug_measure_peaks); achieved counts "
                                    "2 n k d per fit iteration over the Lloyd phase's device time (the direct form "
                                    "executes 3 n k d)"},
    }
    if not args.no_e2e:
        t0 = time.perf_counter()
        _, r2 = F.fit_batched(probs, reduction="f64", ctx=ctx)
        t1 = time.perf_counter()
        out["e2e"] = {"value": r2["iterations_total"] / (t1 - t0), "unit": "iters/s",
                      "h2d_bytes_per_step": int(sum(p["x"].nbytes for p in probs)),
                      "d2h_bytes_per_step": int(sum(p["x"].shape[0] * 8 + p["k"] * p["x"].shape[1] * 4
                                                    for p in probs)),
                      "note": "one fit_batched call on host arrays"}
    if not args.no_cpu:
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        it_cpu, nk_cpu, done = 0, 0.0, 0
        for p in probs:
            o = O.fit_runs(p["x"], p["k"], max_iter=p["max_iter"], tol=p["tol"], n_init=p["n_init"],
                           seed=p["random_state"], wide_sums=True, nthreads=threads)
            it_cpu += int(o["n_iter"].sum())
            nk_cpu += float(p["x"].shape[0]) * p["k"] * float(o["n_iter"].sum())
            done += 1
            if time.perf_counter() - t0 > args.cpu_seconds:
                break
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": it_cpu / dt, "unit": "iters/s", "cores": threads, "cpu_model": cpu_model(),
                               "kind": "port", "pt_k_per_s": nk_cpu / dt,
                               "sample": f"{done} of {len(probs)} problems, all 10 runs each (oracle fit_runs)"}
    print(json.dumps(out))


def _timed_calls(stream, fn, reps):
    """Device time (CUDA events on the library's stream) of `reps` calls of fn."""
    import torch
    times, out = [], None
    for _ in range(reps):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        out = fn()
        b.record(stream)
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    return float(np.sum(times)), out


def run_minibatch(args):
    """MiniBatchKMeans::fit (mini_batch_kmeans.rs:492-591) on the GPU: n =
    1,000,000 x d = 64, k = 256 (the Dirichlet blob mixture), batch 1024, one
    run from the first k rows of a seeded permutation, tol 0; a step is one
    mini-batch iteration; the timed fit includes its final assignment of all
    n rows (assign_clusters_mb, :343-376)."""
    import torch

    import ferrolearn_gb300 as F
    from ferrolearn_gb300 import _native
    from ferrolearn_gb300 import workloads as W
    dev = torch.cuda.current_device()
    w = W.dirichlet_256x64(scale=args.scale, dtype=np.float64)
    x, k = w["x"], w["k"]
    n, d = x.shape
    init = x[np.random.default_rng(1).permutation(n)[:k]][None].copy()
    stream = torch.cuda.Stream()
    ctx = F.Context(dev, stream=stream.cuda_stream)
    xd = torch.from_numpy(x).to(dev)

    def model(iters):
        return F.MiniBatchKMeans(k).with_batch_size(1024).with_max_iter(iters).with_n_init(1).with_tol(0.0) \
            .with_init_centers(init)
    model(args.warmup).fit(xd, ctx=ctx)
    l0 = _native.lib().fk_debug_launch_count()
    with ClockSampler(dev) as clocks:
        clocks.mark_start()
        ms, fitted = _timed_calls(stream, lambda: model(args.steps).fit(xd, ctx=ctx), 1)
        clocks.mark_end()
    launches = int(_native.lib().fk_debug_launch_count() - l0)
    # the final assignment of all rows alone (the fit's fixed part)
    c = fitted.cluster_centers()
    ms_assign, _ = _timed_calls(stream, lambda: F.FittedKMeans(c, None, 0.0, 0, "f64").predict(xd, ctx=ctx), 1)
    out = {"metric": "MiniBatchKMeans mini-batch iterations/s", "value": args.steps / (ms / 1e3), "unit": "iters/s",
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "form": "minibatch",
           "config": {"workload": "minibatch_dirichlet_256x64", "n": n, "d": d, "k": k, "batch_size": 1024,
                      "n_init": 1, "tol": 0.0, "init": "first k rows of a seeded permutation",
                      "l2": f"inputs larger than L2 (X {x.nbytes / 1e9:.2f} GB)", "parallelism": "replicas"},
           "fit_ms": ms, "final_assignment_ms": ms_assign,
           "ms_per_minibatch_iteration": (ms - ms_assign) / args.steps,
           "gpu_launches": launches, "launches_per_iteration": launches / args.steps, "clocks": clocks.summary(),
           "roofline": {"bound": "latency", "achieved": None, "peak": None, "unit": None, "frac": None,
                        "traffic": None,
                        "note": "a mini-batch iteration is four small launches (gather 1024 rows, their direct-form "
                                "assignment, the in-order centre update, the shift); profiles/ has the launch list"}}
    if not args.no_e2e:
        t0 = time.perf_counter()
        f2 = model(args.steps).fit(x, ctx=ctx)
        t1 = time.perf_counter()
        out["e2e"] = {"value": f2.n_iter() / (t1 - t0), "unit": "iters/s", "h2d_bytes_per_step": x.nbytes / args.steps,
                      "d2h_bytes_per_step": (n * 8 + k * d * 8) / args.steps,
                      "note": "one fit call on a host X running K mini-batch iterations"}
    if not args.no_cpu:
        from oracle import oracle as O
        t0 = time.perf_counter()
        O.minibatch_fit(x, k, batch_size=1024, max_iter=args.steps, n_init=1, init_centers=init)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": args.steps / dt, "unit": "iters/s", "cores": os.cpu_count() or 1,
                               "cpu_model": cpu_model(), "kind": "port",
                               "sample": f"the same fit ({args.steps} mini-batch iterations and the final "
                                         "assignment of all rows)"}
    print(json.dumps(out), flush=True)
    ctx.close()


def run_bisecting(args):
    """BisectingKMeans::fit (bisecting_kmeans.rs:326-505) on the GPU: n =
    200,000 x d = 16, target k = 32 (a 32-blob Dirichlet mixture), n_init 10,
    max_iter 300, LargestCluster; a step is one whole fit."""
    import torch

    import ferrolearn_gb300 as F
    from ferrolearn_gb300 import _native
    from ferrolearn_gb300 import workloads as W
    dev = torch.cuda.current_device()
    w = W.dirichlet_256x64(scale=0.2 * args.scale, k=32, d=16, dtype=np.float64)
    x, k = w["x"], w["k"]
    n, d = x.shape
    stream = torch.cuda.Stream()
    ctx = F.Context(dev, stream=stream.cuda_stream)
    xd = torch.from_numpy(x).to(dev)

    def fit():
        return F.BisectingKMeans(k).with_n_init(10).with_random_state(0).fit(xd, ctx=ctx)
    for _ in range(max(1, args.warmup)):
        fit()
    l0 = _native.lib().fk_debug_launch_count()
    with ClockSampler(dev) as clocks:
        clocks.mark_start()
        ms, _ = _timed_calls(stream, fit, args.steps)
        clocks.mark_end()
    launches = int(_native.lib().fk_debug_launch_count() - l0)
    out = {"metric": "BisectingKMeans fits/s", "value": args.steps / (ms / 1e3), "unit": "fits/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "form": "bisecting",
           "config": {"workload": "bisecting_dirichlet_32x16", "n": n, "d": d, "k": k, "n_init": 10,
                      "max_iter": 300, "strategy": "largest_cluster", "random_state": 0,
                      "l2": "inputs smaller than L2 (X 25.6 MB, re-read by every 2-means iteration)",
                      "parallelism": "replicas"},
           "gpu_launches": launches, "launches_per_fit": launches / args.steps, "clocks": clocks.summary(),
           "roofline": {"bound": "latency", "achieved": None, "peak": None, "unit": None, "frac": None,
                        "traffic": None,
                        "note": "hundreds of small launches per fit with a host round trip per 2-means iteration; "
                                "profiles/ has the launch list"}}
    if not args.no_cpu:
        from oracle import oracle as O
        t0 = time.perf_counter()
        O.bisecting_fit(x, k, n_init=10, seed=0)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 1.0 / dt, "unit": "fits/s", "cores": 1, "cpu_model": cpu_model(),
                               "kind": "port", "sample": "one whole fit (the reference's serial 2-means)"}
    print(json.dumps(out), flush=True)
    ctx.close()


def run_transform(args):
    """Transform::transform (kmeans.rs:568-617) at scale: the n x k distance
    matrix of n = 1,000,000 rows x d = 64 (the Dirichlet blob mixture, f32)
    against k = 256 centres (the first k rows of a seeded permutation); a
    step is one transform call over all rows, the output left on the
    device. The direct form (x_j - c_j)^2 summed left to right with no fused
    multiply-add, then the square root, bit for bit the reference's."""
    import ctypes as C

    import torch

    import ferrolearn_gb300 as F
    from ferrolearn_gb300 import _native
    from ferrolearn_gb300 import workloads as W
    from ferrolearn_gb300.kmeans import _check, _ptr
    dev = torch.cuda.current_device()
    w = W.dirichlet_256x64(scale=args.scale, dtype=np.float32)
    x, k = w["x"], w["k"]
    n, d = x.shape
    cen = np.ascontiguousarray(x[np.random.default_rng(1).permutation(n)[:k]])
    stream = torch.cuda.Stream()
    ctx = F.Context(dev, stream=stream.cuda_stream)
    xd = torch.from_numpy(x).to(dev)
    cd = torch.from_numpy(cen).to(dev)
    out = torch.empty((n, k), dtype=torch.float32, device=dev)
    fn = _native.lib().fk_kmeans_transform_f32

    def call():
        _check(fn(ctx.handle, _ptr(cd), k, d, _ptr(xd), n, d, _ptr(out)))
    for _ in range(max(3, args.warmup)):
        call()
    l0 = _native.lib().fk_debug_launch_count()
    with ClockSampler(dev) as clocks:
        clocks.mark_start()
        ms, _ = _timed_calls(stream, call, args.steps)
        clocks.mark_end()
    launches = int(_native.lib().fk_debug_launch_count() - l0)
    per = ms / args.steps
    pk = (C.c_double * 8)()
    _native.lib().fk_debug_measure_peaks(ctx.handle, pk)
    instr_peak = pk[0] / 2.0 / 1e12  # FP32 FMA instructions per second (one op each)
    ops = 3.0 * n * k * d  # sub, mul, add per (row, centre, feature); the direct form has no FMA
    wbytes = 4.0 * n * k
    out_line = {
        "metric": "KMeans transform rows/s (n x k distances, f32)", "value": n / (per / 1e3), "unit": "rows/s",
        "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": per,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "form": "transform",
        "config": {"workload": "transform_dirichlet_256x64", "n": n, "d": d, "k": k,
                   "centres": "first k rows of a seeded permutation",
                   "l2": f"inputs and output larger than L2 (X {x.nbytes / 1e9:.2f} GB, out {wbytes / 1e9:.2f} GB)",
                   "parallelism": "replicas"},
        "gpu_launches": launches, "clocks": clocks.summary(),
        "roofline": {"bound": "fp32-simt", "achieved": ops / (per / 1e3) / 1e12, "peak": instr_peak,
                     "unit": "T op/s", "frac": ops / (per / 1e3) / 1e12 / instr_peak, "traffic": None,
                     "kernel": "assign_direct_kernel<f32, f32, write all> (the transform form)",
                     "ms_per_launch": per,
                     "peak_source": "FP32 FMA instruction rate measured in this run (fk_debug_measure_peaks / 2); "
                                    "achieved counts the 3 n k d separate sub, mul and add of the direct form"},
        "hbm_write": {"bytes_per_step": wbytes, "achieved_gbs": wbytes / (per / 1e3) / 1e9,
                      "note": "the n x k output written once"},
    }
    # parity: a seeded sample of rows against the oracle, bit for bit
    from oracle import oracle as O
    rows = np.sort(np.random.default_rng(5).choice(n, min(n, 20000), replace=False))
    got = out[torch.from_numpy(rows).to(dev)].cpu().numpy()
    want = O.transform(cen, x[rows])
    out_line["parity"] = {"oracle": "oracle/ orc_transform_f32 (direct form + sqrt)", "rows_checked": int(len(rows)),
                          "bit_identical": bool(np.array_equal(got.view(np.uint32), want.view(np.uint32)))}
    if not args.no_e2e:
        fitted = F.FittedKMeans(cen, None, 0.0, 0, "f32")
        fitted.transform(x, ctx=ctx)
        t0 = time.perf_counter()
        for _ in range(3):
            fitted.transform(x, ctx=ctx)
        dt = (time.perf_counter() - t0) / 3
        out_line["e2e"] = {"value": n / dt, "unit": "rows/s", "h2d_bytes_per_step": float(x.nbytes),
                           "d2h_bytes_per_step": wbytes,
                           "note": "FittedKMeans.transform on a host X into a host n x k array (pageable)"}
    if not args.no_cpu:
        m = min(n, 100000)
        t0 = time.perf_counter()
        O.transform(cen, x[:m])
        dt = time.perf_counter() - t0
        out_line["cpu_baseline"] = {"value": m / dt, "unit": "rows/s", "cores": os.cpu_count() or 1,
                                    "cpu_model": cpu_model(), "kind": "port",
                                    "sample": f"the first {m} rows (oracle orc_transform_f32)"}
    print(json.dumps(out_line), flush=True)
    ctx.close()


def parity_leg(w, form, ctx, xd, iters, rows, fit_centres, fit_labels):
    """The timed trajectory replayed one Lloyd step at a time (the same
    entry point's single-iteration form, the same centres), each step checked
    against the FP64 oracle; then the timed fit's outputs against the replay's
    last step. Mixed forms: labels on a seeded sample of `rows` rows (the
    oracle's direct form with the step's centres), centres and inertia
    against the oracle's update over all n rows with the step's labels. Plain
    forms: the oracle's whole Lloyd step in the same precision (bit-identical
    expected)."""
    import ferrolearn_gb300 as F
    from oracle import oracle as O
    t_start = time.perf_counter()
    x32 = w["x"]
    n, d = x32.shape
    mixed = form in ("bf16", "fp8")
    rng = np.random.default_rng(20260)
    m = min(n, rows)
    sample = np.sort(rng.choice(n, m, replace=False)) if m < n else np.arange(n)
    xs64 = x32[sample].astype(np.float64)
    if form == "fp32":
        c = w["init"].astype(np.float32)
        dtype = "f32"
    elif form == "fp64":
        c = w["init"].astype(np.float64)
        dtype = "f64"
    else:
        c = w["init"].astype(np.float64)
        dtype = "f32x64"
    mism_total, mism_max, crel_max, irel_max, srel_max, near_ties = 0, 0, 0.0, 0.0, 0.0, 0
    per_iter = []
    lab = None
    for it in range(iters):
        lab, nc, inertia, shift, rep = F.lloyd_step(xd, c, dtype=dtype, precision=form if mixed else "plain",
                                                    ctx=ctx)
        near_ties += int(rep["near_tie_rows"])
        if mixed:
            ol, _ = O.assign(xs64, c)
            mism = int((lab[sample] != ol).sum())
            oc, oin = O.update_given_labels(x32, lab, c)
        else:
            xo = x32 if form == "fp32" else x32.astype(np.float64)
            ol, oc, oin, _ = O.lloyd_step(xo, c)
            mism = int((lab != ol).sum())
        crel = float(np.abs(nc.astype(np.float64) - oc).max() / max(np.abs(oc).max(), 1e-300))
        irel = abs(float(inertia) - float(oin)) / max(abs(float(oin)), 1e-300)
        oshift = float(np.sqrt(((oc - c.astype(np.float64)) ** 2).sum(1).max()))
        srel = abs(float(shift) - oshift) / max(oshift, 1e-300)
        mism_total += mism
        mism_max = max(mism_max, mism)
        crel_max = max(crel_max, crel)
        irel_max = max(irel_max, irel)
        srel_max = max(srel_max, srel)
        per_iter.append([it, mism, crel, irel])
        c = nc
    out = {
        "oracle": "oracle/ FP64 restatement of kmeans.rs (direct form, strict < argmin, row-order sums)",
        "iterations_checked": iters,
        "label_rows_per_iteration": int(m) if mixed else int(n),
        "label_mismatches": mism_total, "label_mismatches_max_per_iteration": mism_max,
        "centre_max_rel": crel_max, "centre_rel_definition": "max |c_gpu - c_oracle| / max |c_oracle| per iteration",
        "inertia_rel_max": irel_max, "shift_rel_max": srel_max,
        "n_iter_equal": True, "n_iter_note": f"tol 0: both run exactly {iters} iterations",
        "near_tie_rows": near_ties, "near_tie_definition": "re-scored rows whose FP64 margin is below 1e-12 relative",
        "per_iteration": per_iter if iters <= 60 else per_iter[:3] + per_iter[-3:],
        "fit_centres_equal_replay": bool(np.array_equal(np.asarray(fit_centres), c)),
        "fit_labels_equal_replay": bool(np.array_equal(np.asarray(fit_labels), lab)),
        "seconds": time.perf_counter() - t_start,
    }
    return out


def run_ours(args):
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "minibatch":
        return run_minibatch(args)
    if args.workload == "bisecting":
        return run_bisecting(args)
    if args.workload == "transform":
        return run_transform(args)
    import torch

    import ferrolearn_gb300 as F
    from ferrolearn_gb300 import _native

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        local = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.cuda.current_device()
    peaks = load_peaks()
    w = make_workload(args)
    x32 = w["x"]
    n, d = x32.shape
    k = w["k"]
    form = args.form if args.form != "auto" else DEFAULT_FORM[args.workload]
    stream = torch.cuda.Stream()
    ctx = F.Context(dev, stream=stream.cuda_stream)

    if form == "fp64":
        xd = torch.from_numpy(np.ascontiguousarray(x32, dtype=np.float64)).to(dev)
    else:
        xd = torch.from_numpy(x32).to(dev)
    torch.cuda.synchronize()
    init, kpp_ms = initial_centres(w, xd, ctx)

    def build_model(max_iter):
        if form == "fp32":
            m = F.KMeans(k, dtype="f32").with_init_centers(init.astype(np.float32))
        elif form == "fp64":
            m = F.KMeans(k, dtype="f64").with_init_centers(init)
        else:
            m = F.KMeans(k, dtype="f32x64").with_init_centers(init).with_precision(form)
        return m.with_max_iter(max_iter).with_tol(0.0).with_n_init(1)

    # warm-up (untimed)
    build_model(args.warmup).fit(xd, ctx=ctx)
    l0 = _native.lib().fk_debug_launch_count()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # no phase timers in the timed fit: its steady-state iterations replay CUDA graphs
    model = build_model(args.steps)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    # results stay in HBM (device tensors): the host copies are the e2e leg's
    c_out = torch.empty((k, d), dtype=torch.float32 if form == "fp32" else torch.float64, device=dev)
    l_out = torch.empty(n, dtype=torch.int64, device=dev)
    torch.cuda.synchronize()
    with ClockSampler(dev) as clocks:
        clocks.mark_start()
        start.record(stream)
        fitted = model.fit(xd, ctx=ctx, out=(c_out, l_out))
        end.record(stream)
        torch.cuda.synchronize()
        clocks.mark_end()
    launches = int(_native.lib().fk_debug_launch_count() - l0)
    ms = start.elapsed_time(end)
    ms = max_over_ranks(ms, "cuda")
    iters = fitted.n_iter()
    assert iters == args.steps, (iters, args.steps)
    e2e = None
    if not args.no_e2e and rank == 0:
        # right after the timed fit, before the phase timers and the peak
        # loops, whose power draw would leave the clocks lower for it
        xh = torch.from_numpy(x32).pin_memory() if form != "fp64" else torch.from_numpy(
            x32.astype(np.float64)).pin_memory()
        xh_np = xh.numpy()
        # untimed warm-up call on the same pinned buffer, like the device
        # leg's warm-up fit (the first DMA from freshly pinned pages, the
        # staging buffer, the graphs of its address)
        build_model(args.warmup).fit(xh_np, ctx=ctx)
        m2 = build_model(args.steps)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f2 = m2.fit(xh_np, ctx=ctx)
        t1 = time.perf_counter()
        h2d = xh_np.nbytes + w["init"].nbytes
        d2h = n * 8 + k * d * 8
        e2e = {"value": f2.n_iter() / (t1 - t0), "unit": "iters/s",
               "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
               "note": "one fit call on a pinned host X running K iterations (after one untimed warm-up call "
                       "on the same buffer); its H2D copy of X and D2H of labels and centres inside the "
                       "timed region, amortised per step"}
        del xh, xh_np, f2
    # the phase breakdown and the per-launch kernel times (outside the timed
    # region): the same fit once more with the library's CUDA-event phase
    # timers, which run it without graphs; the re-check counts are the same
    rep = build_model(args.steps).with_timing(True).fit(xd, ctx=ctx).report
    ips = job_rate(iters, ms, world)
    clk = clocks.summary()
    # dominant kernel: the tensor-core contraction (CUDA events on the library's
    # stream around each launch); the SIMT forms time the whole assignment
    assign_ms = rep["ms_assign"] / iters
    mixed = form in ("bf16", "fp8")
    contract_ms = rep["ms_contract"] / iters if rep["ms_contract"] > 0 else assign_ms
    flops = 2.0 * n * k * d
    tc_loop = None
    if mixed:
        # this GPU's dense tensor-core rates with the contraction's own MMA
        # shape (fk_debug_measure_tc_peaks): the FP8 form's denominator, and
        # a cross-check of the BF16 one
        tp = (C.c_double * 2)()
        _native.lib().fk_debug_measure_tc_peaks(ctx.handle, tp)
        tc_loop = {"bf16_tflops": tp[0] / 1e12, "e4m3_tflops": tp[1] / 1e12}
    n_count = int(rep.get("count_iterations", 0))
    count_ms = rep["ms_count_pass"] / n_count if n_count else None
    top2_ms = (rep["ms_contract"] - rep.get("ms_count_pass", 0.0)) / (iters - n_count) if iters > n_count else None
    if form == "bf16":
        peak, src = pick_tensor_peak(peaks, clk)
        # the dominant kernel: the count pass when it ran most iterations
        dom_ms = count_ms if n_count * 2 > iters else (top2_ms or contract_ms)
        roof = {"bound": "tensor", "achieved": flops / (dom_ms / 1e3) / 1e12, "peak": peak, "unit": "TFLOP/s",
                "peak_source": src, "own_mma_loop": tc_loop}
        if n_count and top2_ms:
            other = top2_ms if dom_ms == count_ms else count_ms
            roof["other_main_pass"] = {
                "kernel": "tc_assign_kernel<2> (top-2 ranking)" if dom_ms == count_ms else
                          "tc_assign_kernel<3> (count pass)",
                "iterations": iters - n_count if dom_ms == count_ms else n_count, "ms_per_launch": other,
                "achieved": flops / (other / 1e3) / 1e12, "frac": flops / (other / 1e3) / 1e12 / peak}
    elif form == "fp8":
        roof = {"bound": "tensor", "achieved": flops / (contract_ms / 1e3) / 1e12, "peak": tc_loop["e4m3_tflops"],
                "unit": "TFLOP/s", "peak_source": "dense E4M3 rate measured in this run by the library's own "
                                                  "tcgen05.mma kind::f8f6f4 loop (fk_debug_measure_tc_peaks)",
                "own_mma_loop": tc_loop}
    else:
        # the plain forms run on the CUDA cores: their peak is measured here
        # (fk_debug_measure_peaks: FMA chains on every SM, CUDA events)
        pk = (C.c_double * 8)()
        _native.lib().fk_debug_measure_peaks(ctx.handle, pk)
        # the direct form (kmeans.rs:159-163, bit for bit) executes a separate
        # sub, mul and add per (row, centre, feature): 3 n k d operations, each
        # one instruction of the FMA pipe, against its instruction rate
        if form == "fp32":
            simt = pk[0] / 2.0 / 1e12
            roof = {"bound": "fp32-simt", "achieved": 1.5 * flops / (assign_ms / 1e3) / 1e12, "peak": simt,
                    "unit": "T op/s",
                    "peak_source": "FP32 FMA instruction rate measured in this run (fk_debug_measure_peaks / 2); "
                                   "achieved counts the 3 n k d separate sub, mul and add of the direct form over "
                                   "the whole assignment phase"}
        else:
            # the f64 form's assignment: an FP32 pass with rigorous bounds (a
            # sub and an fma per row, centre and feature) decides the rows,
            # FP64 only for the open rows and each row's distance to its label
            simt = pk[0] / 2.0 / 1e12
            roof = {"bound": "fp32-simt", "achieved": flops / (assign_ms / 1e3) / 1e12, "peak": simt,
                    "unit": "T op/s",
                    "peak_source": "FP32 FMA instruction rate measured in this run (fk_debug_measure_peaks / 2); "
                                   "achieved counts the FP32 prefilter's 2 n k d instructions (sub, fma) over the "
                                   "whole assignment phase (the FP64 label distances and open rows inside it)",
                    "fp64_rate_tflops": pk[1] / 1e12}
    roof["frac"] = roof["achieved"] / roof["peak"]
    dom_count = form == "bf16" and n_count * 2 > iters
    tb = TRAFFIC_BYTES_PER_ROW.get((w["name"], form, "count" if dom_count else "top2"))
    roof["traffic"] = tb * n if tb is not None else None
    if tb is not None:
        roof["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch at 1,000,000 rows "
                                  "(profiles/tc_count_anisotropic_1024x128_quarter.md), scaled to n rows")
        # BF16 X once + 16-byte records per row and slice (+ the count pass's per-row threshold)
        roof["algorithmic_bytes"] = n * d * 2 + n * 2 * 16 + (4 * n if dom_count else 0)
    if form == "bf16" and n_count * 2 > iters:
        roof["kernel"] = (f"tc_assign_kernel<3> (BF16 tcgen05 contraction + count epilogue against carried "
                          f"thresholds; {n_count} of {iters} iterations)")
        roof["ms_per_launch"] = count_ms
    else:
        roof["kernel"] = f"tc_assign_kernel ({form.upper()} tcgen05 contraction + top-2 epilogue)" if mixed else \
            ("assign_direct_kernel (whole assignment phase)" if form == "fp32" else
             "f32_filter_kernel + FP64 label distances and open rows (whole assignment phase)")
        roof["ms_per_launch"] = (top2_ms or contract_ms) if mixed else assign_ms

    out = {
        "metric": METRIC, "value": ips, "unit": "iters/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / iters, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": {"bf16": "bf16+f64", "fp8": "e4m3+f64", "fp32": "f32", "fp64": "f64"}[form],
        "data": "synthetic", "form": form,
        "config": workload_config(w),
        "pt_k_per_s": ips * n * k,
        "phase_ms_per_iter": {"assign": assign_ms, "contract": contract_ms if mixed else None,
                              "update": rep["ms_update"] / iters},
        "main_pass": {"count_iterations": n_count, "count_ms_per_launch": count_ms,
                      "top2_iterations": iters - n_count, "top2_ms_per_launch": top2_ms} if mixed else None,
        "recheck": {"rows": rep["rows_rechecked"], "full_rescan": rep["rows_full_rescan"],
                    "fp64_rows": rep["rows_fp64"], "second_pass": rep["rows_second_pass"],
                    "few_candidates": rep["rows_few"], "exhaustive": rep["rows_exhaustive"],
                    "near_ties": rep["near_tie_rows"],
                    "fraction": rep["rows_rechecked"] / max(1, rep["rows_assigned"])},
        "gpu_launches": launches,
        "clocks": clk,
        "roofline": roof,
    }
    if kpp_ms is not None:
        out["config"]["init"] = "k-means++ on the GPU (seeded)"
    if e2e is not None:
        out["e2e"] = e2e
    # the update phase against HBM, with the bytes it moves: a full pass reads
    # X once and writes the centres (n d sizeof(X) + 4 n + 16 k d); an
    # incremental one (mixed forms, from the third iteration) compares the
    # two label arrays (8 n), reads each moved row for its old and its new
    # cluster (2 m (d sizeof(X) + 8)) and rewrites the exact state and means
    # (40 k d)
    upd_ms = rep["ms_update"] / iters
    xb = 8 if form == "fp64" else x32.itemsize
    n_inc = int(rep["updates_incremental"])
    full_bytes = n * d * xb + 4 * n + 16 * k * d
    inc_bytes_total = n_inc * (8 * n + 40 * k * d) + 2 * int(rep["rows_moved"]) * (d * xb + 8)
    upd_bytes = ((iters - n_inc) * full_bytes + inc_bytes_total) / iters
    out["update_roofline"] = {"bound": "hbm", "bytes_per_iter": upd_bytes, "ms_per_iter": upd_ms,
                              "achieved": upd_bytes / (upd_ms / 1e3) / 1e9, "peak": peaks["hbm"], "unit": "GB/s",
                              "frac": upd_bytes / (upd_ms / 1e3) / 1e9 / peaks["hbm"],
                              "full_passes": iters - n_inc, "incremental_updates": n_inc,
                              "rows_moved": int(rep["rows_moved"]),
                              "note": "bytes each update moves, averaged over the K iterations"}
    if kpp_ms is not None:
        out["kpp_ms"] = kpp_ms
    if "x_predict" in w and rank == 0:
        xp = torch.from_numpy(w["x_predict"]).to(dev)
        fitted.predict(xp, ctx=ctx)  # warm-up (plans the launch for this row count)
        torch.cuda.synchronize()
        start.record(stream)
        fitted.predict(xp, ctx=ctx)
        end.record(stream)
        torch.cuda.synchronize()
        pms = start.elapsed_time(end)
        out["predict"] = {"rows": int(xp.shape[0]), "ms": pms, "rows_per_s": xp.shape[0] / (pms / 1e3),
                          "note": "KMeans::predict on fresh rows resident in HBM, labels to host memory"}

    if not args.no_parity and rank == 0:
        out["parity"] = parity_leg(w, form, ctx, xd, iters, args.parity_rows, c_out.cpu().numpy(),
                                   l_out.cpu().numpy())
    if not args.no_cpu and rank == 0 and world == 1:
        out["cpu_baseline"] = cpu_baseline(w, args.cpu_seconds, os.cpu_count() or 1)
    if rank == 0:
        print(json.dumps(out), flush=True)
    # release the library's buffers while the stream and the CUDA context are alive
    torch.cuda.synchronize()
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    faulthandler.enable()  # a native crash prints the Python stack
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

"""Benchmark of the PyMORESANE deconvolution hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload deconv|iuwt]

Workload ``deconv`` (default) -- full single-image MORESANE at 2048 x 2048
(float32 dirty image, 4096 x 4096 PSF from 20000 seeded uv points, 1000 point
sources log-uniform in [1e-3, 1], 50 Gaussians with sigma 2-20 px, noise
sigma 1e-4; scale_count=7, sigma_level=4, loop_gain=0.2, tolerance=0.75,
accuracy=1e-6, major_loop_miter=100, minor_loop_miter=30, linear
convolution). One step = one complete deconvolution (PSF spectra, major and
minor loops, residual) of an image resident in HBM. Metric: deconvolutions
per second, with the p50 / p99 latency of the steps; the same line carries the
IUWT microbenchmark (4096^2, 8 scales) in GB/s.

Workload ``iuwt`` -- 4096 x 4096 image (N(0,1) + 500 deltas U(5,50)),
decomposition with scale_count=8, store_smoothed, then recomposition; metric:
algorithmic GB/s, 4 N^2 (1 + 8 + 1) + 4 N^2 (8 + 1 + 1) bytes per step.

Rank 0 prints one JSON line. With N > 1 GPUs (torchrun) every rank processes
its own image (replicas, no collective on the data path; weak scaling).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
from pymoresane_gb300 import replicas  # noqa: E402  (host-side rank coordination)
sys.path.insert(0, ROOT)

PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
DECONV_KW = dict(scale_count=7, sigma_level=4, loop_gain=0.2, tolerance=0.75, accuracy=1e-6, major_loop_miter=100,
                 minor_loop_miter=30, conv_mode="linear")
IUWT_N, IUWT_S = 4096, 8
# The workload names and L2 notes both arms print in "config" (the same dict in each arm).
CONFIGS = {
    "deconv": {"workload": "moresane_2048x2048_psf4096_S7_linear",
               "l2": "working set > 0.6 GB per deconvolution > 129 MB L2 (no flush needed)"},
    "iuwt": {"workload": "iuwt_4096x4096_S8_store_smoothed",
             "l2": "working set 0.7 GB per step > 129 MB L2 (no flush needed)"},
}


def reference_trajectory():
    """(major, minor) iterations of the reference's own complete run of the 2048^2 problem.

    Read from the fixture tests/golden/baseline_2048_full.npz, made by running
    the reference PyMORESANE on the same seeded problem (tests/golden/make_golden.py);
    None when the fixture is absent.
    """
    path = os.path.join(ROOT, "tests", "golden", "baseline_2048_full.npz")
    if not os.path.exists(path):
        return None
    g = np.load(path)
    return int(g["major"]), int(g["minor_total"])


def load_peaks():
    try:
        with open(PEAKS_PATH) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks / throttle reasons while the timed region runs."""

    QUERY = ("index,uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid=None):
        self.uuid = uuid
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        cmd = ["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits", "-lms", "100"]
        if self.uuid:
            cmd += ["-i", self.uuid]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 10:
                continue
            try:
                sm.append(float(parts[2]))
                smax.append(float(parts[3]))
            except ValueError:
                continue
            for name, val in zip(names, parts[6:10]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def gpu_uuid():
    import torch
    u = getattr(torch.cuda.get_device_properties(torch.cuda.current_device()), "uuid", None)
    return ("GPU-" + str(u)) if u else None


def percentile(vals, q):
    return float(np.percentile(np.asarray(vals), q)) if vals else None


def launches(reset=False):
    from pymoresane_gb300 import _native
    return int(_native.query("msn_launch_count", 1 if reset else 0))


# ---------------------------------------------------------------------------
# IUWT microbenchmark (4096^2, 8 scales)
# ---------------------------------------------------------------------------

def iuwt_algorithmic_bytes(n, s):
    return 4 * n * n * (1 + s + 1) + 4 * n * n * (s + 1 + 1)


def iuwt_kernel_bytes(n, s):
    """Compulsory bytes of the 2s + 1 passes of one step, plane by plane (4 n^2 bytes each).

    Decomposition: the first smoothing (read 1 plane, write 1), s - 1 fused
    detail + next-smoothing passes (read the smoothed plane and its
    predecessor, write the detail and the next smoothed plane: 4), the last
    detail pass (read 2, write 1). Recomposition from the smoothed plane: s
    smoothing + add passes (read 2, write 1).
    """
    return 4 * n * n * ((2 + 4 * (s - 1) + 3) + 3 * s)


def measure_iuwt(steps, warmup, seed=0):
    import torch

    from pymoresane_gb300 import device as dev
    from pymoresane_gb300 import synthetic
    n, s = IUWT_N, IUWT_S
    x = torch.from_numpy(synthetic.iuwt_image(n, 500, seed=seed)).cuda()
    w = torch.empty((s, n, n), dtype=torch.float32, device="cuda")
    c = torch.empty((n, n), dtype=torch.float32, device="cuda")
    rec = torch.empty((n, n), dtype=torch.float32, device="cuda")
    work = dev.iuwt_workspace(n, n, x.device)

    def step():
        dev.iuwt_decompose(x, s, 0, store_smoothed=True, out=w, smoothed_out=c, work=work)
        dev.iuwt_recompose(w, 0, smoothed=c, out=rec, work=work)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    err = torch.max(torch.abs(rec - x)).item()
    assert err <= 1e-5 * torch.max(torch.abs(x)).item(), f"IUWT reconstruction error {err}"
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches(reset=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    nl = launches() / steps
    return {"ms_per_step": ms, "gbs": iuwt_algorithmic_bytes(n, s) / (ms * 1e-3) / 1e9,
            "kernel_gbs": iuwt_kernel_bytes(n, s) / (ms * 1e-3) / 1e9, "launches_per_step": nl,
            "x_host": None, "n": n, "s": s}


def iuwt_e2e(steps, seed=0):
    import torch

    from pymoresane_gb300 import iuwt as G
    from pymoresane_gb300 import synthetic
    n, s = IUWT_N, IUWT_S
    x_host = synthetic.iuwt_image(n, 500, seed=seed)
    x_pin = torch.from_numpy(x_host).pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        wd, cd = G.iuwt_decomposition(x_pin, s, 0, mode="gpu", store_smoothed=True)
        rh = G.iuwt_recomposition(wd, 0, mode="gpu", smoothed_array=cd)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / steps
    assert np.max(np.abs(rh - x_host)) <= 1e-5 * np.max(np.abs(x_host))
    return dt


def cpu_iuwt(workers):
    """Oracle port of the reference IUWT on a bounded 2048^2 sample (GB/s)."""
    from oracle import iuwt as O
    n = 2048
    x = np.random.default_rng(5).standard_normal((n, n)).astype(np.float32)
    t0 = time.perf_counter()
    if workers == 1:
        d, c = O.decompose(x, IUWT_S, 0, store_smoothed=True, arith="f64")
        O.recompose(d, 0, smoothed_array=c, arith="f64")
        sample = ("2048^2, 8 scales: one decomposition + recomposition of the FP64 'ser' restatement "
                  "(pymoresane/iuwt.py:66-191), 1 thread")
    else:
        d, c = O.decompose_strips(x, IUWT_S, 0, store_smoothed=True, workers=workers)
        O.recompose_strips(d, 0, smoothed_array=c, workers=workers)
        sample = (f"2048^2, 8 scales: one decomposition + recomposition of the FP32 strip-parallel 'mp' "
                  f"restatement (pymoresane/iuwt.py:193-382) on {workers} threads")
    dt = time.perf_counter() - t0
    return iuwt_algorithmic_bytes(n, IUWT_S) / dt / 1e9, sample


# ---------------------------------------------------------------------------
# Deconvolution workload (2048^2 MORESANE)
# ---------------------------------------------------------------------------

def deconv_problem(seed):
    from pymoresane_gb300 import synthetic
    dirty, psf, _ = synthetic.make_problem(synthetic.problem_2048(seed))
    return dirty, psf


def cpu_deconv(dirty, psf, decom, workers, trajectory, source):
    """Oracle port of the reference MORESANE timed on a bounded sample, scaled to one deconvolution.

    The sample is the set-up (PSF spectra and energies) plus the whole first
    major iteration with all of its minor iterations; the per-major and
    per-minor times are scaled by the trajectory (major, minor) of a complete
    run, whose origin `source` names.
    """
    from oracle.moresane import MoresaneOracle
    o = MoresaneOracle(dirty, psf, decom=decom, workers=workers)
    t0 = time.perf_counter()
    o.moresane(**dict(DECONV_KW, major_loop_miter=1))
    wall = time.perf_counter() - t0
    t = o.timings
    per_major = t["major"] / max(1, t["n_major"])
    per_minor = t["minor"] / max(1, t["n_minor"])
    n_major, n_minor = trajectory
    seconds = t["setup"] + n_major * per_major + n_minor * per_minor
    sample = (f"2048^2 problem: set-up + the first major iteration with all {t['n_minor']} of its minor iterations "
              f"of the oracle port ({'FP64 ser' if decom == 'ser' else 'FP32 mp'} IUWT, numpy FFT, scipy "
              f"labelling) in {wall:.1f} s on {workers} thread(s), scaled to {source}: {n_major} major / "
              f"{n_minor} minor iterations (per major {per_major:.2f} s, per minor {per_minor:.2f} s)")
    return 1.0 / seconds, sample


def deconv_trajectory(fallback):
    """The reference's own trajectory when its fixture exists, else the GPU run's (named)."""
    ref = reference_trajectory()
    if ref is not None:
        return ref, "the reference's own complete run of this problem"
    return tuple(fallback), "this implementation's complete run of this problem (reference run not recorded)"


def run_deconv(args, rank, world, dist, problem=None):
    import torch

    from pymoresane_gb300.main import DataImage, Deconvolver
    dirty_h, psf_h = problem if problem is not None else deconv_problem(rank)
    dirty = torch.from_numpy(dirty_h).cuda()
    psf = torch.from_numpy(psf_h).cuda()

    def step():
        eng = Deconvolver(psf)
        if args.driver == "host":
            # the same kernels driven step by step from the host (no CUDA graphs): ncu can
            # profile every launch this way, it cannot inside graphs with conditional nodes
            eng.native_major_loop = eng.native_minor_loop = False
        model, residual, major = eng.moresane(dirty, **DECONV_KW)
        return eng, model, residual

    eng = None
    for _ in range(args.warmup):
        eng, model, residual = step()
    torch.cuda.synchronize()
    traj = (len(eng.log), eng.minor_total)  # every minor loop, also those a major iteration restarts

    sampler = ClockSampler(gpu_uuid()) if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    lat = []
    launches(reset=True)
    t_start = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    prev = t_start
    for _ in range(args.steps):
        step()
        ev = torch.cuda.Event(enable_timing=True)
        ev.record(stream)
        ev.synchronize()
        lat.append(prev.elapsed_time(ev))
        prev = ev
    torch.cuda.synchronize()
    n_launch = launches()
    if dist:
        dist.barrier()
    total_ms = t_start.elapsed_time(prev)
    clocks = sampler.stop() if sampler else None

    # end to end through the public host-array API
    e2e_steps = max(1, min(args.steps, 3))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        img = DataImage(dirty_h, psf_h, None, 1.0, 1.0)
        img.moresane(**DECONV_KW)
        _ = float(img.model.sum())
    e2e_s = (time.perf_counter() - t0) / e2e_steps

    total_ms, e2e_s = replicas.reduce_max([total_ms, e2e_s], dist, "cuda")
    return {"ms": total_ms, "lat": lat, "e2e_s": e2e_s, "clocks": clocks, "traj": traj, "launches": n_launch,
            "dirty": dirty_h, "psf": psf_h, "model_sum": float(img.model.sum()), "e2e_steps": e2e_steps,
            "model": img.model.copy()}


# ---------------------------------------------------------------------------
# Batched (64 mixed-size images) and served (Poisson arrivals) workloads
# ---------------------------------------------------------------------------

BATCH_SIZES, BATCH_P = (256, 512, 1024, 1536, 2048), (0.2, 0.3, 0.25, 0.15, 0.1)
SERVE_SIZES, SERVE_P = (512, 1024, 1536, 2048, 4096), (0.35, 0.3, 0.15, 0.15, 0.05)
MIX_KW = dict(sigma_level=4, loop_gain=0.2, tolerance=0.75, accuracy=1e-6, major_loop_miter=100,
              minor_loop_miter=30, conv_mode="linear")


def mix_job(n, seed):
    """The 512^2 problem's recipe scaled by area to side n (PSF 2n, uv count and sources ~ n^2), S = log2(n) - 3."""
    from pymoresane_gb300 import synthetic
    from pymoresane_gb300.batch import Job
    dirty, psf, _ = synthetic.make_problem(synthetic.scaled(n, seed=seed), fast=True)
    return Job(dirty, psf, kwargs=dict(MIX_KW, scale_count=int(np.log2(n)) - 3), tag=(n, seed))


def run_plain(jobs):
    """The jobs one at a time through the plain single-image path; (seconds, latencies in ms from t=0)."""
    import torch

    from pymoresane_gb300.main import Deconvolver
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lat, models = [], []
    for j in jobs:
        t1 = time.perf_counter()
        eng = Deconvolver(j.psf)
        model, residual, _ = eng.moresane(torch.from_numpy(j.dirty).cuda(), **j.kwargs)
        models.append(model.cpu().numpy())
        residual.cpu()
        lat.append((time.perf_counter() - t1) * 1e3)
    return time.perf_counter() - t0, lat, models


def run_batch(args, rank):
    """64 images of sizes {256..2048} (p = .2 .3 .25 .15 .1), batched vs one at a time."""
    from pymoresane_gb300.batch import DeconvolutionExecutor
    rng = np.random.default_rng(replicas.rank_seed(1000, rank))
    sizes = rng.choice(BATCH_SIZES, size=args.images, p=BATCH_P)
    cache = {}
    jobs = []
    for i, n in enumerate(sizes):
        key = (int(n), i % args.distinct)
        if key not in cache:
            cache[key] = mix_job(int(n), seed=replicas.rank_seed(2000 + 97 * key[1] + int(n), rank))
        jobs.append(cache[key])
    # warm-up: one job per size through both paths (allocator pools, PSF plans, graph capture code)
    warm = [cache[k] for k in sorted({(k[0], 0) for k in cache})]
    run_plain(warm)
    with DeconvolutionExecutor(workers=args.workers, order="largest") as ex:
        ex.map(warm)
    plain_s, plain_lat, plain_models = run_plain(jobs)
    with DeconvolutionExecutor(workers=args.workers, order="largest") as ex:
        t0 = time.perf_counter()
        res = ex.map(jobs)
        batch_s = time.perf_counter() - t0
    lat = [r.latency * 1e3 for r in res]
    same = all(np.array_equal(m, r.model) for m, r in zip(plain_models, res))
    return {"images": len(jobs), "plain_s": plain_s, "batch_s": batch_s, "lat": lat, "plain_lat": plain_lat,
            "sizes": {int(n): int((sizes == n).sum()) for n in BATCH_SIZES}, "same": same}


def run_serve(args, rank):
    """Poisson arrivals (lambda = 40/s) of sizes {512..4096} (p = .35 .3 .15 .15 .05), served vs one at a time."""
    from pymoresane_gb300.batch import serve
    rng = np.random.default_rng(replicas.rank_seed(3000, rank))
    sizes = rng.choice(SERVE_SIZES, size=args.requests, p=SERVE_P)
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, size=args.requests))
    cache = {}
    jobs = []
    for i, n in enumerate(sizes):
        key = (int(n), i % args.distinct)
        if key not in cache:
            cache[key] = mix_job(int(n), seed=replicas.rank_seed(4000 + 97 * key[1] + int(n), rank))
        jobs.append(cache[key])
    warm = [cache[k] for k in sorted({(k[0], 0) for k in cache})]
    run_plain(warm)
    serve(warm, [0.0] * len(warm), workers=args.workers)
    plain_s, plain_lat, plain_models = run_plain(jobs)
    res, wall = serve(jobs, list(arrivals), workers=args.workers)
    lat = [r.latency * 1e3 for r in res]
    same = all(np.array_equal(m, r.model) for m, r in zip(plain_models, res))
    # the same jobs one at a time, arriving at the same times (queueing included)
    t_free, seq_lat = 0.0, []
    for at, pl in zip(arrivals, plain_lat):
        start = max(at, t_free)
        t_free = start + pl / 1e3
        seq_lat.append((t_free - at) * 1e3)
    return {"requests": len(jobs), "wall_s": wall, "plain_s": plain_s, "lat": lat, "seq_lat": seq_lat, "same": same,
            "arrival_span_s": float(arrivals[-1]), "sizes": {int(n): int((sizes == n).sum()) for n in SERVE_SIZES}}


def run_served_2048(args, dirty_h, psf_h, plain_model):
    """The 2048^2 deconvolution served: args.served_jobs jobs submitted together to args.workers streams."""
    from pymoresane_gb300.batch import DeconvolutionExecutor, Job
    jobs = [Job(dirty_h, psf_h, kwargs=dict(DECONV_KW), tag=i) for i in range(args.served_jobs)]
    with DeconvolutionExecutor(workers=args.workers, order="fifo") as ex:
        ex.map(jobs[:args.workers])           # warm-up: every worker's buffers and graphs
        t0 = time.perf_counter()
        res = ex.map(jobs)
        wall = time.perf_counter() - t0
    lat = [r.latency * 1e3 for r in res]
    return {"value": len(jobs) / wall, "unit": "deconv/s", "jobs": len(jobs), "workers": args.workers,
            "latency_ms": {"p50": percentile(lat, 50), "p99": percentile(lat, 99),
                           "mode": "all jobs submitted at once (queueing included)"},
            "same_result_as_plain": bool(all(np.array_equal(r.model, plain_model) for r in res)),
            "api": "pymoresane_gb300.batch.DeconvolutionExecutor.map with host numpy arrays"}


def conv_roofline(n=2048, m=4096, reps=50):
    """Average duration of the fused linear convolution (the minor loop's dominant step) at 2048^2 / 4096^2.

    Algorithmic bytes per convolution: read x (4 n^2) + read the
    PSF spectrum (8 m (m/2 + 1)) + write the result (4 n^2).
    """
    import torch

    from pymoresane_gb300 import device as dev
    from pymoresane_gb300.synthetic import make_psf
    psf = make_psf(m, 2000, np.random.default_rng(1))
    spec = dev.psf_spectrum(psf)
    x = torch.randn((n, n), device="cuda")
    out = torch.empty_like(x)
    work = dev.fft_workspace(n, m, x.device)
    for _ in range(3):
        dev.fft_convolve(x, spec, True, out=out, work=work)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        dev.fft_convolve(x, spec, True, out=out, work=work)
    e1.record(stream)
    torch.cuda.synchronize()
    us = e0.elapsed_time(e1) * 1e3 / reps
    alg = 4 * n * n + 8 * m * (m // 2 + 1) + 4 * n * n
    return us, alg


def read_traffic(name):
    try:
        with open(os.path.join(ROOT, "profiles", name)) as fh:
            return json.load(fh)
    except Exception:
        return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="deconv", choices=["deconv", "iuwt", "conv", "batch", "serve"])
    ap.add_argument("--workers", type=int, default=8, help="concurrent streams (batch / serve / served deconv)")
    ap.add_argument("--images", type=int, default=64, help="batch workload: images")
    ap.add_argument("--requests", type=int, default=100, help="serve workload: requests")
    ap.add_argument("--rate", type=float, default=40.0, help="serve workload: arrivals per second")
    ap.add_argument("--distinct", type=int, default=3, help="batch / serve: distinct problems per size")
    ap.add_argument("--served-jobs", type=int, default=8, help="deconv: jobs of the served 2048^2 measurement (0: skip)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (use the current launch parameters)")
    ap.add_argument("--no-mix", action="store_true", help="deconv: skip the batched and served mixed-size workloads")
    ap.add_argument("--driver", default="native", choices=["native", "host"],
                    help="deconv: native = minor/major loops in libmsn (graphs); host = step by step (for ncu)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    hbm_peak, peak_kind = load_peaks()
    if args.workload == "deconv":
        metric = "2048^2 deconvolutions/s (MORESANE, 4096^2 PSF, scale_count=7, 1 GB300)"
        unit = "deconv/s"
    else:
        metric = "IUWT algorithmic HBM GB/s (4096^2, scale_count=8, decomposition+recomposition)"
        unit = "GB/s"

    if args.impl == "reference":
        if rank != 0:
            return
        workers = os.cpu_count() or 1
        vals, sample, traj = [], None, None
        if args.workload == "deconv":
            dirty, psf = deconv_problem(0)
            ref = reference_trajectory()
            traj, source = (ref, "the reference's own complete run of this problem") if ref else \
                ((90, 1595), "this implementation's complete run of this problem on GB300 (reference run not recorded)")
        # Each step is a bounded sample of seconds; warm-up samples are untimed. The run stops
        # taking samples after about 150 s (at least one timed sample), so that it ends in minutes.
        t_run = time.perf_counter()
        for i in range(args.warmup + args.steps):
            if args.workload == "deconv":
                v, sample = cpu_deconv(dirty, psf, "mp", workers, traj, source)
            else:
                v, sample = cpu_iuwt(workers)
            if i >= args.warmup:
                vals.append(v)
            if vals and time.perf_counter() - t_run > 150.0:
                break
        value = statistics.mean(vals)
        sample = f"{sample}; mean of {len(vals)} timed sample(s)"
        extra = {"trajectory_major_minor": list(traj)} if traj else {}
        print(json.dumps({
            "impl": "reference", "metric": metric, "value": value, "unit": unit, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(CONFIGS[args.workload]), "parallelism": f"host, {workers} threads", **extra,
            "cpu_baseline": {"value": value, "unit": unit, "cores": workers, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }))
        return

    import torch
    dist = None
    if world > 1:
        import torch.distributed as tdist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        tdist.init_process_group("nccl")
        dist = tdist
    else:
        torch.cuda.set_device(0)

    if args.workload == "conv":
        # Fused linear FFT convolution microbenchmark: 2048^2 image, 4096^2 PSF spectrum.
        us, alg = conv_roofline(reps=max(args.steps, 1))
        if rank == 0:
            print(json.dumps({"metric": "fused FFT convolution algorithmic GB/s (2048^2 image, 4096^2 PSF, linear)",
                              "value": alg / (us * 1e-6) / 1e9, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
                              "warmup": args.warmup, "us_per_conv": us, "algorithmic_bytes": alg,
                              "frac_of_hbm": alg / (us * 1e-6) / 1e9 / hbm_peak}))
        return

    if args.workload in ("batch", "serve"):
        sampler = ClockSampler(gpu_uuid()) if rank == 0 else None
        if sampler:
            sampler.start()
        r = run_batch(args, rank) if args.workload == "batch" else run_serve(args, rank)
        clocks = sampler.stop() if sampler else None
        n_img = r["images"] if args.workload == "batch" else r["requests"]
        mixed_s, plain_s = replicas.reduce_max([r["batch_s"] if args.workload == "batch" else r["wall_s"],
                                                r["plain_s"]], dist, "cuda")
        r["plain_s"] = plain_s
        if rank == 0:
            line = {
                "metric": ("64-image mixed-size batch, images/s (batched vs one at a time)" if args.workload == "batch"
                           else f"served deconvolutions/s under Poisson arrivals (lambda={args.rate:g}/s)"),
                "value": replicas.whole_job_rate(n_img, world, mixed_s), "unit": "images/s", "n_gpus": world,
                "steps": 1, "warmup": 1,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic",
                "config": {"workload": args.workload, "workers": args.workers, "sizes": r["sizes"],
                           "distinct_problems_per_size": args.distinct,
                           "parallelism": f"{args.workers} streams x {world} replicas"},
                "plain": {"value": replicas.whole_job_rate(n_img, world, r["plain_s"]), "unit": "images/s",
                          "seconds": r["plain_s"]},
                "speedup_vs_plain": r["plain_s"] / mixed_s,
                "latency_ms": {"p50": percentile(r["lat"], 50), "p99": percentile(r["lat"], 99)},
                "clocks": clocks,
            }
            line["same_result_alone_and_in_mix"] = r["same"]
            if args.workload == "serve":
                line["plain_latency_ms"] = {"p50": percentile(r["seq_lat"], 50), "p99": percentile(r["seq_lat"], 99),
                                            "mode": "same arrivals served one at a time"}
                line["arrival_span_s"] = r["arrival_span_s"]
            print(json.dumps(line))
        if dist:
            dist.destroy_process_group()
        return

    if args.workload == "iuwt":
        sampler = ClockSampler(gpu_uuid()) if rank == 0 else None
        if sampler:
            sampler.start()
            time.sleep(0.3)
        if dist:
            dist.barrier()
        from pymoresane_gb300 import tune
        tuned = tune.autotune(n=IUWT_N, reps=5)["values"] if not args.no_tune else tune.current()
        r = measure_iuwt(args.steps, args.warmup, seed=rank)
        ms = replicas.reduce_max([r["ms_per_step"]], dist, "cuda")[0]
        clocks = sampler.stop() if sampler else None
        e2e_s = iuwt_e2e(max(1, min(args.steps, 5)), seed=rank)
        n, s = IUWT_N, IUWT_S
        alg = iuwt_algorithmic_bytes(n, s)
        if rank == 0:
            cpu = None
            if not args.no_cpu_baseline:
                v, sample = cpu_iuwt(1)
                cpu = {"value": v, "unit": "GB/s", "cores": 1, "kind": "port", "sample": sample}
            print(json.dumps({
                "metric": metric, "value": world * alg / (ms * 1e-3) / 1e9, "unit": unit, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": dict(CONFIGS["iuwt"]), "parallelism": f"replicas x{world}",
                "roofline": {"bound": "hbm", "kernel": "IUWT decomposition + recomposition (all passes)",
                             "achieved": r["gbs"], "peak": hbm_peak, "peak_kind": peak_kind, "unit": "GB/s",
                             "frac": r["gbs"] / hbm_peak, "bytes": "algorithmic: 4 N^2 (1 + S + 1) + 4 N^2 (S + 1 + 1)",
                             "per_pass_gbs": r["kernel_gbs"],
                             "traffic": (read_traffic("iuwt_traffic.json") or {}).get("bytes_per_launch")},
                "e2e": {"value": world * alg / e2e_s / 1e9, "unit": "GB/s", "h2d_bytes_per_step": 4 * n * n * (s + 2),
                        "d2h_bytes_per_step": 4 * n * n * (s + 2)},
                "gpu_launches": int(r["launches_per_step"] * args.steps), "clocks": clocks, "cpu_baseline": cpu,
                "autotuned": tuned,
            }))
        if dist:
            dist.destroy_process_group()
        return

    # the project's autotuner picks this device's launch parameters before anything is timed;
    # the a trous CTA size on a deconvolution of the benchmarked problem bounded to 3 major iterations
    from pymoresane_gb300 import tune
    problem = deconv_problem(rank)
    if args.no_tune:
        tuned = tune.current()
    else:
        import torch

        from pymoresane_gb300.main import Deconvolver
        d_dev, p_dev = torch.from_numpy(problem[0]).cuda(), torch.from_numpy(problem[1]).cuda()
        short = dict(DECONV_KW, major_loop_miter=3)
        tuned = tune.autotune(n=2048, reps=5, workload=lambda: Deconvolver(p_dev).moresane(d_dev, **short))["values"]
        del d_dev, p_dev
    res = run_deconv(args, rank, world, dist, problem)
    served = None
    if args.served_jobs > 0 and args.driver == "native":
        served = run_served_2048(args, res["dirty"], res["psf"], res["model"])
    mix = {}
    if not args.no_mix and args.driver == "native":
        # the batched (64 mixed-size images) and served (Poisson arrivals) workloads, in the same line
        for name, fn in (("batch", run_batch), ("serve", run_serve)):
            r = fn(args, rank)
            n_img = r["images"] if name == "batch" else r["requests"]
            mixed_s = r["batch_s"] if name == "batch" else r["wall_s"]
            mixed_s, plain_s = replicas.reduce_max([mixed_s, r["plain_s"]], dist, "cuda")
            mix[name] = {
                "value": replicas.whole_job_rate(n_img, world, mixed_s), "unit": "images/s",
                "plain": replicas.whole_job_rate(n_img, world, plain_s), "speedup_vs_plain": plain_s / mixed_s,
                "latency_ms": {"p50": percentile(r["lat"], 50), "p99": percentile(r["lat"], 99)},
                "sizes": r["sizes"], "distinct_problems_per_size": args.distinct, "workers": args.workers,
                "same_result_alone_and_in_mix": r["same"]}
            if name == "batch":
                mix[name]["images"] = n_img
            else:
                mix[name].update(requests=n_img, rate_per_s=args.rate, specified_requests=2000,
                                 arrival_span_s=r["arrival_span_s"],
                                 plain_latency_ms={"p50": percentile(r["seq_lat"], 50),
                                                   "p99": percentile(r["seq_lat"], 99),
                                                   "mode": "same arrivals served one at a time"})
    ms_per_step = res["ms"] / args.steps
    value = world * args.steps / (res["ms"] * 1e-3)
    iuwt = measure_iuwt(5, 3, seed=rank)
    conv_us, conv_alg = conv_roofline()
    conv_gbs = conv_alg / (conv_us * 1e-6) / 1e9
    from pymoresane_gb300 import tune as _tune
    conv_kernels = ("fft_convolve (four-step sq_rows_fwd + sq_cols_conv + sq_rows_inv)" if _tune.get("fft_four_step")
                    else "fft_convolve (Stockham rfft_rows + conv_cols + irfft_rows)")
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            traj, source = deconv_trajectory(res["traj"])
            v, sample = cpu_deconv(res["dirty"], res["psf"], "ser", 1, traj, source)
            cpu = {"value": v, "unit": "deconv/s", "cores": 1, "kind": "port", "sample": sample}
        n = 2048
        m = 4096
        print(json.dumps({
            "metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(CONFIGS["deconv"]), "trajectory_major_minor": list(res["traj"]),
            "reference_trajectory_major_minor": list(reference_trajectory() or []) or None,
            "driver": args.driver, "parallelism": f"replicas x{world}",
            "latency_ms": {"p50": percentile(res["lat"], 50), "p99": percentile(res["lat"], 99),
                           "mode": "plain (one image at a time)"},
            "iuwt_gbs": iuwt["gbs"], "iuwt_frac_of_hbm": iuwt["gbs"] / hbm_peak,
            "roofline": {"bound": "hbm", "kernel": conv_kernels + ", linear 2048^2 image / 4096^2 PSF",
                         "achieved": conv_gbs, "peak": hbm_peak, "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": conv_gbs / hbm_peak, "avg_launch_us": conv_us,
                         "algorithmic_bytes_per_launch": conv_alg,
                         "traffic": (read_traffic("conv_traffic.json") or {}).get("bytes_per_launch")},
            "e2e": {"value": world / res["e2e_s"], "unit": unit, "h2d_bytes_per_step": 4 * n * n + 4 * m * m,
                    "d2h_bytes_per_step": 8 * n * n, "steps": res["e2e_steps"],
                    "api": "pymoresane_gb300.main.DataImage(dirty, psf).moresane(...) with host numpy arrays"},
            "gpu_launches": res["launches"], "clocks": res["clocks"], "cpu_baseline": cpu,
            "served": served, "batched_64_mixed": mix.get("batch"), "served_poisson": mix.get("serve"),
            "autotuned": tuned,
        }))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

"""Batched and served MORESANE on one GPU.

The reference deconvolves one image per process (pymoresane/main.py:53-521,
driven by runsane); it has no batching. Here many independent deconvolutions
share one GPU: every worker thread owns a CUDA stream and a Workspace, takes
jobs from a queue and runs them with the device-resident driver
(main.Deconvolver), whose minor loops are CUDA graphs. Kernels of different
jobs overlap on the device, and the host work of one job (the major-loop
decisions) overlaps the device work of the others. Jobs never share mutable
device memory, so a job's result is bit-identical whether it runs alone or in
a mix (every reduction in libmsn has a fixed order).

Admission is by device memory: a worker starts a job only when the bytes it
needs (its workspace growth plus inputs, spectra and outputs) fit in the
budget taken from the free HBM at start-up; otherwise it first gives back its
own cached buffers of other image sizes and then waits for other jobs to end.
"""
import concurrent.futures as cf
import ctypes
import heapq
import itertools
import threading
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native
from . import device as dev
from . import tune

F32 = 4
C64 = 8


def job_bytes(n, psf_side, scale_count, conv_mode="linear"):
    """Device bytes of one deconvolution of an n x n image: (workspace buffers, per-job transients)."""
    double = psf_side == 2 * n
    if conv_mode == "linear":
        m = psf_side if double else 2 * psf_side
    else:
        m = n
    spec = m * (m // 2 + 1) * C64
    fft_work = 2 * m * (m // 2 + 1) * C64
    planes = 6 * scale_count * n * n * F32                      # dec, thr, emask, esrc, planes, ms
    vectors = 9 * n * n * F32                                    # x xn r rn p ap tmp rec + full conv
    buffers = planes + vectors + 2 * fft_work + spec + 2 * n * n * F32 + (1 << 20)
    transient = 2 * spec + psf_side * psf_side * F32 + 4 * n * n * F32 + scale_count * n * n * F32
    return buffers, transient


def _tensor_bytes(obj):
    """Bytes of the device tensors held by obj's attributes (one level, dicts included)."""
    total = 0
    for v in vars(obj).values():
        for t in (v.values() if isinstance(v, dict) else (v,)):
            if isinstance(t, torch.Tensor):
                total += t.numel() * t.element_size()
    return total


class Workspace:
    """Device state one worker keeps between jobs: buffers per image geometry and a minor-loop engine."""

    def __init__(self, device):
        self.device = device
        self._buffers = {}
        self._bytes = {}
        self._engine = None

    def buffers_for(self, key, build):
        if key not in self._buffers:
            self._buffers[key] = build()
            self._bytes[key] = _tensor_bytes(self._buffers[key])
        return self._buffers[key]

    def has_geometry(self, n, scale_count):
        """Buffers for an n x n image with scale_count scales are cached (key: n, ns, scales, m_sub, m_data)."""
        return any(k[0] == n and k[2] == scale_count for k in self._buffers)

    def nbytes(self):
        return sum(self._bytes.values())

    def drop_other_geometries(self, n, scale_count):
        """Release the buffers of every other geometry; returns the bytes released."""
        freed = 0
        for k in [k for k in self._buffers if not (k[0] == n and k[2] == scale_count)]:
            del self._buffers[k]
            freed += self._bytes.pop(k)
        return freed

    def engine(self):
        if self._engine is None:
            h = ctypes.c_void_p()
            _native.call("msn_minor_engine_create", ctypes.byref(h))
            self._engine = h
        return self._engine

    def close(self):
        self._buffers.clear()
        self._bytes.clear()
        if self._engine is not None:
            _native.query("msn_minor_engine_destroy", self._engine)
            self._engine = None


class MemoryGate:
    """Byte budget shared by the workers (admission by free HBM)."""

    def __init__(self, budget):
        self.budget = int(budget)
        self.used = 0
        self._cv = threading.Condition()

    def acquire(self, nbytes, shrink=None, timeout=None):
        """Reserve nbytes; ``shrink()`` may give back bytes (returns how many) before waiting."""
        nbytes = int(nbytes)
        if nbytes > self.budget:
            raise MemoryError(f"job needs {nbytes} bytes, more than the whole budget of {self.budget}")
        with self._cv:
            short = self.used + nbytes > self.budget
        if short and shrink is not None:
            # shrink() can take a while (it may empty torch's cache): run it without the
            # lock so the other workers' acquire / release calls are not held up.
            freed = shrink()
            with self._cv:
                self.used -= freed
                self._cv.notify_all()
        with self._cv:
            ok = self._cv.wait_for(lambda: self.used + nbytes <= self.budget, timeout)
            if not ok:
                raise TimeoutError("no device memory became free for the job")
            self.used += nbytes

    def release(self, nbytes):
        with self._cv:
            self.used -= int(nbytes)
            self._cv.notify_all()


@dataclass
class Job:
    """One deconvolution: host (numpy) or device (torch) dirty image and PSF, MORESANE keyword arguments."""

    dirty: object
    psf: object
    mask: object = None
    kwargs: dict = field(default_factory=dict)
    tag: object = None


@dataclass
class JobResult:
    tag: object
    model: np.ndarray
    residual: np.ndarray
    major: int
    log: list
    t_submit: float
    t_start: float
    t_end: float
    worker: int

    @property
    def latency(self):
        return self.t_end - self.t_submit


class DeconvolutionExecutor:
    """Runs Jobs concurrently on one GPU with ``workers`` streams.

    ``order``: "fifo" serves jobs in arrival order (serving); "largest" starts
    the largest images first (a batch, so that the long jobs do not end last).
    ``hbm_fraction`` of the device's free memory at start-up is the admission
    budget.
    """

    def __init__(self, workers=8, device=None, order="fifo", hbm_fraction=0.85):
        dev.require_cuda()
        _native.load()
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        free, _ = torch.cuda.mem_get_info(self.device)
        self.gate = MemoryGate(free * hbm_fraction)
        self.order = order
        self._heap = []
        self._seq = itertools.count()
        self._cv = threading.Condition()
        self._closed = False
        # this device's tuned values first, then (with several workers) the values that favour
        # concurrent deconvolutions, restored when the executor shuts down
        tune.ensure_applied()
        self._concurrent = workers > 1
        if self._concurrent:
            tune.enter_concurrent()
        self._threads = [threading.Thread(target=self._worker, args=(i,), daemon=True) for i in range(workers)]
        for t in self._threads:
            t.start()

    # -- submission -------------------------------------------------------
    def submit(self, job):
        fut = cf.Future()
        n = int(np.shape(job.dirty)[0])
        prio = -n if self.order == "largest" else 0
        with self._cv:
            if self._closed:
                raise RuntimeError("executor is shut down")
            heapq.heappush(self._heap, (prio, next(self._seq), job, fut, time.perf_counter()))
            self._cv.notify()
        return fut

    def map(self, jobs):
        """Run every job; results in the order of ``jobs``."""
        futs = [self.submit(j) for j in jobs]
        return [f.result() for f in futs]

    def shutdown(self):
        with self._cv:
            if self._closed:
                return
            self._closed = True
            self._cv.notify_all()
        for t in self._threads:
            t.join()
        if self._concurrent:
            tune.leave_concurrent()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.shutdown()

    # -- workers ----------------------------------------------------------
    def _next(self):
        with self._cv:
            self._cv.wait_for(lambda: self._heap or self._closed)
            if not self._heap:
                return None
            return heapq.heappop(self._heap)

    def _worker(self, wid):
        from .main import Deconvolver
        torch.cuda.set_device(self.device)
        stream = torch.cuda.Stream(self.device)
        ws = Workspace(self.device)
        held = 0  # bytes of ws counted in the gate
        try:
            while True:
                item = self._next()
                if item is None:
                    break
                _, _, job, fut, t_submit = item
                if not fut.set_running_or_notify_cancel():
                    continue
                n = int(np.shape(job.dirty)[0])
                psf_side = int(np.shape(job.psf)[0])
                kw = dict(job.kwargs)
                scale_count = kw.get("scale_count") or int(np.log2(n) - 1)
                buf_bytes, transient = job_bytes(n, psf_side, scale_count, kw.get("conv_mode", "linear"))

                def shrink():
                    nonlocal held
                    freed = ws.drop_other_geometries(n, scale_count)
                    if freed:
                        # cached blocks stay in this stream's pool unless handed back to CUDA
                        torch.cuda.empty_cache()
                    held -= freed
                    return freed

                need = transient + (0 if ws.has_geometry(n, scale_count) else buf_bytes)
                try:
                    self.gate.acquire(need, shrink=shrink)
                except Exception as e:  # noqa: BLE001 - reported through the future
                    fut.set_exception(e)
                    continue
                try:
                    t_start = time.perf_counter()
                    with torch.cuda.stream(stream):
                        dirty = dev.as_f32_cuda(job.dirty, device=self.device)
                        eng = Deconvolver(job.psf, job.mask, workspace=ws)
                        model, residual, major = eng.moresane(dirty, **kw)
                        model_h = model.cpu().numpy()
                        residual_h = residual.cpu().numpy()
                    stream.synchronize()
                    t_end = time.perf_counter()
                    fut.set_result(JobResult(job.tag, model_h, residual_h, major, eng.log, t_submit, t_start,
                                             t_end, wid))
                except Exception as e:  # noqa: BLE001
                    fut.set_exception(e)
                finally:
                    # keep exactly the workspace's bytes reserved; the job's transients are gone
                    now = ws.nbytes()
                    self.gate.release(held + need - now)
                    held = now
        finally:
            self.gate.release(held)
            ws.close()


def serve(jobs, arrivals, workers=8, device=None):
    """Submit ``jobs[i]`` at ``arrivals[i]`` seconds after the start; returns (results, wall seconds)."""
    results = [None] * len(jobs)
    with DeconvolutionExecutor(workers=workers, device=device, order="fifo") as ex:
        t0 = time.perf_counter()
        futs = []
        for job, at in zip(jobs, arrivals):
            delay = t0 + at - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            futs.append(ex.submit(job))
        for i, f in enumerate(futs):
            results[i] = f.result()
        wall = time.perf_counter() - t0
    return results, wall

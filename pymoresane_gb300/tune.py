"""Autotuner for libmsn's launch parameters.

The library reads a few tunable launch parameters at every launch (declared
with msn_tune_set in include/msn.h): which kernels run the 2048^2 linear
convolution with a 4096^2 PSF (the four-step kernels or the Stockham ones),
how many CTAs of each four-step kernel share an SM, and how many threads a CTA
of the a trous passes has (one value for rows of up to 2048 floats, one for wider
rows). None of them changes a result; they only change the
speed, and the best values depend on the device.

``autotune()`` times the candidates of each parameter on the real operation
(CUDA events on the current stream, the median of several runs after a
warm-up; the a trous CTA size on a short deconvolution when the caller gives one), keeps the fastest, sets it in the library and stores the choice in a
JSON cache keyed by the device (name, SM count, compute capability).
``ensure_applied()`` loads the cache once per process and sets the cached
values; the deconvolution driver calls it, so a tuned device keeps its choices
across processes. The cache lives in ``$PYMORESANE_GB300_TUNE_CACHE`` or
``~/.cache/pymoresane_gb300/tune.json``.

Parameters are tuned one after another (coordinate descent from the current
values): first the convolution kernels, then each four-step CTA count, then
the a trous CTA size.
"""
import ctypes
import json
import os
import statistics
import threading

from . import _native

CACHE_ENV = "PYMORESANE_GB300_TUNE_CACHE"
KNOBS = ("fft_four_step", "fft_sq_fwd_ctas", "fft_sq_col_ctas", "fft_sq_inv_ctas", "iuwt_threads", "iuwt_threads_wide")
CANDIDATES = {
    "fft_four_step": (1, 0),
    "fft_sq_fwd_ctas": (0, 2, 3),
    "fft_sq_col_ctas": (0, 2),
    "fft_sq_inv_ctas": (0, 2),
    "iuwt_threads": (256, 128, 64),
    "iuwt_threads_wide": (256, 128, 64),
}
_applied = False
_lock = threading.Lock()


def cache_path():
    return os.environ.get(CACHE_ENV) or os.path.join(os.path.expanduser("~"), ".cache", "pymoresane_gb300",
                                                     "tune.json")


def load_cache(path=None):
    path = path or cache_path()
    try:
        with open(path) as fh:
            data = json.load(fh)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def save_cache(data, path=None):
    path = path or cache_path()
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as fh:
        json.dump(data, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)
    return path


def device_key():
    import torch
    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    return f"{p.name}|sm{p.multi_processor_count}|cc{p.major}.{p.minor}"


def get(name):
    v = ctypes.c_int()
    _native.call("msn_tune_get", name.encode(), ctypes.byref(v))
    return v.value


def current():
    return {k: get(k) for k in KNOBS}


def sq_grids():
    """(forward rows, columns, inverse rows) persistent grids of the four-step kernels on this device."""
    out = (ctypes.c_int * 3)()
    _native.call("msn_fft_sq_grids", out)
    return tuple(out)


def set_values(values):
    for k, v in values.items():
        if k in KNOBS:
            _native.call("msn_tune_set", k.encode(), int(v))


def reset():
    _native.call("msn_tune_reset")


def choose(name, candidates, measure):
    """Sets each candidate value of ``name``, calls ``measure()`` (seconds) and keeps the fastest.

    Returns (best value, {value: seconds}); the library is left at the best value.
    """
    times = {}
    for v in candidates:
        set_values({name: v})
        times[v] = measure()
    best = min(times, key=times.get)
    set_values({name: best})
    return best, times


def _timer(fn, reps, warmup=2):
    import torch
    stream = torch.cuda.current_stream()

    def measure():
        for _ in range(warmup):
            fn()
        vals = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            vals.append(e0.elapsed_time(e1) * 1e-3)
        return statistics.median(vals)
    return measure


def autotune(n=2048, reps=10, path=None, save=True, workload=None):
    """Tunes every parameter on an n x n problem (convolution with a 2n x 2n PSF spectrum,
    decomposition + recomposition with log2(n) - 4 scales) and caches the result.

    workload (optional): a callable that runs a short piece of the real computation, such as a
    deconvolution bounded to a few major iterations. The a trous CTA size is then timed on it
    instead of on the dense decomposition + recomposition: a deconvolution's passes are masked
    and skip rows, and on GB300 they favour a different CTA size (a 2048^2 deconvolution took
    497.6 ms with 256 threads against 506.4 ms with the 128 the dense passes favour).

    Returns {"device": key, "values": {...}, "times_s": {...}}.
    """
    import numpy as np
    import torch

    from . import device as dev
    from . import synthetic
    rng = np.random.default_rng(0)
    x = torch.from_numpy(rng.standard_normal((n, n)).astype(np.float32)).cuda()
    psf = synthetic.make_psf(2 * n, 2000, rng)
    spec = dev.psf_spectrum(psf)
    out = torch.empty_like(x)
    fwork = dev.fft_workspace(n, 2 * n, x.device)
    scales = max(2, int(np.log2(n)) - 4)
    w = torch.empty((scales, n, n), dtype=torch.float32, device=x.device)
    c = torch.empty_like(x)
    rec = torch.empty_like(x)
    iwork = dev.iuwt_workspace(n, n, x.device)

    def conv():
        dev.fft_convolve(x, spec, True, out=out, work=fwork)

    def iuwt():
        dev.iuwt_decompose(x, scales, 0, store_smoothed=True, out=w, smoothed_out=c, work=iwork)
        dev.iuwt_recompose(w, 0, smoothed=c, out=rec, work=iwork)

    times = {}
    tuned = {}
    for name in KNOBS:
        # the convolution parameters only matter for the 2048^2 / 4096^2 case the
        # four-step kernels serve; the a trous CTA size for this problem's row width
        if name.startswith("fft_") and n != 2048:
            continue
        if name.startswith("fft_sq_") and get("fft_four_step") == 0:
            continue
        if name == ("iuwt_threads_wide" if n <= 2048 else "iuwt_threads"):
            continue
        op = (workload or iuwt) if name.startswith("iuwt_") else conv
        best, t = choose(name, CANDIDATES[name], _timer(op, reps))
        times[name] = {str(k): v for k, v in t.items()}
        tuned[name] = best
    torch.cuda.synchronize()
    result = {"device": device_key(), "n": n, "values": current(), "tuned": tuned, "times_s": times}
    if save:
        # one entry per device; each run updates only the parameters it tuned
        data = load_cache(path)
        entry = data.get(device_key(), {})
        values = dict(entry.get("values", {}))
        values.update(tuned)
        data[device_key()] = {"device": device_key(), "values": values,
                              "runs": dict(entry.get("runs", {}), **{str(n): {"tuned": tuned, "times_s": times}})}
        save_cache(data, path)
    return result


# Launch parameters for concurrent deconvolutions on one GPU (DeconvolutionExecutor with
# more than one worker). Smaller a trous CTAs and fewer resident four-step row-transform CTAs
# interleave better across streams: 8 concurrent 2048^2 deconvolutions ran at 2.39 deconv/s
# with 128-thread a trous CTAs against 2.25 with 256, and at 2.54 against 2.38 with the two
# row kernels capped at 2 CTAs per SM (GB300, same process); a single deconvolution is faster
# with the tuned values.
CONCURRENT = {"iuwt_threads": 128, "fft_sq_fwd_ctas": 2, "fft_sq_inv_ctas": 2}
_conc_lock = threading.Lock()
_conc_depth = 0
_conc_saved = None


def enter_concurrent():
    """Sets CONCURRENT while any concurrent executor runs (paired with leave_concurrent)."""
    global _conc_depth, _conc_saved
    with _conc_lock:
        if _conc_depth == 0:
            _conc_saved = {k: get(k) for k in CONCURRENT}
            set_values(CONCURRENT)
        _conc_depth += 1


def leave_concurrent():
    """Restores the values enter_concurrent replaced once the last concurrent executor stops."""
    global _conc_depth, _conc_saved
    with _conc_lock:
        _conc_depth -= 1
        if _conc_depth == 0 and _conc_saved is not None:
            set_values(_conc_saved)
            _conc_saved = None


def ensure_applied(path=None):
    """Sets the cached values for this device once per process; returns them (or None)."""
    global _applied
    with _lock:
        if _applied:
            return None
        _applied = True
        entry = load_cache(path).get(device_key())
        if not entry:
            return None
        set_values(entry.get("values", {}))
        return entry.get("values")

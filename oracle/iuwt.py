"""Oracle: isotropic undecimated wavelet transform (a trous, B3 spline).

Restates pymoresane/iuwt.py:

* ``a_trous``           -- ser_a_trous, pymoresane/iuwt.py:151-191 (FP64), and
                           the pyCUDA row/column kernels gpu_a_trous,
                           pymoresane/iuwt.py:588-659 (FP32, fused multiply-add
                           chain), selected by ``arith``.
* ``decompose``         -- ser_iuwt_decomposition, pymoresane/iuwt.py:66-111 and
                           gpu_iuwt_decomposition, pymoresane/iuwt.py:384-499.
* ``recompose``         -- ser_iuwt_recomposition, pymoresane/iuwt.py:113-149 and
                           gpu_iuwt_recomposition, pymoresane/iuwt.py:501-581.
* ``decompose_strips`` /
  ``recompose_strips``  -- the multi-core strip variant (mp_a_trous,
                           pymoresane/iuwt.py:281-382): every 1-D pass computed
                           in FP64 and stored to an FP32 buffer, strips
                           processed by a thread pool (the reference forks one
                           process per strip; threads are used here because the
                           numpy kernels release the GIL and because forking
                           after a CUDA context exists is unsafe).

Per-element order of operations (both precisions): centre tap first, then the
taps at -2d, -d, +d, +2d (d = 2**scale), first along axis 0, then along axis 1,
with half-sample-symmetric mirroring at the borders: x[-k] = x[k-1] and
x[n-1+k] = x[n-k] (pymoresane/iuwt.py:163-189 and :600-620).

``arith='f32fma'`` reproduces the GPU kernels' FP32 rounding exactly: the
first product is rounded (``wfil[2]*in1``), every further tap is one fused
multiply-add, emulated here with a correctly-rounded FMA (``fma32``).
"""
from concurrent.futures import ThreadPoolExecutor

import numpy as np

B3 = np.array([1.0, 4.0, 6.0, 4.0, 1.0]) / 16.0
B3_F32 = B3.astype(np.float32)


def mirror_index(n, offset):
    """Indices of x[i + offset] with half-sample-symmetric mirroring (|offset| <= n)."""
    i = np.arange(n) + offset
    i = np.where(i < 0, -i - 1, i)
    i = np.where(i >= n, 2 * n - i - 1, i)
    return i


def fma32(a, b, c):
    """Correctly rounded float32 fused multiply-add a*b + c (vectorised).

    a*b of two float32 values is exact in float64; the float64 sum is then
    rounded to float32, and the only double-rounding case (the float64 sum
    lands exactly on a float32 midpoint while the exact sum does not) is
    resolved with the TwoSum error term.
    """
    p = np.asarray(a, np.float64) * np.asarray(b, np.float64)
    c64 = np.asarray(c, np.float64)
    s = p + c64
    bb = s - p
    err = (p - (s - bb)) + (c64 - bb)
    r = s.astype(np.float32)
    r64 = r.astype(np.float64)
    up = np.nextafter(r, np.float32(np.inf))
    dn = np.nextafter(r, np.float32(-np.inf))
    mid_up = (r64 + up.astype(np.float64)) * 0.5
    mid_dn = (r64 + dn.astype(np.float64)) * 0.5
    at_up = (s == mid_up) & (err != 0)
    at_dn = (s == mid_dn) & (err != 0)
    # s is the midpoint between r and its upper (lower) neighbour: the exact
    # value lies on the side given by err.
    r = np.where(at_up, np.where(err > 0, up, r), r)
    r = np.where(at_dn, np.where(err < 0, dn, r), r)
    return r.astype(np.float32)


def _pass(x, scale, axis, arith):
    n = x.shape[axis]
    d = 2 ** scale
    take = (lambda idx: x[idx, :]) if axis == 0 else (lambda idx: x[:, idx])
    if arith == "f64":
        f = B3
        acc = f[2] * x
        for tap, off in ((0, -2 * d), (1, -d), (3, d), (4, 2 * d)):
            acc = acc + f[tap] * take(mirror_index(n, off))
        return acc
    f = B3_F32
    acc = (f[2] * x).astype(np.float32)
    for tap, off in ((0, -2 * d), (1, -d), (3, d), (4, 2 * d)):
        acc = fma32(f[tap], take(mirror_index(n, off)), acc)
    return acc


def a_trous(c0, scale, arith="f64"):
    """One B3-spline smoothing at dilation 2**scale: axis 0, then axis 1."""
    if arith == "f64":
        c0 = np.asarray(c0, np.float64)
    else:
        c0 = np.asarray(c0, np.float32)
    return _pass(_pass(c0, scale, 0, arith), scale, 1, arith)


def decompose(in1, scale_count, scale_adjust=0, store_smoothed=False, arith="f64"):
    """Detail coefficients [scale_count - scale_adjust, ny, nx] (+ smoothest plane).

    w_s = C_s - h_s*(h_s*C_s), C_{s+1} = h_s*C_s (pymoresane/iuwt.py:102-106).
    """
    dt = np.float64 if arith == "f64" else np.float32
    c0 = np.asarray(in1, dt)
    for s in range(scale_adjust):
        c0 = a_trous(c0, s, arith)
    out = np.empty((scale_count - scale_adjust,) + c0.shape, dt)
    for s in range(scale_adjust, scale_count):
        c = a_trous(c0, s, arith)
        c1 = a_trous(c, s, arith)
        out[s - scale_adjust] = c0 - c1
        c0 = c
    if store_smoothed:
        return out, c0
    return out


def recompose(in1, scale_adjust=0, smoothed_array=None, arith="f64"):
    """rec = h_s*rec + w_s from the top scale down, then scale_adjust extra smoothings."""
    dt = np.float64 if arith == "f64" else np.float32
    w = np.asarray(in1, dt)
    max_scale = w.shape[0] + scale_adjust
    if smoothed_array is None:
        rec = np.zeros(w.shape[1:], dt)
    else:
        rec = np.asarray(smoothed_array, dt)
    for s in range(max_scale - 1, scale_adjust - 1, -1):
        rec = (a_trous(rec, s, arith) + w[s - scale_adjust]).astype(dt)
    for s in range(scale_adjust - 1, -1, -1):
        rec = a_trous(rec, s, arith)
    return rec


# ----------------------------------------------------------------------------
# Strip-parallel FP32 variant (pymoresane/iuwt.py:281-382), used as the timed
# multi-core CPU baseline.
# ----------------------------------------------------------------------------

def _strip_pass(src, dst, scale, axis, lo, hi):
    n = src.shape[axis]
    d = 2 ** scale
    if axis == 0:
        blk = src[:, lo:hi]
        acc = B3[2] * blk
        for tap, off in ((0, -2 * d), (1, -d), (3, d), (4, 2 * d)):
            acc += B3[tap] * blk[mirror_index(n, off), :]
        dst[:, lo:hi] = acc
    else:
        blk = src[lo:hi, :]
        acc = B3[2] * blk
        for tap, off in ((0, -2 * d), (1, -d), (3, d), (4, 2 * d)):
            acc += B3[tap] * blk[:, mirror_index(n, off)]
        dst[lo:hi, :] = acc


def a_trous_strips(c0, scale, pool, workers):
    c0 = np.asarray(c0, np.float32)
    tmp = np.empty_like(c0)
    out = np.empty_like(c0)
    ny, nx = c0.shape
    for axis, src, dst, n in ((0, c0, tmp, nx), (1, tmp, out, ny)):
        bounds = np.linspace(0, n, workers + 1).astype(int)
        futs = [pool.submit(_strip_pass, src, dst, scale, axis, bounds[i], bounds[i + 1])
                for i in range(workers) if bounds[i + 1] > bounds[i]]
        for f in futs:
            f.result()
    return out


def decompose_strips(in1, scale_count, scale_adjust=0, store_smoothed=False, workers=8):
    with ThreadPoolExecutor(workers) as pool:
        c0 = np.asarray(in1, np.float32)
        for s in range(scale_adjust):
            c0 = a_trous_strips(c0, s, pool, workers)
        out = np.empty((scale_count - scale_adjust,) + c0.shape, np.float32)
        for s in range(scale_adjust, scale_count):
            c = a_trous_strips(c0, s, pool, workers)
            c1 = a_trous_strips(c, s, pool, workers)
            np.subtract(c0, c1, out=out[s - scale_adjust])
            c0 = c
    if store_smoothed:
        return out, c0
    return out


def recompose_strips(in1, scale_adjust=0, smoothed_array=None, workers=8):
    w = np.asarray(in1, np.float32)
    max_scale = w.shape[0] + scale_adjust
    rec = np.zeros(w.shape[1:], np.float32) if smoothed_array is None else np.asarray(smoothed_array, np.float32)
    with ThreadPoolExecutor(workers) as pool:
        for s in range(max_scale - 1, scale_adjust - 1, -1):
            rec = a_trous_strips(rec, s, pool, workers)
            rec += w[s - scale_adjust]
        for s in range(scale_adjust - 1, -1, -1):
            rec = a_trous_strips(rec, s, pool, workers)
    return rec

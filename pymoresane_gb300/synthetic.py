"""Seeded synthetic radio-interferometric inputs (dirty image + PSF).

The reference ships no benchmark data, so every workload here is generated
from a seed with the shapes and value distributions of the published
workloads:

* PSF: an M x M uv grid is filled from ``n_uv`` seeded samples (radius
  uniform in [0, 0.4 * Nyquist], angle uniform, each sample gridded together
  with its Hermitian mirror), inverse-FFT'd, its magnitude fft-shifted to the
  centre and normalised to peak 1 (float32).
* Sky: point sources at uniform positions with log-uniform flux plus
  elliptical Gaussians (sigma uniform in a range, random position angle,
  log-uniform peak in the same flux range).
* Dirty: sky convolved with the PSF ("same" size) plus white Gaussian noise.

This is input generation only: it runs once per workload on the host and is
not part of the deconvolution path.
"""
from dataclasses import dataclass

import numpy as np


@dataclass
class Workload:
    """Parameters of one synthetic deconvolution problem."""

    n: int                      # image side (pixels)
    psf_factor: int = 2         # PSF side = psf_factor * n
    n_uv: int = 3000
    n_points: int = 40
    flux_range: tuple = (0.01, 1.0)
    n_gauss: int = 5
    sigma_range: tuple = (2.0, 8.0)
    noise: float = 1e-3
    seed: int = 0


def make_psf(m, n_uv, rng, fast=False):
    """|ifft2| of a seeded uv grid, shifted to the centre, peak-normalised.

    fast=True takes the transform with scipy.fft on all host threads; the
    result then equals the default one only to rounding (used where inputs need
    not match other runs bit for bit)."""
    nyq = m / 2.0
    r = rng.uniform(0.0, 0.4 * nyq, n_uv)
    th = rng.uniform(0.0, 2.0 * np.pi, n_uv)
    u = np.rint(r * np.cos(th)).astype(np.int64)
    v = np.rint(r * np.sin(th)).astype(np.int64)
    grid = np.zeros((m, m), np.float64)
    np.add.at(grid, (v % m, u % m), 1.0)
    np.add.at(grid, ((-v) % m, (-u) % m), 1.0)
    if fast:
        import scipy.fft as sfft
        psf = np.abs(np.fft.fftshift(sfft.ifft2(grid, workers=-1)))
    else:
        psf = np.abs(np.fft.fftshift(np.fft.ifft2(grid)))
    psf /= psf.max()
    return psf.astype(np.float32)


def make_sky(n, n_points, flux_range, n_gauss, sigma_range, rng, window=False):
    """Point sources plus elliptical Gaussians on an n x n grid (float64).

    window=True evaluates each Gaussian only within 40 sigma of its centre,
    beyond which exp(-r^2 / 2) is below 1e-300 (for the mixes, whose inputs
    need not match other runs bit for bit)."""
    sky = np.zeros((n, n), np.float64)
    lo, hi = np.log(flux_range[0]), np.log(flux_range[1])
    margin = max(4, n // 16)
    ys = rng.integers(margin, n - margin, n_points)
    xs = rng.integers(margin, n - margin, n_points)
    flux = np.exp(rng.uniform(lo, hi, n_points))
    np.add.at(sky, (ys, xs), flux)
    yy, xx = np.mgrid[0:n, 0:n]
    for _ in range(n_gauss):
        cy, cx = rng.uniform(margin, n - margin, 2)
        sa, sb = rng.uniform(sigma_range[0], sigma_range[1], 2)
        pa = rng.uniform(0.0, np.pi)
        amp = np.exp(rng.uniform(lo, hi))
        if window:
            rad = int(np.ceil(40 * max(sa, sb)))
            r0, r1 = max(0, int(cy) - rad), min(n, int(cy) + rad + 1)
            c0, c1 = max(0, int(cx) - rad), min(n, int(cx) + rad + 1)
            ys, xs = yy[r0:r1, c0:c1], xx[r0:r1, c0:c1]
        else:
            ys, xs = yy, xx
        dy, dx = ys - cy, xs - cx
        a = dx * np.cos(pa) + dy * np.sin(pa)
        b = -dx * np.sin(pa) + dy * np.cos(pa)
        g = amp * np.exp(-0.5 * ((a / sa) ** 2 + (b / sb) ** 2))
        if window:
            sky[r0:r1, c0:c1] += g
        else:
            sky += g
    return sky


def make_problem(w: Workload, fast=False):
    """Return (dirty float32 [n,n], psf float32 [m,m], sky float64 [n,n]).

    fast=True uses multi-threaded transforms (see make_psf) and a direct
    "same"-size FFT convolution: equal to the default problem only to rounding.
    """
    from scipy.signal import fftconvolve

    rng = np.random.default_rng(w.seed)
    m = w.psf_factor * w.n
    psf = make_psf(m, w.n_uv, rng, fast=fast)
    sky = make_sky(w.n, w.n_points, w.flux_range, w.n_gauss, w.sigma_range, rng, window=fast)
    if fast:
        import scipy.fft as sfft
        shape = [sfft.next_fast_len(w.n + m - 1, real=True)] * 2
        full = sfft.irfft2(sfft.rfft2(sky, shape, workers=-1) * sfft.rfft2(psf.astype(np.float64), shape, workers=-1),
                           shape, workers=-1)
        o = (m - 1) // 2  # start of the "same" window
        dirty = full[o:o + w.n, o:o + w.n]
    else:
        dirty = fftconvolve(sky, psf.astype(np.float64), mode="same")
    dirty += rng.normal(0.0, w.noise, dirty.shape)
    return dirty.astype(np.float32), psf, sky


def problem_512(seed=0):
    """512^2 dirty image, 1024^2 PSF, 3000 uv points, 40 points, 5 Gaussians."""
    return Workload(n=512, n_uv=3000, n_points=40, flux_range=(0.01, 1.0), n_gauss=5,
                    sigma_range=(2.0, 8.0), noise=1e-3, seed=seed)


def problem_2048(seed=0):
    """2048^2 dirty image, 4096^2 PSF, 20000 uv points, 1000 points, 50 Gaussians."""
    return Workload(n=2048, n_uv=20000, n_points=1000, flux_range=(1e-3, 1.0), n_gauss=50,
                    sigma_range=(2.0, 20.0), noise=1e-4, seed=seed)


def scaled(n, seed=0):
    """The 512^2 problem's recipe scaled by area to side n (uv count and sources)."""
    f = (n / 512.0) ** 2
    return Workload(n=n, n_uv=int(3000 * f), n_points=max(4, int(40 * f)), flux_range=(0.01, 1.0),
                    n_gauss=max(1, int(round(5 * f))), sigma_range=(2.0, 8.0), noise=1e-3, seed=seed)


def iuwt_image(n=4096, n_deltas=500, seed=0):
    """N(0,1) noise plus seeded deltas of amplitude U(5,50) (float32)."""
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, n), dtype=np.float32)
    ys = rng.integers(0, n, n_deltas)
    xs = rng.integers(0, n, n_deltas)
    x[ys, xs] += rng.uniform(5.0, 50.0, n_deltas).astype(np.float32)
    return x

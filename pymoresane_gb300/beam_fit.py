"""Restoring beam: an elliptical Gaussian fitted to the central lobe of the PSF.

Follows pymoresane/beam_fit.py:6-69. The fit runs once per image on a window of
at most 512 x 512 PSF pixels, so it stays on the host, with scipy's
Levenberg-Marquardt ``curve_fit`` and ``ndimage.label`` as in the reference. The
restoring convolution itself runs on the GPU (``DataImage.restore``).

Window. The reference selects the PSF window with ``if psf.shape > 512``
(beam_fit.py:16), a tuple-versus-int comparison. Python 2, the reference's
interpreter, evaluates it as True for every shape, so the reference always
takes ``psf[n/2-256 : n/2+256]`` (integer division, Python slice rules). For a
side below 512 the negative start wraps, e.g. a 256 x 256 PSF gives rows and
columns 128..255, with the peak at the window's corner. This module keeps that
behaviour, so beams and beam parameters match the reference run under
Python 2.
"""
import numpy as np

__all__ = ["beam_fit", "elliptical_gaussian"]


def _window(n):
    """[start, stop) of psf[n // 2 - 256 : n // 2 + 256] under Python slice rules (beam_fit.py:16-17)."""
    return slice(n // 2 - 256, n // 2 + 256).indices(n)[:2]


def elliptical_gaussian(xy, amp, xsigma, ysigma, theta):
    """A * exp(-(u^2 / 2 xsigma^2 + v^2 / 2 ysigma^2)), (u, v) = (x, y) rotated by theta (beam_fit.py:49-51).

    The operations are evaluated in the reference's order so that the fit sees
    the same function values.
    """
    c, s = np.cos(theta), np.sin(theta)
    u = xy[:, 0] * c - xy[:, 1] * s
    v = xy[:, 0] * s + xy[:, 1] * c
    return amp * np.exp(-1 * ((u ** 2) / (2 * (xsigma ** 2)) + (v ** 2) / (2 * (ysigma ** 2))))


def beam_fit(psf, cdelt1, cdelt2):
    """Clean beam (float32, the PSF's shape, peak 1) and [bmaj, bmin, bpa] (beam_fit.py:6-69).

    bmaj / bmin are FWHMs scaled by cdelt1 / cdelt2, bpa is in degrees.
    """
    from scipy import ndimage
    from scipy.optimize import curve_fit

    psf = np.asarray(psf)
    r0, r1 = _window(psf.shape[0])
    c0, c1 = _window(psf.shape[1])
    centre = psf[r0:r1, c0:c1] / np.max(psf[r0:r1, c0:c1])
    peak = np.unravel_index(np.argmax(centre), centre.shape)

    # the primary lobe: the 4-connected island above half maximum that holds the peak
    islands, _ = ndimage.label(np.where(centre > 0.5, centre, 0))
    lobe = np.where(islands == islands[peak], centre, 0)

    cols = np.arange(-peak[1], -peak[1] + centre.shape[1], 1)
    rows = np.arange(-peak[0], -peak[0] + centre.shape[0], 1)
    grid_x, grid_y = np.meshgrid(cols, -rows)
    samples = np.column_stack((grid_x.reshape(-1, 1), grid_y.reshape(-1, 1), lobe.reshape(-1, 1, order="C")))
    xy = samples[:, 0:2]

    opt = curve_fit(elliptical_gaussian, xy, samples[:, 2], (1, 1, 1, 0))[0]

    beam = np.zeros_like(psf)
    beam[r0:r1, c0:c1] = elliptical_gaussian(xy, opt[0], opt[1], opt[2], opt[3]).reshape(centre.shape, order="C")
    beam = beam / np.max(beam)

    fwhm = 2 * np.sqrt(2 * np.log(2))
    bmaj = fwhm * max(opt[1], opt[2]) * cdelt1
    bmin = fwhm * min(opt[1], opt[2]) * cdelt2
    bpa = np.degrees(opt[3]) % 360 - 90
    return beam, [abs(bmaj), abs(bmin), bpa]

"""Oracle: the MORESANE major / minor loops on the CPU.

Restates DataImage.moresane (pymoresane/main.py:53-521) and
DataImage.moresane_by_scale (pymoresane/main.py:523-599) on top of the other
oracle modules, with the reference's 'ser' IUWT, 'cpu' convolution and 'cpu'
extraction. With ``precision='ref'`` the dtype flow is the reference's own
(dirty / PSF / model cast to float32, main.py:34-35,238; float32 linear
convolution, iuwt_convolution.py:70), so results equal the reference's path.
``precision='f64'`` removes those casts: the float64 oracle used to state the
error of the GPU path.

Every major iteration appends a record to ``self.log`` (min_scale,
max_scale, scale_adjust, minor iterations, final SNR, residual std) so that
trajectories can be compared decision by decision.
"""
import time

import numpy as np

from . import convolution as C
from . import iuwt as I
from . import toolbox as T


def _conv(x, spec, mode, f64):
    if f64 and mode == "linear":
        full = np.fft.fftshift(np.fft.irfft2(spec * np.fft.rfft2(C.pad_array(x))))
        n = x.shape[0]
        return np.ascontiguousarray(full[n // 2:3 * n // 2, n // 2:3 * n // 2])
    return C.fft_convolve(x, spec, mode)


def suppression_array(scale_count, subregion, edge_suppression, edge_offset):
    """Edge-suppression weights (pymoresane/main.py:249-260), or None."""
    if edge_suppression:
        arr = np.zeros([scale_count, subregion, subregion], np.float32)
        corruption = 0
        for i in range(scale_count):
            corruption += 2 * 2 ** i
            e = edge_offset if edge_offset > corruption else corruption
            arr[i, e:-e, e:-e] = 1
        return arr
    if edge_offset > 0:
        arr = np.zeros([scale_count, subregion, subregion], np.float32)
        arr[:, edge_offset:-edge_offset, edge_offset:-edge_offset] = 1
        return arr
    return None


class MoresaneOracle:
    """``decom='mp'`` swaps the 'ser' IUWT for the strip-parallel FP32 'mp'
    restatement on ``workers`` threads (the reference's mode='mp',
    pymoresane/iuwt.py:193-382). ``self.timings`` accumulates wall time of the
    set-up, of the per-major-iteration work and of the minor iterations."""

    def __init__(self, dirty, psf, mask=None, precision="ref", decom="ser", workers=1):
        self.decom, self.workers = decom, workers
        self.timings = {"setup": 0.0, "major": 0.0, "minor": 0.0, "n_major": 0, "n_minor": 0}
        self.f64 = precision == "f64"
        dt = np.float64 if self.f64 else np.float32
        self.dirty_data = np.asarray(dirty).astype(dt)
        self.psf_data = np.asarray(psf).astype(dt)
        self.mask = mask
        self.model = np.zeros_like(self.dirty_data)
        self.residual = np.copy(self.dirty_data)
        self.complete = False
        self.log = []

    def moresane(self, subregion=None, scale_count=None, sigma_level=4, loop_gain=0.1, tolerance=0.75,
                 accuracy=1e-6, major_loop_miter=100, minor_loop_miter=30, conv_mode="linear",
                 enforce_positivity=False, edge_suppression=False, edge_offset=0, flux_threshold=0,
                 neg_comp=False, edge_excl=0, int_excl=0):
        n = self.dirty_data.shape[0]
        if n % 2 == 1:
            raise ValueError("Image size is uneven. Please use even dimensions.")
        if subregion is None or subregion > n:
            subregion = n
        if scale_count is None or scale_count > (np.log2(n) - 1):
            scale_count = int(np.log2(n) - 1)
        t_setup = time.perf_counter()
        if self.decom == "mp":
            def dec_fn(x, s, adj):
                return I.decompose_strips(x, s, adj, workers=self.workers)

            def rec_fn(w, adj):
                return I.recompose_strips(w, adj, workers=self.workers)
        else:
            def dec_fn(x, s, adj):
                return I.decompose(x, s, adj, arith="f64")

            def rec_fn(w, adj):
                return I.recompose(w, adj, arith="f64")
        sub_fft, data_fft, psf_sub, sub_sl = C.psf_spectra(self.psf_data, self.dirty_data.shape, subregion, conv_mode)
        dirty_sub = self.dirty_data[sub_sl]

        psf_dec = dec_fn(psf_sub, scale_count, 0)
        energies = np.empty([psf_dec.shape[0], 1, 1], dtype=np.float32)
        for i in range(energies.shape[0]):
            energies[i] = np.sqrt(np.sum(np.square(psf_dec[i])))

        major = 0
        max_coeff = 1
        model = np.zeros_like(self.dirty_data)
        std_current, std_ratio = 1000, 1
        min_scale = 0
        supp = suppression_array(scale_count, subregion, edge_suppression, edge_offset)
        residual = None
        x = None
        self.timings["setup"] += time.perf_counter() - t_setup
        t_major = time.perf_counter()
        while (major < major_loop_miter and max_coeff > 0 and std_ratio > accuracy
               and np.max(dirty_sub) > flux_threshold):
            rec = {"major": major}
            while min_scale < scale_count:
                if min_scale == 0:
                    dec = dec_fn(dirty_sub, scale_count, 0)
                    thresholds = T.estimate_threshold(dec, edge_excl, int_excl)
                    if self.mask is not None:
                        dec = dec_fn(dirty_sub * self.mask[sub_sl], scale_count, 0)
                    dec_thr = T.apply_threshold(dec, thresholds, sigma_level=sigma_level)
                    if supp is not None:
                        dec_thr *= supp
                    normalised = np.empty_like(energies)
                    for i in range(dec_thr.shape[0]):
                        normalised[i] = np.max(dec_thr[i]) / energies[i]
                max_index = int(np.argmax(normalised[min_scale:, :, :])) + min_scale
                max_scale = max_index + 1
                max_coeff = normalised[max_index, 0, 0]
                if max_coeff == 0:
                    break
                scale_adjust = 0
                for i in range(max_index - 1, -1, -1):
                    if normalised[i, 0, 0] == 0:
                        scale_adjust = i + 1
                        break
                extracted, ext_mask = T.source_extraction(dec_thr[scale_adjust:max_scale], tolerance, neg_comp,
                                                          semantics="cpu")
                recomposed = rec_fn(extracted, scale_adjust)

                def apply_a(v):
                    a = _conv(v, sub_fft, conv_mode, self.f64)
                    a = dec_fn(a, max_scale, scale_adjust)
                    return rec_fn(ext_mask * a, scale_adjust)

                x = np.zeros_like(recomposed)
                r = recomposed.copy()
                p = recomposed.copy()
                minor = 0
                snr_last = snr_current = 0
                while minor < minor_loop_miter:
                    t_minor = time.perf_counter()
                    ap = apply_a(p)
                    alpha = np.dot(r.reshape(1, -1), r.reshape(-1, 1))[0, 0] / np.dot(p.reshape(1, -1),
                                                                                     ap.reshape(-1, 1))[0, 0]
                    xn = x + alpha * p
                    if (np.min(xn) < 0) & enforce_positivity:
                        xn[xn < 0] = 0
                        p = (xn - x) / alpha
                        ap = apply_a(p)
                    rn = r - alpha * ap
                    beta = (np.dot(rn.reshape(1, -1), rn.reshape(-1, 1))[0, 0]
                            / np.dot(r.reshape(1, -1), r.reshape(-1, 1))[0, 0])
                    p = rn + beta * p
                    ms = _conv(xn, sub_fft, conv_mode, self.f64)
                    ms = ext_mask * dec_fn(ms, max_scale, scale_adjust)
                    snr_last = snr_current
                    snr_current = T.snr_ratio(extracted, ms)
                    minor += 1
                    dt = time.perf_counter() - t_minor
                    self.timings["minor"] += dt
                    self.timings["n_minor"] += 1
                    t_major += dt
                    if minor == 1 and snr_current > 40:
                        min_scale += 1
                        break
                    if snr_current > 40:
                        x = xn
                        min_scale = 0
                        break
                    if minor > 2 and snr_current <= snr_last:
                        if snr_current > 10.5:
                            min_scale = 0
                        else:
                            min_scale += 1
                        break
                    r = rn
                    x = xn
                rec.update(max_scale=max_scale, scale_adjust=scale_adjust, minor=minor, snr=float(snr_current))
                if minor == minor_loop_miter and snr_current > 10.5:
                    min_scale = 0
                    break
                if min_scale == 0:
                    break
            if min_scale == scale_count:
                break
            if max_coeff > 0:
                model[sub_sl] += loop_gain * x
                residual = self.dirty_data - _conv(model, data_fft, conv_mode, self.f64)
                std_last = std_current
                std_current = np.std(residual[sub_sl])
                std_ratio = (std_last - std_current) / std_last
                rec["std"] = float(std_current)
                rec["reverted"] = bool(std_ratio < 0)
                if std_ratio < 0:
                    model[sub_sl] -= loop_gain * x
                    residual = self.dirty_data - _conv(model, data_fft, conv_mode, self.f64)
                dirty_sub = residual[sub_sl]
                major += 1
                self.log.append(rec)
                now = time.perf_counter()
                self.timings["major"] += now - t_major
                self.timings["n_major"] += 1
                t_major = now
            if major == 0:
                self.complete = True
                break
        if major > 0:
            self.model += model
            self.residual = residual
        return major

    def moresane_by_scale(self, start_scale=1, stop_scale=20, **kw):
        dirty = self.dirty_data
        scale_count = start_scale
        while not self.complete:
            self.moresane(scale_count=scale_count, **kw)
            self.dirty_data = self.residual
            scale_count += 1
            if scale_count > (np.log2(self.dirty_data.shape[0])) - 1:
                break
            if scale_count > stop_scale:
                break
        self.dirty_data = dirty
        self.complete = False

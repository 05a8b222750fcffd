"""Drop-in for pymoresane.main: DataImage / FitsImage with a device-resident MORESANE.

The major loop (pymoresane/main.py:266-514), the conjugate-gradient minor
loop (:378-457) and moresane_by_scale (:523-599) run with every image, PSF
spectrum, coefficient stack, mask and CG vector resident on the GPU. Each
step is a libmsn kernel (C ABI, include/msn.h); the host only reads back the
scalars the reference's control flow branches on: the normalised scale
maxima, the SNR of each minor iteration, the positivity flag, the residual
standard deviation and the peak of the dirty subregion. The CG inner
products and step sizes are float64, the bulk arithmetic float32.

Signatures and defaults follow the reference except that the mode arguments
default to the GPU path ('gpu'); CPU modes raise ValueError (this package
has no CPU implementation).
"""
import ctypes
import logging
import math
import threading

import numpy as np
import torch

from . import _native
from .beam_fit import beam_fit
from . import device as dev
from . import fits
from . import tune

logger = logging.getLogger(__name__)


def _check_modes(all_on_gpu, decom_mode, conv_device, extraction_mode):
    if all_on_gpu:
        return
    bad = [f"{k}={v!r}" for k, v in (("decom_mode", decom_mode), ("conv_device", conv_device),
                                     ("extraction_mode", extraction_mode)) if v != "gpu"]
    if bad:
        raise ValueError("pymoresane_gb300 implements the GPU path only; got " + ", ".join(bad)
                         + " (use the 'gpu' modes or all_on_gpu=True)")


def _rects_for(slc, n):
    return slc.indices(n)[:2]


class _PsfCache:
    """PSF spectra and PSF scale energies, built once per (PSF, configuration) on the device."""

    def __init__(self):
        self.entries = {}

    def get(self, key, build):
        if key not in self.entries:
            self.entries[key] = build()
        return self.entries[key]


class _Buffers:
    """Per-(subregion, scale_count) device buffers reused across major iterations."""

    def __init__(self, ns, n_full, m_sub, m_data, scale_count, device):
        f32 = dict(dtype=torch.float32, device=device)
        s = scale_count
        self.dec = torch.empty((s, ns, ns), **f32)
        self.thr = torch.empty((s, ns, ns), **f32)
        self.emask = torch.empty((s, ns, ns), **f32)
        self.esrc = torch.empty((s, ns, ns), **f32)
        self.planes = torch.empty((s, ns, ns), **f32)
        self.ms = torch.empty((s, ns, ns), **f32)   # running model sources mask * W(H x)
        self.vec = {k: torch.empty((ns, ns), **f32)
                    for k in ("x", "xn", "r", "rn", "p", "ap", "tmp", "rec", "masked", "sub")}
        self.conv_full = torch.empty((n_full, n_full), **f32)
        self.iuwt_work = dev.iuwt_workspace(ns, ns, device)
        self.fft_work = dev.fft_workspace(ns, m_sub, device)
        self.fft_work_full = dev.fft_workspace(n_full, m_data, device)
        self.tool_work = dev.toolbox_workspace(s, ns, ns, device)
        self.red_work = dev.reduce_workspace(device)
        self.scal = torch.zeros(8, dtype=torch.float64, device=device)
        self.snr2 = torch.zeros(2, dtype=torch.float64, device=device)
        self.std4 = torch.zeros(4, dtype=torch.float64, device=device)
        self.neg = torch.zeros(1, dtype=torch.int32, device=device)
        self.small = torch.empty(256, dtype=torch.uint8, device=device)
        self.fmax = torch.empty(1, dtype=torch.float32, device=device)
        self.sigma = torch.empty(s, dtype=torch.float64, device=device)
        self.pmax = torch.empty(s, dtype=torch.float32, device=device)
        self.seg_flags = torch.empty(max(1, _native.query("msn_segment_flags_bytes", s * ns * ns)), dtype=torch.uint8,
                                     device=device)
        self.row_flags = torch.empty(s * ns, dtype=torch.uint8, device=device)
        self.rec_rows = torch.empty(s * ns, dtype=torch.uint8, device=device)


_ENGINES = threading.local()


def _thread_engine(device):
    """The calling thread's minor-loop engine for ``device``, created on first use and kept.

    Its graph cache is keyed by every buffer address, so a later Deconvolver
    whose buffers land at the same addresses re-uses the captured graphs.
    """
    engines = getattr(_ENGINES, "by_device", None)
    if engines is None:
        engines = _ENGINES.by_device = {}
    key = device.index
    if key not in engines:
        h = ctypes.c_void_p()
        _native.call("msn_minor_engine_create", ctypes.byref(h))
        engines[key] = h
    return engines[key]


def _replay(events):
    """Emit the log messages of a native run, in order (texts of pymoresane/main.py)."""
    for e in events:
        c = e.code
        if c == _native.EV_MINIMUM_SCALE:
            logger.info("Minimum scale = %d", e.a)
        elif c == _native.EV_MAXIMUM_SCALE:
            logger.info("Maximum scale = %d", e.a)
        elif c == _native.EV_SCALE_EMPTY:
            logger.info("Scale %d is empty. Ignoring scales <= %d", e.a, e.a)
        elif c == _native.EV_NO_COEFFICIENTS:
            logger.info("No significant wavelet coefficients detected.")
        elif c == _native.EV_MINOR_DONE:
            if e.b == _native.MINOR_FALSE_DETECTION:
                logger.info("SNR too large on first iteration - false detection. Incrementing the minimum scale.")
            elif e.b == _native.MINOR_CONVERGED:
                logger.info("Model has reached <1% error - exiting minor loop.")
            logger.info("%d minor loop iterations performed.", e.a)
        elif c == _native.EV_ALL_SCALES_POOR:
            logger.info("All scales are performing poorly - stopping.")
        elif c == _native.EV_REVERTED:
            logger.info("Residual has worsened - reverting changes.")
        elif c == _native.EV_MAJOR_DONE:
            logger.info("%d major loop iterations performed.", e.a)
        elif c == _native.EV_NO_WORK:
            logger.info("Current MORESANE iteration did no work - finished.")


class Deconvolver:
    """Device-resident MORESANE for one PSF (and optional mask) on the current CUDA device.

    ``psf`` and ``mask`` are CUDA tensors (or arrays, uploaded once); the PSF
    spectra, PSF scale energies and every work buffer are built on first use
    and kept for later calls. ``moresane(dirty, ...)`` takes a CUDA tensor and
    returns device tensors, so a caller can keep whole deconvolutions on the
    GPU; DataImage wraps it with the reference's host-array interface.
    """

    def __init__(self, psf, mask=None, dirty_shape=None, workspace=None):
        dev.require_cuda()
        tune.ensure_applied()  # this device's cached autotuner choices, once per process
        _native.load()
        self.device = torch.device("cuda", torch.cuda.current_device())
        self.psf = dev.as_f32_cuda(psf, device=self.device)
        self.mask = None if mask is None else dev.as_f32_cuda(mask, device=self.device)
        self.psf_data_shape = tuple(self.psf.shape)
        self.dirty_data_shape = dirty_shape
        self.log = []
        self.minor_total = 0  # minor iterations over every minor loop run so far
        self.complete = False
        # True: keep mask * W(H x) as a running sum (ms += alpha * mask * W(H p), exact by
        # linearity) instead of recomputing mask * W(H xn) with a convolution and a
        # decomposition every minor iteration as pymoresane/main.py:413-416 does.
        self.incremental_snr = True
        # True: each minor loop runs as one CUDA graph with its stop rules on the
        # device (msn_minor_loop); False: the host drives every iteration, as the
        # reference does (pymoresane/main.py:365-457).
        self.native_minor_loop = True
        # True: the whole major loop runs inside libmsn (msn_moresane_run), one call
        # per deconvolution; needs native_minor_loop. False: this module drives it.
        self.native_major_loop = True
        self._psf_cache = _PsfCache()
        self._bufs = {}
        # A Workspace (pymoresane_gb300.batch) shared by the deconvolutions that one
        # worker runs one after another: buffers, the sub-PSF spectrum slot and the
        # minor-loop engine (with its cached graphs) outlive this object.
        self.workspace = workspace

    def _spectra(self, subregion, conv_mode):
        """(spec_sub, spec_data, psf_subregion) per pymoresane/main.py:118-213 (GPU branches)."""
        psf = self.psf
        n = self.dirty_data_shape[0]
        p0 = self.psf_data_shape[0]
        double = all(p == 2 * d for p, d in zip(self.psf_data_shape, self.dirty_data_shape))
        full = subregion == n

        def crop(c, half):
            return psf[c - half:c + half, c - half:c + half].contiguous()

        def build():
            if double:
                psf_sub = crop(p0 // 2, subregion // 2)
            else:
                psf_sub = psf[n // 2 - subregion // 2:n // 2 + subregion // 2,
                              n // 2 - subregion // 2:n // 2 + subregion // 2].contiguous()
            if conv_mode == "circular":
                spec_sub = dev.psf_spectrum(psf_sub, m=subregion)
                if double:
                    spec_data = dev.psf_spectrum(crop(p0 // 2, n // 2), m=n)
                else:
                    spec_data = spec_sub if subregion == p0 else dev.psf_spectrum(psf, m=p0)
            elif conv_mode == "linear":
                if double:
                    if full:
                        spec_sub = spec_data = dev.psf_spectrum(psf, m=p0)
                    else:
                        spec_sub = dev.psf_spectrum(crop(p0 // 2, subregion), m=2 * subregion)
                        spec_data = dev.psf_spectrum(psf, m=p0)
                else:
                    if full:
                        spec_sub = spec_data = dev.psf_spectrum(psf, m=2 * p0)   # rfft2(pad_array(psf))
                    else:
                        spec_sub = dev.psf_spectrum(crop(p0 // 2, subregion), m=2 * subregion)
                        spec_data = dev.psf_spectrum(psf, m=2 * p0)
            else:
                raise ValueError(f"unknown conv_mode {conv_mode!r}")
            return spec_sub, spec_data, psf_sub

        return self._psf_cache.get((n, subregion, conv_mode), build)

    def _energies(self, psf_sub, scale_count, bufs):
        """||w_s||_2 of the PSF-subregion decomposition, as float32 (pymoresane/main.py:221-226)."""
        def build():
            ns = psf_sub.shape[0]
            dec = torch.empty((scale_count, ns, ns), dtype=torch.float32, device=psf_sub.device)
            dev.iuwt_decompose(psf_sub, scale_count, 0, out=dec, work=bufs.iuwt_work)
            sums = torch.empty((scale_count, 2), dtype=torch.float64, device=psf_sub.device)
            for s in range(scale_count):
                dev.dot2(dec[s].reshape(-1), dec[s].reshape(-1), out=sums[s], work=bufs.red_work)
            return np.sqrt(sums[:, 0].cpu().numpy()).astype(np.float32)
        return self._psf_cache.get(("energies", psf_sub.data_ptr(), scale_count), build)

    def _buffers(self, ns, scale_count, spec_sub, spec_data):
        key = (self.dirty_data_shape[0], ns, scale_count, spec_sub.m, spec_data.m)
        if self.workspace is not None:
            return self.workspace.buffers_for(key, lambda: _Buffers(ns, self.dirty_data_shape[0], spec_sub.m,
                                                                    spec_data.m, scale_count, self.device))
        if key not in self._bufs:
            self._bufs = {key: _Buffers(ns, self.dirty_data_shape[0], spec_sub.m, spec_data.m, scale_count,
                                        self.device)}
        return self._bufs[key]

    def _engine_handle(self):
        if self.workspace is not None:
            return self.workspace.engine()
        return _thread_engine(self.device)

    def _native_minor(self, B, V, spec_sub, linear, max_scale, scale_adjust, planes, ns, miter, positivity, st):
        """One minor loop through msn_minor_loop; returns (MinorResult, per-iteration SNRs)."""
        engine = self._engine_handle()
        a = _native.MinorArgs()
        a.n, a.m, a.linear = ns, spec_sub.m, 1 if linear else 0
        a.max_scale, a.scale_adjust = max_scale, scale_adjust
        a.minor_loop_miter, a.enforce_positivity = int(miter), 1 if positivity else 0
        a.spec = (B.spec_slot if self.workspace is not None else spec_sub.packed).data_ptr()
        a.rec = V["rec"].data_ptr()
        for name in ("x", "xn", "r", "rn", "p", "ap", "tmp"):
            setattr(a, name, V[name].data_ptr())
        a.planes, a.emask, a.esrc, a.ms = (B.planes.data_ptr(), B.emask.data_ptr(), B.esrc.data_ptr(),
                                           B.ms.data_ptr())
        a.scal, a.snr2, a.neg = B.scal.data_ptr(), B.snr2.data_ptr(), B.neg.data_ptr()
        a.seg_flags, a.row_flags, a.rec_rows = B.seg_flags.data_ptr(), B.row_flags.data_ptr(), B.rec_rows.data_ptr()
        a.fft_work, a.fft_work_bytes = B.fft_work.data_ptr(), B.fft_work.numel()
        a.iuwt_work, a.iuwt_work_bytes = B.iuwt_work.data_ptr(), B.iuwt_work.numel()
        a.red_work, a.red_work_bytes = B.red_work.data_ptr(), B.red_work.numel()
        res = _native.MinorResult()
        hist = (ctypes.c_double * max(int(miter), 1))()
        _native.call("msn_minor_loop", engine, ctypes.byref(a), ctypes.byref(res), hist, len(hist), st)
        return res, list(hist[:min(res.minor, len(hist))])

    def _native_run(self, dirty, B, spec_sub, spec_data, energies, mask_sub, supp, n, ns, o, scale_count, linear,
                    sigma_level, loop_gain, tolerance, accuracy, major_loop_miter, minor_loop_miter,
                    enforce_positivity, flux_threshold, neg_comp, edge_excl, int_excl, st):
        """The major loop through msn_moresane_run; log events are replayed into this module's logger."""
        engine = self._engine_handle()
        model = torch.empty((n, n), dtype=torch.float32, device=dirty.device)
        residual = torch.empty((n, n), dtype=torch.float32, device=dirty.device)
        energies_h = np.ascontiguousarray(energies, dtype=np.float32)
        V = B.vec
        a = _native.MoresaneArgs()
        a.n, a.ns, a.off, a.scale_count = n, ns, o, scale_count
        a.m_sub, a.m_data, a.linear = spec_sub.m, spec_data.m, 1 if linear else 0
        a.major_loop_miter, a.minor_loop_miter = int(major_loop_miter), int(minor_loop_miter)
        a.enforce_positivity, a.neg_comp = 1 if enforce_positivity else 0, 1 if neg_comp else 0
        a.noise_rects[:] = dev.noise_rects(ns, ns, edge_excl, int_excl)
        a.sigma_level, a.tolerance, a.accuracy = float(sigma_level), float(tolerance), float(accuracy)
        a.flux_threshold, a.loop_gain = float(flux_threshold), float(loop_gain)
        a.dirty = dirty.data_ptr()
        a.mask_sub = None if mask_sub is None else mask_sub.data_ptr()
        a.supp_rects = None if supp is None else supp.data_ptr()
        a.energies = energies_h.ctypes.data
        a.spec_sub = (B.spec_slot if self.workspace is not None else spec_sub.packed).data_ptr()
        a.spec_data = spec_data.packed.data_ptr()
        a.model, a.residual = model.data_ptr(), residual.data_ptr()
        for k in ("dec", "thr", "emask", "esrc", "planes", "ms", "conv_full", "sigma", "pmax", "scal", "snr2",
                  "std4", "neg", "seg_flags", "row_flags", "rec_rows", "fmax", "small"):
            setattr(a, k, getattr(B, k).data_ptr())
        for k in ("x", "xn", "r", "rn", "p", "ap", "tmp", "rec", "masked", "sub"):
            setattr(a, k, V[k].data_ptr())
        a.small_bytes = B.small.numel()
        for k in ("iuwt_work", "fft_work", "fft_work_full", "tool_work", "red_work"):
            w = getattr(B, k)
            setattr(a, k, w.data_ptr())
            setattr(a, k + "_bytes", w.numel())
        res = _native.MoresaneResult()
        cap = max(1, int(major_loop_miter))
        records = (_native.MajorRecord * cap)()
        events = (_native.Event * (cap * (4 * scale_count + 8) + 8))()
        _native.call("msn_moresane_run", engine, ctypes.byref(a), ctypes.byref(res), records, cap, events,
                     len(events), st)
        _replay(events[:res.n_events])
        self.minor_total += sum(e.a for e in events[:res.n_events] if e.code == _native.EV_MINOR_DONE)
        for r in records[:res.n_records]:
            self.log.append({"major": r.major, "max_scale": r.max_scale, "scale_adjust": r.scale_adjust,
                             "minor": r.minor, "snr": r.snr, "std": r.std, "reverted": bool(r.reverted)})
        self.complete = bool(res.complete)
        return model, (residual if res.have_residual else None), res.major

    def moresane(self, dirty, subregion=None, scale_count=None, sigma_level=4, loop_gain=0.1, tolerance=0.75,
                 accuracy=1e-6, major_loop_miter=100, minor_loop_miter=30, conv_mode='linear',
                 enforce_positivity=False, edge_suppression=False, edge_offset=0, flux_threshold=0, neg_comp=False,
                 edge_excl=0, int_excl=0):
        """One MORESANE run (pymoresane/main.py:99-521) on the device image ``dirty``.

        Returns (model, residual, major_iterations) as CUDA tensors (residual
        is None when no major iteration ran); sets ``self.complete`` when the
        run did no work, as the reference does.
        """
        dirty = dev.as_f32_cuda(dirty, device=self.device)
        self.dirty_data_shape = tuple(dirty.shape)
        self.complete = False
        n = self.dirty_data_shape[0]
        if n % 2 == 1:
            logger.error("Image size is uneven. Please use even dimensions.")
            raise ValueError("Image size is uneven. Please use even dimensions.")
        if subregion is None or subregion > n:
            subregion = n
        if scale_count is None or scale_count > (np.log2(n) - 1):
            scale_count = int(np.log2(n) - 1)
        ns = subregion
        o = n // 2 - ns // 2
        linear = conv_mode == "linear"
        spec_sub, spec_data, psf_sub = self._spectra(subregion, conv_mode)
        B = self._buffers(ns, scale_count, spec_sub, spec_data)
        if self.workspace is not None:
            # a fixed device address for the sub-PSF spectrum keeps the cached minor-loop graphs valid
            if getattr(B, "spec_slot", None) is None or B.spec_slot.shape != spec_sub.packed.shape:
                B.spec_slot = torch.empty_like(spec_sub.packed)
            B.spec_slot.copy_(spec_sub.packed)
        energies = self._energies(psf_sub, scale_count, B)
        st = dev.stream_handle()
        call = _native.call
        V = B.vec
        nvec = ns * ns
        mask_sub = None
        if self.mask is not None:
            mask_sub = self.mask[o:o + ns, o:o + ns].contiguous()

        supp = None
        if edge_suppression or edge_offset > 0:
            rects = []
            corruption = 0
            for i in range(scale_count):
                if edge_suppression:
                    corruption += 2 * 2 ** i
                    e = edge_offset if edge_offset > corruption else corruption
                else:
                    e = edge_offset
                y0, y1 = _rects_for(slice(e, -e), ns)
                rects.append([y0, y1, y0, y1])
            supp = torch.tensor(rects, dtype=torch.int32, device=dirty.device)

        if self.native_major_loop and self.native_minor_loop:
            return self._native_run(dirty, B, spec_sub, spec_data, energies, mask_sub, supp, n, ns, o, scale_count,
                                    linear, sigma_level, loop_gain, tolerance, accuracy, major_loop_miter,
                                    minor_loop_miter, enforce_positivity, flux_threshold, neg_comp, edge_excl,
                                    int_excl, st)

        def sub_view(img):
            return img if ns == n else img[o:o + ns, o:o + ns].contiguous()

        def apply_a(vec_in, vec_out, max_scale, adj, planes):
            # the same entry points as the native minor loop: the mask's empty rows are skipped in
            # the decomposition (Q is cleared at the start of the minor loop) and the recomposition
            # computes only the rows of its support (B.rec_rows)
            dev.fft_convolve(vec_in, spec_sub, linear, out=V["tmp"], work=B.fft_work)
            call("msn_iuwt_decompose_masked_rows", V["tmp"].data_ptr(), B.emask.data_ptr(), B.row_flags.data_ptr(),
                 B.planes.data_ptr(), ns, ns, max_scale, adj, B.iuwt_work.data_ptr(), B.iuwt_work.numel(), st)
            call("msn_iuwt_recompose_rows", B.planes.data_ptr(), planes, B.rec_rows.data_ptr(), vec_out.data_ptr(),
                 ns, ns, adj, B.iuwt_work.data_ptr(), B.iuwt_work.numel(), st)

        def residual_of(model):
            res = torch.empty((n, n), dtype=torch.float32, device=dirty.device)
            dev.fft_convolve(model, spec_data, linear, out=B.conv_full, work=B.fft_work_full)
            call("msn_sub", dirty.data_ptr(), B.conv_full.data_ptr(), res.data_ptr(), n * n, st)
            return res

        major = 0
        max_coeff = 1
        model = torch.zeros((n, n), dtype=torch.float32, device=dirty.device)
        std_current, std_ratio = 1000, 1
        min_scale = 0
        residual = None
        dirty_sub = sub_view(dirty)
        normalised = None
        have_x = False

        def dirty_peak():
            dev.plane_max(dirty_sub, out=B.fmax, work=B.small)
            return float(B.fmax.item())

        while (major < major_loop_miter and max_coeff > 0 and std_ratio > accuracy
               and dirty_peak() > flux_threshold):
            rec = {"major": major}
            while min_scale < scale_count:
                if min_scale == 0:
                    dev.iuwt_decompose(dirty_sub, scale_count, 0, out=B.dec, work=B.iuwt_work)
                    sigma = dev.mad_sigma(B.dec, edge_excl, int_excl, work=B.tool_work)
                    if mask_sub is not None:
                        masked = torch.empty_like(dirty_sub)
                        call("msn_mul", dirty_sub.data_ptr(), mask_sub.data_ptr(), masked.data_ptr(), nvec, st)
                        dev.iuwt_decompose(masked, scale_count, 0, out=B.dec, work=B.iuwt_work)
                    _, pmax = dev.apply_threshold(B.dec, sigma, sigma_level, supp_rects=supp, out=B.thr,
                                                  want_max=True, work=B.small)
                    normalised = pmax.cpu().numpy() / energies
                max_index = int(np.argmax(normalised[min_scale:])) + min_scale
                max_scale = max_index + 1
                max_coeff = normalised[max_index]
                if max_coeff == 0:
                    logger.info("No significant wavelet coefficients detected.")
                    break
                logger.info("Minimum scale = %d", min_scale)
                logger.info("Maximum scale = %d", max_scale)
                scale_adjust = 0
                for i in range(max_index - 1, -1, -1):
                    if normalised[i] == 0:
                        scale_adjust = i + 1
                        logger.info("Scale %d is empty. Ignoring scales <= %d", scale_adjust, scale_adjust)
                        break
                planes = max_scale - scale_adjust
                thr = B.thr[scale_adjust:max_scale]
                dev.source_extraction(thr, tolerance, neg_comp, mask=B.emask[:planes], extracted=B.esrc[:planes],
                                      work=B.tool_work)
                dev.iuwt_recompose(B.esrc[:planes], scale_adjust, out=V["rec"], work=B.iuwt_work)

                if self.native_minor_loop:
                    res, hist = self._native_minor(B, V, spec_sub, linear, max_scale, scale_adjust, planes, ns,
                                                   minor_loop_miter, enforce_positivity, st)
                    minor, snr_current = res.minor, res.snr_current
                    for i, v in enumerate(hist):
                        logger.debug("SNR at iteration %d = %s", i + 1, v)
                    if res.outcome == _native.MINOR_FALSE_DETECTION:
                        logger.info("SNR too large on first iteration - false detection. "
                                    "Incrementing the minimum scale.")
                        min_scale += 1
                    elif res.outcome == _native.MINOR_CONVERGED:
                        logger.info("Model has reached <1% error - exiting minor loop.")
                        min_scale = 0
                    elif res.outcome == _native.MINOR_STALLED:
                        min_scale = 0 if snr_current > 10.5 else min_scale + 1
                else:
                    x, xn, r, rn, p, ap = V["x"], V["xn"], V["r"], V["rn"], V["p"], V["ap"]
                    x.zero_()
                    if self.incremental_snr:
                        B.ms[:planes].zero_()
                    # supports of the (fixed) extraction mask, as the native minor loop's prologue
                    B.planes[:planes].zero_()
                    call("msn_segment_flags", B.emask.data_ptr(), planes * nvec, B.seg_flags.data_ptr(), st)
                    call("msn_row_flags", B.emask.data_ptr(), planes * ns, ns, B.row_flags.data_ptr(), st)
                    call("msn_recompose_row_activity", B.row_flags.data_ptr(), planes, ns, scale_adjust,
                         B.rec_rows.data_ptr(), st)
                    r.copy_(V["rec"])
                    p.copy_(V["rec"])
                    minor = 0
                    snr_last = snr_current = 0.0
                    while minor < minor_loop_miter:
                        apply_a(p, ap, max_scale, scale_adjust, planes)
                        dev.dot2(r.reshape(-1), r.reshape(-1), p.reshape(-1), ap.reshape(-1), out=B.scal[0:2],
                                 work=B.red_work)
                        call("msn_cg_alpha_x", x.data_ptr(), p.data_ptr(), B.scal.data_ptr(), xn.data_ptr(), nvec,
                             B.neg.data_ptr(), st)
                        if enforce_positivity and int(B.neg.item()) > 0:
                            call("msn_cg_positivity", x.data_ptr(), xn.data_ptr(), p.data_ptr(), B.scal.data_ptr(),
                                 nvec, st)
                            apply_a(p, ap, max_scale, scale_adjust, planes)
                        call("msn_cg_residual", r.data_ptr(), ap.data_ptr(), B.scal.data_ptr(), rn.data_ptr(), nvec,
                             B.red_work.data_ptr(), B.red_work.numel(), st)
                        call("msn_cg_direction", rn.data_ptr(), p.data_ptr(), B.scal.data_ptr(), nvec, st)
                        # model_sources = mask * W(H xn) and the SNR against the extracted sources
                        if self.incremental_snr:
                            # ms += alpha * (mask * W(H p)), the plane stack left in B.planes by apply_a
                            call("msn_snr_update_masked", B.esrc.data_ptr(), B.ms.data_ptr(), B.planes.data_ptr(),
                                 B.scal.data_ptr(), planes * nvec, B.seg_flags.data_ptr(), B.snr2.data_ptr(),
                                 B.red_work.data_ptr(), B.red_work.numel(), st)
                        else:
                            dev.fft_convolve(xn, spec_sub, linear, out=V["tmp"], work=B.fft_work)
                            w = B.planes[:planes]
                            dev.iuwt_decompose_masked(V["tmp"], B.emask, max_scale, scale_adjust, out=w,
                                                      work=B.iuwt_work)
                            dev.snr_sums(B.esrc[:planes].reshape(-1), w.reshape(-1), out=B.snr2, work=B.red_work)
                        s2 = B.snr2.cpu().numpy()
                        snr_last = snr_current
                        with np.errstate(divide="ignore", invalid="ignore"):
                            snr_current = float(20 * np.log10(np.sqrt(s2[0]) / np.sqrt(s2[1])))
                        minor += 1
                        logger.debug("SNR at iteration %d = %s", minor, snr_current)
                        if minor == 1 and snr_current > 40:
                            logger.info("SNR too large on first iteration - false detection. "
                                        "Incrementing the minimum scale.")
                            min_scale += 1
                            break
                        if snr_current > 40:
                            logger.info("Model has reached <1% error - exiting minor loop.")
                            V["x"], V["xn"] = xn, x
                            x, xn = xn, x
                            min_scale = 0
                            break
                        if minor > 2 and snr_current <= snr_last:
                            if snr_current > 10.5:
                                min_scale = 0
                            else:
                                min_scale += 1
                            break
                        V["r"], V["rn"] = rn, r
                        r, rn = rn, r
                        V["x"], V["xn"] = xn, x
                        x, xn = xn, x
                have_x = True
                self.minor_total += minor
                logger.info("%d minor loop iterations performed.", minor)
                rec.update(max_scale=max_scale, scale_adjust=scale_adjust, minor=minor, snr=snr_current)
                if minor == minor_loop_miter and snr_current > 10.5:
                    min_scale = 0
                    break
                if min_scale == 0:
                    break
            if min_scale == scale_count:
                logger.info("All scales are performing poorly - stopping.")
                break
            if max_coeff > 0 and have_x:
                x = V["x"]
                call("msn_model_update", model.data_ptr(), n, x.data_ptr(), ns, o, o, float(loop_gain), 1, st)
                residual = residual_of(model)
                std_last = std_current
                call("msn_region_std", residual.data_ptr(), n, ns, ns, o, o, B.std4.data_ptr(),
                     B.red_work.data_ptr(), B.red_work.numel(), st)
                std_current = float(B.std4[3].item())
                std_ratio = (std_last - std_current) / std_last
                rec["std"] = std_current
                rec["reverted"] = bool(std_ratio < 0)
                if std_ratio < 0:
                    logger.info("Residual has worsened - reverting changes.")
                    call("msn_model_update", model.data_ptr(), n, x.data_ptr(), ns, o, o, float(loop_gain), -1, st)
                    residual = residual_of(model)
                dirty_sub = sub_view(residual)
                major += 1
                self.log.append(rec)
                logger.info("%d major loop iterations performed.", major)
            if major == 0:
                logger.info("Current MORESANE iteration did no work - finished.")
                self.complete = True
                break
        return model, residual, major



class DataImage(object):
    """MORESANE on one dirty image / PSF pair with host arrays (pymoresane/main.py:18-676)."""

    def __init__(self, dirty_data, psf_data, mask_data, cdelt1, cdelt2):
        self.dirty_data = np.asarray(dirty_data).astype(np.float32)
        self.psf_data = np.asarray(psf_data).astype(np.float32)
        self.mask_name = None if mask_data is None else getattr(self, "mask_name", "mask")
        self.mask = None if mask_data is None else np.asarray(mask_data)
        self.dirty_data_shape = self.dirty_data.shape
        self.psf_data_shape = self.psf_data.shape
        self.complete = False
        self.model = np.zeros_like(self.dirty_data)
        self.residual = np.copy(self.dirty_data)
        self.restored = np.zeros_like(self.dirty_data)
        self.cdelt1 = cdelt1
        self.cdelt2 = cdelt2
        self._engine = None

    @property
    def engine(self):
        if self._engine is None:
            mask = None if self.mask is None else np.ascontiguousarray(self.mask, dtype=np.float32)
            self._engine = Deconvolver(np.ascontiguousarray(self.psf_data), mask, self.dirty_data_shape)
        return self._engine

    @property
    def log(self):
        return self.engine.log

    def moresane(self, subregion=None, scale_count=None, sigma_level=4, loop_gain=0.1, tolerance=0.75, accuracy=1e-6,
                 major_loop_miter=100, minor_loop_miter=30, all_on_gpu=False, decom_mode="gpu", core_count=1,
                 conv_device='gpu', conv_mode='linear', extraction_mode='gpu', enforce_positivity=False,
                 edge_suppression=False, edge_offset=0, flux_threshold=0, neg_comp=False, edge_excl=0, int_excl=0):
        """MORESANE deconvolution (pymoresane/main.py:53-521); updates self.model and self.residual."""
        _check_modes(all_on_gpu, decom_mode, conv_device, extraction_mode)
        eng = self.engine
        dirty = torch.from_numpy(np.ascontiguousarray(self.dirty_data)).to(eng.device)
        model, residual, major = eng.moresane(
            dirty, subregion, scale_count, sigma_level, loop_gain, tolerance, accuracy, major_loop_miter,
            minor_loop_miter, conv_mode, enforce_positivity, edge_suppression, edge_offset, flux_threshold,
            neg_comp, edge_excl, int_excl)
        self.complete = eng.complete
        if major > 0:
            self.model += model.cpu().numpy()
            self.residual = residual.cpu().numpy()
        return major

    def moresane_by_scale(self, start_scale=1, stop_scale=20, subregion=None, sigma_level=4, loop_gain=0.1,
                          tolerance=0.75, accuracy=1e-6, major_loop_miter=100, minor_loop_miter=30, all_on_gpu=False,
                          decom_mode="gpu", core_count=1, conv_device='gpu', conv_mode='linear',
                          extraction_mode='gpu', enforce_positivity=False, edge_suppression=False, edge_offset=0,
                          flux_threshold=0, neg_comp=False, edge_excl=0, int_excl=0):
        """Scale-by-scale MORESANE (pymoresane/main.py:523-599), residual kept on the device between scales."""
        _check_modes(all_on_gpu, decom_mode, conv_device, extraction_mode)
        eng = self.engine
        d = eng.device
        dirty = torch.from_numpy(np.ascontiguousarray(self.dirty_data)).to(d)
        model_acc = torch.from_numpy(np.ascontiguousarray(self.model)).to(d)
        residual = torch.from_numpy(np.ascontiguousarray(self.residual)).to(d)
        n = self.dirty_data_shape[0]
        st = dev.stream_handle()
        scale_count = start_scale
        self.complete = False
        while not self.complete:
            logger.info("MORESANE at scale %d", scale_count)
            model, res, major = eng.moresane(
                dirty, subregion, scale_count, sigma_level, loop_gain, tolerance, accuracy, major_loop_miter,
                minor_loop_miter, conv_mode, enforce_positivity, edge_suppression, edge_offset, flux_threshold,
                neg_comp, edge_excl, int_excl)
            self.complete = eng.complete
            if major > 0:
                _native.call("msn_model_update", model_acc.data_ptr(), n, model.data_ptr(), n, 0, 0, 1.0, 1, st)
                residual = res
            dirty = residual
            scale_count += 1
            if scale_count > (np.log2(n)) - 1:
                logger.info("Maximum scale reached - finished.")
                break
            if scale_count > stop_scale:
                logger.info("Maximum scale reached - finished.")
                break
        self.model = model_acc.cpu().numpy()
        self.residual = residual.cpu().numpy()
        self.complete = False

    def restore(self):
        """Restored image: model convolved with the fitted clean beam, plus the residual (main.py:601-616).

        The beam fit runs on the host (pymoresane_gb300.beam_fit); the
        convolution (linear for a double-size PSF, circular for a same-size one,
        as the reference) and the addition run on the GPU. Sets self.restored
        (float32) and returns [bmaj, bmin, bpa].
        """
        clean_beam, beam_params = beam_fit(self.psf_data, self.cdelt1, self.cdelt2)
        self.restore_with(clean_beam)
        return beam_params

    def restore_with(self, clean_beam):
        """The GPU half of restore(): self.restored = model (*) clean_beam + residual (main.py:607-615)."""
        n, p = tuple(self.dirty_data_shape), tuple(self.psf_data_shape)
        if p == tuple(2 * d for d in n):
            linear = True
        elif p == n:
            linear = False
        else:
            raise ValueError(f"restore needs a PSF of the image's size or twice it; got {p} for {n}")
        dev.require_cuda()
        device = torch.device("cuda", torch.cuda.current_device())
        spec = dev.psf_spectrum(torch.from_numpy(np.ascontiguousarray(clean_beam, dtype=np.float32)).to(device),
                                m=p[0], off_r=0, off_c=0)
        model = torch.from_numpy(np.ascontiguousarray(self.model, dtype=np.float32)).to(device)
        residual = torch.from_numpy(np.ascontiguousarray(self.residual, dtype=np.float32)).to(device)
        beam_model = dev.fft_convolve(model, spec, linear)
        restored = torch.empty_like(beam_model)
        _native.call("msn_add", beam_model.data_ptr(), residual.data_ptr(), restored.data_ptr(), restored.numel(),
                     dev.stream_handle())
        self.restored = restored.cpu().numpy()
        return self.restored

    # ------------------------------------------------------------------ outputs
    def save_fits(self, data, name):
        data = np.asarray(data).reshape(1, 1, data.shape[0], data.shape[0])
        fits.write(name, data, getattr(self, "img_hdr", None))

    def make_logger(self, level="INFO"):
        level = getattr(logging, level.upper())
        lg = logging.getLogger(__name__)
        lg.setLevel(logging.DEBUG)
        fh = logging.FileHandler('PyMORESANE.log', mode='w')
        fh.setLevel(level)
        ch = logging.StreamHandler()
        ch.setLevel(level)
        fmt = logging.Formatter('%(asctime)s [%(levelname)s]: %(message)s', datefmt='[%m/%d/%Y] [%I:%M:%S]')
        fh.setFormatter(fmt)
        ch.setFormatter(fmt)
        lg.addHandler(fh)
        lg.addHandler(ch)
        return lg


class FitsImage(DataImage):
    """DataImage read from FITS files (pymoresane/main.py:678-733), without astropy."""

    def __init__(self, image_name, psf_name, mask_name=None):
        self.image_name = image_name
        self.psf_name = psf_name
        self.mask_name = mask_name
        img, self.img_hdr = fits.read(image_name)
        psf, self.psf_hdr = fits.read(psf_name)
        cdelt1 = self.psf_hdr['CDELT1']
        cdelt2 = self.psf_hdr['CDELT1']   # the reference reads CDELT1 twice (main.py:704-705)
        mask = None
        if mask_name is not None:
            from scipy.signal import fftconvolve
            m, mhdr = fits.read(mask_name)
            m = m[tuple(self.handle_input(mhdr))].astype(np.float64)
            m = m / np.max(m)
            m = fftconvolve(m, np.ones([5, 5]), mode="same")
            mask = m / np.max(m)
        super(FitsImage, self).__init__(dirty_data=img[tuple(self.handle_input(self.img_hdr))],
                                        psf_data=psf[tuple(self.handle_input(self.psf_hdr))],
                                        mask_data=mask, cdelt1=cdelt1, cdelt2=cdelt2)
        self.mask_name = mask_name

    def handle_input(self, input_hdr):
        """Index selecting the RA/DEC plane of an N-D FITS cube (pymoresane/main.py:618-634)."""
        input_slice = input_hdr['NAXIS'] * [0]
        for i in range(input_hdr['NAXIS']):
            if str(input_hdr.get('CTYPE%d' % (i + 1), "")).startswith("RA"):
                input_slice[-1] = slice(None)
            if str(input_hdr.get('CTYPE%d' % (i + 1), "")).startswith("DEC"):
                input_slice[-2] = slice(None)
        return input_slice

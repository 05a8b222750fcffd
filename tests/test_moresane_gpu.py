"""GPU MORESANE (DataImage / FitsImage) against the reference's own runs.

Golden runs (tests/golden/moresane.npz, tart.npz) were produced by the
reference PyMORESANE itself (tests/golden/make_golden.py). Acceptance, per
case: the same number of major iterations (+-1 allowed), the model within
1e-4 of its peak and the residual standard deviation within 1e-4 relative.
The per-major-iteration decisions (max_scale, scale_adjust, minor count) are
also compared against the oracle's log.
"""
import os
import sys

import numpy as np
import pytest

from oracle.moresane import MoresaneOracle
from pymoresane_gb300.main import DataImage, FitsImage

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(__file__)
GOLDEN = os.path.join(HERE, "golden")
sys.path.insert(0, GOLDEN)
import cases as mg  # noqa: E402

MODEL_TOL = 1e-4   # max |model - reference| / max |reference model|
STD_TOL = 1e-4     # relative residual-std difference


def run_case(name):
    g = np.load(os.path.join(GOLDEN, "moresane.npz"))
    pk, rk = mg.MORESANE_CASES[name]
    kw = dict(mg.RUN_DEFAULTS, **rk)
    img = DataImage(g[f"{name}_dirty"], g[f"{name}_psf"], None, 1.0, 1.0)
    img.moresane(**kw)
    return g, kw, img


@pytest.mark.parametrize("name", list(mg.MORESANE_CASES))
def test_moresane_matches_reference(cuda, name):
    g, kw, img = run_case(name)
    ref_m, ref_r = g[f"{name}_model"], g[f"{name}_residual"]
    assert img.model.dtype == np.float32 and img.residual.dtype == ref_r.dtype
    assert np.max(np.abs(img.model - ref_m)) <= MODEL_TOL * np.max(np.abs(ref_m))
    assert abs(np.std(img.residual) - np.std(ref_r)) <= STD_TOL * np.std(ref_r)
    o = MoresaneOracle(g[f"{name}_dirty"], g[f"{name}_psf"])
    o.moresane(**kw)
    assert abs(len(o.log) - len(img.log)) <= 1
    same = [(a["max_scale"], a["scale_adjust"], a["minor"]) == (b["max_scale"], b["scale_adjust"], b["minor"])
            for a, b in zip(o.log, img.log)]
    assert all(same), (o.log, img.log)


def test_moresane_vs_fp64_oracle(cuda):
    # The error statement against the float64 oracle (reference casts removed).
    g, kw, img = run_case("lin_double")
    o = MoresaneOracle(g["lin_double_dirty"], g["lin_double_psf"], precision="f64")
    o.moresane(**kw)
    assert np.max(np.abs(img.model - o.model)) <= MODEL_TOL * np.max(np.abs(o.model))
    assert abs(np.std(img.residual) - np.std(o.residual)) <= STD_TOL * np.std(o.residual)


def test_moresane_deterministic(cuda):
    _, _, a = run_case("circ_pos")
    _, _, b = run_case("circ_pos")
    assert np.array_equal(a.model, b.model) and np.array_equal(a.residual, b.residual)


def test_tart_fits_by_scale(cuda):
    # tests/Makefile:8 of the reference: runsane -ep dirty beam (by-scale, circular, gain 0.2, minor 50).
    t = np.load(os.path.join(GOLDEN, "tart.npz"))
    img = FitsImage(os.path.join(GOLDEN, "tart_dirty.fits"), os.path.join(GOLDEN, "tart_beam.fits"))
    img.moresane_by_scale(1, 20, subregion=256, sigma_level=4, loop_gain=0.2, tolerance=0.75, accuracy=1e-6,
                          major_loop_miter=100, minor_loop_miter=50, conv_mode="circular", enforce_positivity=True)
    assert np.max(np.abs(img.model - t["model"])) <= MODEL_TOL * np.max(t["model"])
    assert abs(np.std(img.residual) - np.std(t["residual"])) <= STD_TOL * np.std(t["residual"])
    assert abs(float(img.model.sum()) - float(t["model"].sum())) <= 1e-4 * float(t["model"].sum())


def test_save_fits_roundtrip(cuda, tmp_path):
    from pymoresane_gb300 import fits
    img = FitsImage(os.path.join(GOLDEN, "tart_dirty.fits"), os.path.join(GOLDEN, "tart_beam.fits"))
    out = tmp_path / "m.fits"
    img.save_fits(img.dirty_data, str(out))
    data, hdr = fits.read(str(out))
    assert data.shape == (1, 1, 256, 256) and hdr["CDELT1"] == 0.703125
    assert np.array_equal(data[0, 0], img.dirty_data)


def test_errors(cuda):
    with pytest.raises(ValueError):
        DataImage(np.zeros((63, 63), np.float32), np.zeros((126, 126), np.float32), None, 1, 1).moresane()
    img = DataImage(np.zeros((64, 64), np.float32), np.zeros((128, 128), np.float32), None, 1, 1)
    with pytest.raises(ValueError):
        img.moresane(decom_mode="ser", conv_device="gpu", extraction_mode="gpu")
    # all_on_gpu overrides the individual modes, as in the reference (main.py:113-116)
    img.moresane(all_on_gpu=True, decom_mode="ser", conv_device="cpu", extraction_mode="cpu", major_loop_miter=1)


@pytest.mark.parametrize("name", ["lin_double", "circ_pos", "neg_excl"])
def test_incremental_model_sources_same_decisions(cuda, name):
    # The running model sources (ms += alpha mask W(H p)) against the reference's direct
    # recomputation of mask W(H xn) every minor iteration: same decisions, same model.
    from pymoresane_gb300.main import Deconvolver
    import torch
    g = np.load(os.path.join(GOLDEN, "moresane.npz"))
    pk, rk = mg.MORESANE_CASES[name]
    kw = dict(mg.RUN_DEFAULTS, **rk)
    dirty = torch.from_numpy(g[f"{name}_dirty"]).cuda()
    runs = []
    for inc in (True, False):
        eng = Deconvolver(g[f"{name}_psf"])
        eng.native_minor_loop = False
        eng.incremental_snr = inc
        model, residual, major = eng.moresane(dirty, **kw)
        runs.append((eng.log, model.cpu().numpy()))
    (la, ma), (lb, mb) = runs
    assert [(r["max_scale"], r["scale_adjust"], r["minor"]) for r in la] == \
           [(r["max_scale"], r["scale_adjust"], r["minor"]) for r in lb]
    assert np.max(np.abs(ma - mb)) <= MODEL_TOL * np.max(np.abs(mb))


@pytest.mark.parametrize("name", ["lin_double", "circ_pos", "neg_excl"])
def test_native_minor_loop_matches_host_loop(cuda, name):
    # One CUDA graph per minor loop with the stop rules on the device against the
    # host-driven loop: same decisions, same iteration counts, the same model bit for bit.
    # The graph's passes (the row-support dot product, the fused CG step / SNR pass, r.r
    # carried from rn.rn) keep the host loop's separate kernels' sums and orders.
    from pymoresane_gb300.main import Deconvolver
    import torch
    g = np.load(os.path.join(GOLDEN, "moresane.npz"))
    pk, rk = mg.MORESANE_CASES[name]
    kw = dict(mg.RUN_DEFAULTS, **rk)
    dirty = torch.from_numpy(g[f"{name}_dirty"]).cuda()
    runs = []
    for native in (True, False):
        eng = Deconvolver(g[f"{name}_psf"])
        eng.native_minor_loop = native
        model, residual, major = eng.moresane(dirty, **kw)
        runs.append((eng.log, model.cpu().numpy(), major))
    (la, ma, ka), (lb, mb, kb) = runs
    assert ka == kb
    assert [(r["max_scale"], r["scale_adjust"], r["minor"]) for r in la] == \
           [(r["max_scale"], r["scale_adjust"], r["minor"]) for r in lb]
    assert np.array_equal(ma, mb)


@pytest.mark.parametrize("name", ["lin_double", "circ_pos", "neg_excl"])
def test_native_major_loop_matches_host_major_loop(cuda, name, caplog):
    # The whole major loop inside libmsn (msn_moresane_run) against this package's
    # host-driven major loop over the same calls: identical model, residual, records
    # and log messages.
    import logging

    from pymoresane_gb300.main import Deconvolver
    import torch
    g = np.load(os.path.join(GOLDEN, "moresane.npz"))
    pk, rk = mg.MORESANE_CASES[name]
    kw = dict(mg.RUN_DEFAULTS, **rk)
    dirty = torch.from_numpy(g[f"{name}_dirty"]).cuda()
    runs = []
    for native in (True, False):
        caplog.clear()
        with caplog.at_level(logging.INFO, logger="pymoresane_gb300.main"):
            eng = Deconvolver(g[f"{name}_psf"])
            eng.native_major_loop = native
            model, residual, major = eng.moresane(dirty, **kw)
        msgs = [r.getMessage() for r in caplog.records if r.levelno >= logging.INFO]
        runs.append((model.cpu().numpy(), None if residual is None else residual.cpu().numpy(), major, eng.log,
                     msgs, eng.complete))
    (ma, ra, ka, la, ga, ca), (mb, rb, kb, lb, gb, cb) = runs
    assert ka == kb and ca == cb
    assert np.array_equal(ma, mb)
    assert (ra is None) == (rb is None) and (ra is None or np.array_equal(ra, rb))
    keys = ("major", "max_scale", "scale_adjust", "minor", "reverted")
    assert [[r[k] for k in keys] for r in la] == [[r[k] for k in keys] for r in lb]
    assert ga == gb


def test_engine_rejects_bad_arguments(cuda):
    """msn_minor_loop / msn_moresane_run validate their argument blocks before touching the device."""
    import ctypes

    from pymoresane_gb300 import _native
    h = ctypes.c_void_p()
    _native.call("msn_minor_engine_create", ctypes.byref(h))
    try:
        a, r = _native.MinorArgs(), _native.MinorResult()
        a.n, a.max_scale, a.scale_adjust, a.minor_loop_miter = 30, 3, 0, 5      # n not a multiple of 4
        with pytest.raises(ValueError, match="multiple of 4"):
            _native.call("msn_minor_loop", h, ctypes.byref(a), ctypes.byref(r), None, 0, None)
        a.n, a.max_scale = 64, 7                                                  # 2^7 > 64
        with pytest.raises(ValueError, match="exceeds the side"):
            _native.call("msn_minor_loop", h, ctypes.byref(a), ctypes.byref(r), None, 0, None)
        a.max_scale = 3                                                           # buffers missing
        with pytest.raises(ValueError, match="null buffer"):
            _native.call("msn_minor_loop", h, ctypes.byref(a), ctypes.byref(r), None, 0, None)
        m, mr = _native.MoresaneArgs(), _native.MoresaneResult()
        m.n, m.ns, m.off, m.scale_count = 64, 32, 40, 3                           # subregion outside the image
        with pytest.raises(ValueError, match="bad sides"):
            _native.call("msn_moresane_run", h, ctypes.byref(m), ctypes.byref(mr), None, 0, None, 0, None)
    finally:
        _native.query("msn_minor_engine_destroy", h)

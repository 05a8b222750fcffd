"""Generate the golden fixtures in tests/golden/ by running the reference itself.

The reference PyMORESANE (Python 2 sources) is loaded under Python 3 by
``refshim.load_reference()`` -- syntactic patches only, see refshim.py -- and
its own 'ser' / 'mp' / 'cpu' code paths are executed on small seeded inputs.
The outputs are stored as compressed .npz files that pin the CPU oracle
(``oracle/``) in tests/test_oracle_golden.py.

Run from the repository root in a checkout where the reference sources exist:
    python tests/golden/make_golden.py [--only NAME ...]
The GPU machine never runs this script; it only reads the committed fixtures.
"""
import argparse
import hashlib
import logging
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import refshim  # noqa: E402
from cases import (BASELINE_2048_RUN, BASELINE_RUN, MORESANE_CASES, RUN_DEFAULTS,  # noqa: E402
                   parse_major_log, problem, restore_inputs)


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    print("wrote", path, sum(a.nbytes for a in map(np.asarray, arrays.values())), "bytes raw")


def gen_iuwt(ref):
    rng = np.random.default_rng(1234)
    x = rng.standard_normal((48, 64))
    x[10, 20] += 40.0
    x[30, 5] += 25.0
    out = {"x": x}
    for adj in (0, 1, 2):
        d, c = ref.iuwt.iuwt_decomposition(x, 4, adj, "ser", store_smoothed=True)
        out[f"ser_detail_adj{adj}"] = d
        out[f"ser_smoothed_adj{adj}"] = c
        out[f"ser_recomp_smoothed_adj{adj}"] = ref.iuwt.iuwt_recomposition(d, adj, "ser", smoothed_array=c)
        out[f"ser_recomp_zero_adj{adj}"] = ref.iuwt.iuwt_recomposition(d, adj, "ser")
    xs = x[:32, :32].astype(np.float32)
    out["mp_x"] = xs
    d, c = ref.iuwt.iuwt_decomposition(xs, 3, 1, "mp", core_count=2, store_smoothed=True)
    out["mp_detail_adj1"] = d
    out["mp_smoothed_adj1"] = c
    out["mp_recomp_adj1"] = ref.iuwt.iuwt_recomposition(d, 1, "mp", core_count=2, smoothed_array=c)
    save("iuwt", **out)


def gen_conv(ref):
    from pymoresane_gb300.synthetic import make_psf
    rng = np.random.default_rng(99)
    x = rng.standard_normal((64, 64)).astype(np.float32)
    psf2 = make_psf(128, 400, np.random.default_rng(5))
    psf1 = make_psf(64, 200, np.random.default_rng(6))
    h2 = np.fft.rfft2(psf2)
    h1 = np.fft.rfft2(psf1)
    conv = ref.iuwt_convolution
    save("conv", x=x, psf2=psf2, psf1=psf1,
         linear=conv.fft_convolve(x, h2, "cpu", "linear"),
         circular=conv.fft_convolve(x, h1, "cpu", "circular"),
         pad=conv.pad_array(x))


def gen_toolbox(ref):
    from pymoresane_gb300 import synthetic
    dirty, psf, _ = synthetic.make_problem(synthetic.Workload(n=128, n_uv=800, n_points=12, n_gauss=2,
                                                              sigma_range=(2.0, 5.0), noise=1e-2, seed=21))
    tb = ref.iuwt_toolbox
    d = ref.iuwt.iuwt_decomposition(dirty, 5, 0, "ser").astype(np.float32)
    out = {"decomp": d}
    for ee, ie in ((0, 0), (3, 0), (0, 5), (4, 7), (0, 70)):
        out[f"thr_{ee}_{ie}"] = tb.estimate_threshold(d, ee, ie)
    thr = out["thr_0_0"]
    dt = tb.apply_threshold(d, thr, sigma_level=4)
    out["thresh"] = dt
    out["thresh_2d"] = tb.apply_threshold(d[1], thr[1], sigma_level=3)
    for neg in (False, True):
        src, msk = tb.source_extraction(dt[1:4], 0.75, mode="cpu", neg_comp=neg)
        out[f"src_neg{int(neg)}"] = src
        out[f"mask_neg{int(neg)}"] = msk
    out["snr"] = np.array(tb.snr_ratio(dt[1:4].astype(np.float64), d[1:4]))
    save("toolbox", **out)


def gen_moresane(ref):
    out = {}
    for name, (pk, rk) in MORESANE_CASES.items():
        dirty, psf, _ = problem(**pk)
        kw = dict(RUN_DEFAULTS, **rk)
        kw.setdefault("subregion", dirty.shape[0])
        img = ref.main.DataImage(dirty, psf, None, 1.0, 1.0)
        img.moresane(**kw)
        out[f"{name}_dirty"] = dirty
        out[f"{name}_psf"] = psf
        out[f"{name}_model"] = img.model
        out[f"{name}_residual"] = img.residual
        print(name, float(img.model.sum()), float(np.count_nonzero(img.model)), float(img.residual.std()))
    save("moresane", **out)


def read_fits(path):
    raw = open(path, "rb").read()
    hdr = raw[:2880].decode()
    cards = {hdr[i:i + 8].strip(): hdr[i + 10:i + 80].split("/")[0].strip() for i in range(0, 2880, 80)}
    n1, n2 = int(cards["NAXIS1"]), int(cards["NAXIS2"])
    return np.frombuffer(raw[2880:2880 + 8 * n1 * n2], dtype=">f8").reshape(n2, n1).astype(np.float64)


def gen_tart(ref):
    root = os.path.join(refshim.REF_ROOT, "tests")
    dirty = read_fits(os.path.join(root, "dirty_2017-10-15_20:33:35_UTC.fits"))
    beam = read_fits(os.path.join(root, "beam_2017-10-15_20:33:35_UTC.fits"))
    img = ref.main.DataImage(dirty, beam, None, 0.703125, 0.703125)
    img.moresane_by_scale(1, 20, subregion=256, sigma_level=4, loop_gain=0.2, tolerance=0.75, accuracy=1e-6,
                          major_loop_miter=100, minor_loop_miter=50, conv_mode="circular",
                          enforce_positivity=True)
    print("tart", float(img.model.sum()), float(img.model.max()), int(np.count_nonzero(img.model)),
          float(img.residual.std()))
    save("tart", model=img.model, residual=img.residual)


def gen_restore(ref):
    """beam_fit (beam_fit.py:6-69) on three PSF sizes and DataImage.restore (main.py:601-616).

    The clean beams are stored as their non-zero bounding box (they are zero
    elsewhere); the PSFs, models and residuals are regenerated from seeds.
    """
    psfs, cases = restore_inputs()
    out = {}
    for tag, psf in psfs.items():
        beam, params = ref.beam_fit.beam_fit(psf, 0.5, 0.25)
        nz = np.nonzero(beam)
        r0, r1, c0, c1 = nz[0].min(), nz[0].max() + 1, nz[1].min(), nz[1].max() + 1
        out[f"{tag}_beam_box"] = np.array([r0, r1, c0, c1])
        out[f"{tag}_beam_crop"] = beam[r0:r1, c0:c1]
        out[f"{tag}_params"] = np.asarray(params, np.float64)
    for tag, (ptag, model, residual) in cases.items():
        img = ref.main.DataImage(np.zeros_like(model), psfs[ptag], None, 0.5, 0.25)
        img.model = model
        img.residual = residual
        out[f"{tag}_restore_params"] = np.asarray(img.restore(), np.float64)
        out[f"{tag}_restored"] = img.restored
    save("restore", **out)


class _InfoLines(logging.Handler):
    """Collects the INFO messages of the reference's logger (pymoresane/main.py:15)."""

    def __init__(self):
        super().__init__(logging.INFO)
        self.lines = []

    def emit(self, record):
        self.lines.append(record.getMessage())


def digest(a):
    """sha256 of an array's bytes, as uint8 (pins regenerated inputs to the ones used here)."""
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), np.uint8)


def run_logged(ref, dirty, psf, kw):
    """DataImage.moresane of the reference with its INFO log captured; returns (img, lines, seconds)."""
    lg = logging.getLogger(ref.main.__name__)
    h = _InfoLines()
    lg.addHandler(h)
    old = lg.level
    lg.setLevel(logging.INFO)
    try:
        img = ref.main.DataImage(dirty, psf, None, 1.0, 1.0)
        t0 = time.perf_counter()
        img.moresane(subregion=dirty.shape[0], **kw)
        dt = time.perf_counter() - t0
    finally:
        lg.removeHandler(h)
        lg.setLevel(old)
    return img, h.lines, dt


def save_baseline(name, dirty, psf, kw, img, lines, dt, full_residual):
    """Sparse model, residual (whole or a 256^2 centre crop + std), log text and run time."""
    recs = parse_major_log(lines)
    flat = img.model.ravel()
    idx = np.flatnonzero(flat).astype(np.int64)
    n = dirty.shape[0]
    c = slice(n // 2 - 128, n // 2 + 128)
    # a model with more than a quarter of its pixels set is smaller stored whole
    model = dict(model=img.model) if 4 * idx.size > flat.size else dict(model_idx=idx, model_val=flat[idx])
    out = dict(dirty_sha=digest(dirty), psf_sha=digest(psf), **model,
               model_shape=np.array(img.model.shape), residual_std=np.array(np.std(img.residual)),
               residual_centre=img.residual[c, c], log=np.array(lines), seconds=np.array(dt),
               major=np.array(len(recs)), minor_total=np.array(sum(sum(r["minor"]) for r in recs)),
               major_loop_miter=np.array(kw["major_loop_miter"]))
    if full_residual:
        out["residual"] = img.residual
    print(name, "major", len(recs), "minor", int(out["minor_total"]), "seconds", round(dt, 1),
          "model nnz", idx.size, "residual std", float(out["residual_std"]))
    save(name, **out)


def gen_baseline_512(ref):
    """The 512^2 problem (1024^2 PSF, 3000 uv points) with its full run parameters, linear."""
    from pymoresane_gb300 import synthetic
    dirty, psf, _ = synthetic.make_problem(synthetic.problem_512(0))
    img, lines, dt = run_logged(ref, dirty, psf, dict(BASELINE_RUN))
    save_baseline("baseline_512", dirty, psf, BASELINE_RUN, img, lines, dt, full_residual=True)


def _gen_2048(ref, name, miter):
    from pymoresane_gb300 import synthetic
    dirty, psf, _ = synthetic.make_problem(synthetic.problem_2048(0))
    kw = dict(BASELINE_2048_RUN, major_loop_miter=miter)
    img, lines, dt = run_logged(ref, dirty, psf, kw)
    save_baseline(name, dirty, psf, kw, img, lines, dt, full_residual=False)


def gen_baseline_2048_m3(ref):
    """The 2048^2 problem (4096^2 PSF, 20000 uv points, S=7) bounded to 3 major iterations."""
    _gen_2048(ref, "baseline_2048_m3", 3)


def gen_baseline_2048_full(ref):
    """The same 2048^2 problem run to completion (hours on one core)."""
    _gen_2048(ref, "baseline_2048_full", BASELINE_2048_RUN["major_loop_miter"])


def gen_oracle_f64_2048_m3(ref):
    """The float64 oracle (oracle/moresane.py, precision='f64': the reference's float32
    casts removed) on the 2048^2 problem, three major iterations: the yardstick of
    the float32 versus float64-reduction error statement. Does not use `ref`."""
    from oracle.moresane import MoresaneOracle
    from pymoresane_gb300 import synthetic
    dirty, psf, _ = synthetic.make_problem(synthetic.problem_2048(0))
    kw = dict(BASELINE_2048_RUN, major_loop_miter=3)
    o = MoresaneOracle(dirty, psf, precision="f64")
    t0 = time.perf_counter()
    o.moresane(subregion=dirty.shape[0], **kw)
    dt = time.perf_counter() - t0
    flat = o.model.ravel()
    idx = np.flatnonzero(flat).astype(np.int64)
    n = dirty.shape[0]
    c = slice(n // 2 - 128, n // 2 + 128)
    recs = np.array([[r["max_scale"], r["scale_adjust"], r["minor"], int(r["reverted"])] for r in o.log], np.int64)
    print("oracle_f64_2048_m3 majors", len(o.log), "seconds", round(dt, 1), "nnz", idx.size)
    save("oracle_f64_2048_m3", dirty_sha=digest(dirty), psf_sha=digest(psf), model_idx=idx, model_val=flat[idx],
         model_shape=np.array(o.model.shape), residual_std=np.array(np.std(o.residual)),
         residual_rms=np.array(np.sqrt(np.mean(np.square(o.residual)))), residual_centre=o.residual[c, c],
         records=recs, seconds=np.array(dt))


GENERATORS = {"restore": gen_restore, "iuwt": gen_iuwt, "conv": gen_conv, "toolbox": gen_toolbox, "moresane": gen_moresane,
              "tart": gen_tart, "baseline_512": gen_baseline_512, "baseline_2048_m3": gen_baseline_2048_m3,
              "baseline_2048_full": gen_baseline_2048_full, "oracle_f64_2048_m3": gen_oracle_f64_2048_m3}
# slow: run only when named with --only
SLOW = {"baseline_512", "baseline_2048_m3", "baseline_2048_full", "oracle_f64_2048_m3"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", nargs="*", default=None)
    args = ap.parse_args()
    ref = refshim.load_reference()
    for name, fn in GENERATORS.items():
        if (args.only and name not in args.only) or (not args.only and name in SLOW):
            continue
        fn(ref)


if __name__ == "__main__":
    main()

"""Float32 versus float64-reduction error statement on the 2048^2 problem.

The yardstick is the float64 oracle (oracle/moresane.py with precision='f64',
the reference's float32 casts removed) run on the seeded 2048^2 problem
(4096^2 PSF, scale_count=7) for three major iterations; its result is the
fixture tests/golden/oracle_f64_2048_m3.npz (tests/golden/make_golden.py).

The GPU path runs three times on the same input: with the library's default
reductions (float64 accumulation of float32 partials), with float-float
accumulation within each CTA (msn_set_reduction_precision(48)) and with plain
float32 accumulation (msn_set_reduction_precision(32)). For each, the test states the
model error (max |model - oracle| / peak), the residual RMS error (relative)
and whether the per-major decisions match the oracle's; the wavelet
coefficients of the dirty image (GPU float32 decomposition against the float64
'ser' restatement) are stated once. Acceptance for the default path: model
within 1e-4 of the peak, residual RMS within 1e-4 relative, the same
decisions.
"""
import hashlib
import os
import sys

import numpy as np
import pytest

from pymoresane_gb300 import _native, synthetic
from pymoresane_gb300 import iuwt as G
from pymoresane_gb300.main import DataImage

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
sys.path.insert(0, GOLDEN)
import cases as mg  # noqa: E402

MODEL_TOL = 1e-4
RMS_TOL = 1e-4
NAMES = {64: "float64", 48: "float-float", 32: "float32"}


def oracle_fixture():
    path = os.path.join(GOLDEN, "oracle_f64_2048_m3.npz")
    if not os.path.exists(path):
        pytest.skip("oracle_f64_2048_m3.npz not generated")
    return np.load(path)


def run(dirty, psf, bits):
    _native.call("msn_set_reduction_precision", bits)
    try:
        img = DataImage(dirty, psf, None, 1.0, 1.0)
        img.moresane(subregion=dirty.shape[0], **dict(mg.BASELINE_2048_RUN, major_loop_miter=3))
    finally:
        _native.call("msn_set_reduction_precision", 64)
    return img


def test_float32_vs_float64_reductions_against_fp64_oracle(cuda):
    g = oracle_fixture()
    dirty, psf, _ = synthetic.make_problem(synthetic.problem_2048(0))
    digest = np.frombuffer(hashlib.sha256(dirty.tobytes()).digest(), np.uint8)
    assert np.array_equal(digest, g["dirty_sha"])
    ref_model = np.zeros(int(np.prod(g["model_shape"])), np.float64)
    ref_model[g["model_idx"]] = g["model_val"]
    ref_model = ref_model.reshape(tuple(g["model_shape"]))
    peak = float(np.max(np.abs(ref_model)))
    ref_rms = float(g["residual_rms"])
    ref_recs = [tuple(int(v) for v in r) for r in g["records"]]
    stats = {}
    for bits in (64, 48, 32):
        img = run(dirty, psf, bits)
        recs = [(r["max_scale"], r["scale_adjust"], r["minor"], int(r["reverted"])) for r in img.log]
        rms = float(np.sqrt(np.mean(np.square(img.residual.astype(np.float64)))))
        stats[bits] = dict(model=float(np.max(np.abs(img.model - ref_model))) / peak,
                           rms=abs(rms - ref_rms) / ref_rms, decisions=recs == ref_recs)
    # wavelet coefficients of the dirty image: GPU float32 against the float64 'ser' restatement
    from oracle import iuwt as OI
    w32 = G.iuwt_decomposition(dirty, 7, 0, mode="gpu")
    w64 = OI.decompose(dirty.astype(np.float64), 7, 0, arith="f64")
    coef = float(np.max(np.abs(w32 - w64))) / float(np.max(np.abs(w64)))
    print(f"\nerror vs float64 oracle (2048^2, 3 major iterations): wavelet coefficients {coef:.2e} of peak; "
          + "; ".join(f"{NAMES[b]} reductions: model {s['model']:.2e} of peak, "
                      f"residual RMS {s['rms']:.2e} relative, decisions {'identical' if s['decisions'] else 'differ'}"
                      for b, s in stats.items()))
    assert coef <= 2e-6
    s64 = stats[64]
    assert s64["decisions"] and s64["model"] <= MODEL_TOL and s64["rms"] <= RMS_TOL
    assert np.isfinite(stats[32]["model"]) and np.isfinite(stats[32]["rms"])
    assert stats[48]["decisions"] and stats[48]["model"] <= MODEL_TOL
    assert _native.query("msn_reduction_precision") == 64


def test_reduction_precision_setting(cuda):
    with pytest.raises(ValueError):
        _native.call("msn_set_reduction_precision", 16)
    _native.call("msn_set_reduction_precision", 48)
    assert _native.query("msn_reduction_precision") == 48
    _native.call("msn_set_reduction_precision", 64)
    assert _native.query("msn_reduction_precision") == 64


def test_float32_reductions_on_a_long_run(cuda):
    # the 512^2 problem run to completion (62 major iterations in the reference's own run,
    # tests/golden/baseline_512.npz): float32 accumulation against the float64 default, both
    # measured against the reference's result; stated, not bounded, for float32
    path = os.path.join(GOLDEN, "baseline_512.npz")
    if not os.path.exists(path):
        pytest.skip("baseline_512.npz not generated")
    g = np.load(path)
    dirty, psf, _ = synthetic.make_problem(synthetic.problem_512(0))
    ref = np.zeros(int(np.prod(g["model_shape"])), np.float32)
    ref[g["model_idx"]] = g["model_val"]
    ref = ref.reshape(tuple(g["model_shape"]))
    peak = float(np.max(np.abs(ref)))
    ref_majors = int(g["major"])
    out = {}
    for bits in (64, 48, 32):
        _native.call("msn_set_reduction_precision", bits)
        try:
            img = DataImage(dirty, psf, None, 1.0, 1.0)
            img.moresane(subregion=dirty.shape[0], **mg.BASELINE_RUN)
        finally:
            _native.call("msn_set_reduction_precision", 64)
        out[bits] = (float(np.max(np.abs(img.model - ref))) / peak, len(img.log),
                     sum(r["minor"] for r in img.log))
    print(f"\n512^2 run to completion against the reference ({ref_majors} major iterations): "
          + "; ".join(f"{NAMES[b]} reductions: model {e:.2e} of peak, {mj} major / "
                      f"{mn} minor iterations" for b, (e, mj, mn) in out.items()))
    assert out[64][0] <= 2e-4 and abs(out[64][1] - ref_majors) <= 1

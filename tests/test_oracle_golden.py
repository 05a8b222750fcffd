"""Pin the CPU oracle against golden outputs of the reference's own code.

The fixtures in tests/golden/*.npz were produced by tests/golden/make_golden.py,
which runs the reference PyMORESANE ('ser', 'mp', 'cpu' paths) on seeded
inputs. The oracle restatement must reproduce them.
"""
import os
import sys

import numpy as np
import pytest

from oracle import iuwt as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.mark.parametrize("adj", [0, 1, 2])
def test_iuwt_ser_bit_exact(adj):
    g = load("iuwt")
    d, c = O.decompose(g["x"], 4, adj, store_smoothed=True, arith="f64")
    assert np.array_equal(d, g[f"ser_detail_adj{adj}"])
    assert np.array_equal(c, g[f"ser_smoothed_adj{adj}"])
    r = O.recompose(d, adj, smoothed_array=c, arith="f64")
    assert np.array_equal(r, g[f"ser_recomp_smoothed_adj{adj}"])
    r0 = O.recompose(d, adj, arith="f64")
    assert np.array_equal(r0, g[f"ser_recomp_zero_adj{adj}"])


def test_iuwt_mp_strips_bit_exact():
    g = load("iuwt")
    d, c = O.decompose_strips(g["mp_x"], 3, 1, store_smoothed=True, workers=2)
    assert np.array_equal(d, g["mp_detail_adj1"].astype(np.float32))
    assert np.array_equal(c, g["mp_smoothed_adj1"])
    r = O.recompose_strips(d, 1, smoothed_array=c, workers=2)
    assert np.array_equal(r, g["mp_recomp_adj1"])


def test_iuwt_perfect_reconstruction_f64():
    g = load("iuwt")
    assert np.max(np.abs(g["ser_recomp_smoothed_adj0"] - g["x"])) < 1e-12


def test_f32_oracle_close_to_f64():
    g = load("iuwt")
    d32 = O.decompose(g["x"].astype(np.float32), 4, 0, arith="f32fma")
    d64 = g["ser_detail_adj0"]
    assert np.max(np.abs(d32 - d64)) < 1e-5 * np.max(np.abs(d64))


def test_fma32_correctly_rounded():
    from fractions import Fraction
    rng = np.random.default_rng(7)
    a = rng.standard_normal(3000).astype(np.float32)
    b = rng.standard_normal(3000).astype(np.float32)
    c = (rng.standard_normal(3000) * np.exp(rng.uniform(-20, 20, 3000))).astype(np.float32)
    r = O.fma32(a, b, c)
    for i in range(0, 3000, 7):
        exact = Fraction(float(a[i])) * Fraction(float(b[i])) + Fraction(float(c[i]))
        cands = [np.nextafter(r[i], np.float32(-np.inf)), r[i], np.nextafter(r[i], np.float32(np.inf))]
        errs = [abs(Fraction(float(v)) - exact) for v in cands]
        assert errs[1] <= min(errs)


def test_convolution_oracle_bit_exact():
    from oracle import convolution as C
    g = load("conv")
    assert np.array_equal(C.fft_convolve(g["x"], np.fft.rfft2(g["psf2"]), "linear"), g["linear"])
    assert np.array_equal(C.fft_convolve(g["x"], np.fft.rfft2(g["psf1"]), "circular"), g["circular"])
    assert np.array_equal(C.pad_array(g["x"]), g["pad"])


@pytest.mark.parametrize("ee,ie", [(0, 0), (3, 0), (0, 5), (4, 7), (0, 70)])
def test_estimate_threshold_bit_exact(ee, ie):
    from oracle import toolbox as T
    g = load("toolbox")
    assert np.array_equal(T.estimate_threshold(g["decomp"], ee, ie), g[f"thr_{ee}_{ie}"])


def test_apply_threshold_bit_exact():
    from oracle import toolbox as T
    g = load("toolbox")
    d = g["decomp"]
    got = T.apply_threshold(d, g["thr_0_0"], 4)
    assert np.array_equal(got.view(np.uint32), g["thresh"].view(np.uint32))   # signed zeros included
    assert np.array_equal(T.apply_threshold(d[1], g["thr_0_0"][1], 3), g["thresh_2d"])


@pytest.mark.parametrize("neg", [0, 1])
def test_source_extraction_bit_exact(neg):
    from oracle import toolbox as T
    g = load("toolbox")
    src, msk = T.source_extraction(g["thresh"][1:4], 0.75, bool(neg), semantics="cpu")
    assert src.dtype == np.float64 and msk.dtype == np.int32
    assert np.array_equal(src, g[f"src_neg{neg}"]) and np.array_equal(msk, g[f"mask_neg{neg}"])


def test_snr_ratio():
    from oracle import toolbox as T
    g = load("toolbox")
    assert T.snr_ratio(g["thresh"][1:4].astype(np.float64), g["decomp"][1:4]) == float(g["snr"])


@pytest.mark.parametrize("name", ["lin_double", "circ_pos", "lin_same_edge", "lin_subregion", "neg_excl"])
def test_moresane_oracle_bit_exact(name):
    """oracle/moresane.py (precision='ref') reproduces the reference's own runs bit for bit."""
    import sys
    sys.path.insert(0, GOLDEN)
    import cases as mg
    from oracle.moresane import MoresaneOracle
    g = load("moresane")
    kw = dict(mg.RUN_DEFAULTS, **mg.MORESANE_CASES[name][1])
    o = MoresaneOracle(g[f"{name}_dirty"], g[f"{name}_psf"], precision="ref")
    o.moresane(**kw)
    assert o.model.dtype == g[f"{name}_model"].dtype
    assert np.array_equal(o.model, g[f"{name}_model"])
    assert np.array_equal(o.residual, g[f"{name}_residual"])


@pytest.mark.parametrize("name,majors,minors", [("baseline_512", 62, None), ("baseline_2048_m3", 3, None),
                                                ("baseline_2048_full", 90, 1595)])
def test_baseline_fixtures_hold_the_reference_trajectory(name, majors, minors):
    # the reference's own runs of the benchmark problems: the parsed INFO log gives the major count
    # and the minor-iteration total stored beside it (bench.py scales its CPU baseline by the 2048^2
    # full run's); every minor loop of a major iteration is counted
    path = os.path.join(GOLDEN, name + ".npz")
    if not os.path.exists(path):
        pytest.skip(f"{name}.npz not generated")
    g = np.load(path)
    sys.path.insert(0, GOLDEN)
    import cases as mg
    recs = mg.parse_major_log([str(s) for s in g["log"]])
    assert len(recs) == int(g["major"]) == majors
    total = sum(sum(r["minor"]) for r in recs)
    assert total == int(g["minor_total"])
    if minors is not None:
        assert total == minors
    model = g["model"] if "model" in g else None
    if model is None:
        model = np.zeros(int(np.prod(g["model_shape"])), np.float32)
        model[g["model_idx"]] = g["model_val"]
    assert np.isfinite(model).all() and np.count_nonzero(model) > 0

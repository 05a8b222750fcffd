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
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import refshim  # noqa: E402


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


GENERATORS = {"iuwt": gen_iuwt, "conv": gen_conv, "toolbox": gen_toolbox}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", nargs="*", default=None)
    args = ap.parse_args()
    ref = refshim.load_reference()
    for name, fn in GENERATORS.items():
        if args.only and name not in args.only:
            continue
        fn(ref)


if __name__ == "__main__":
    main()

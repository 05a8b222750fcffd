"""Seeded MORESANE test cases shared by make_golden.py and the GPU tests.

Each case is (problem kwargs, run kwargs); the problem is a synthetic dirty
image / PSF pair (pymoresane_gb300.synthetic) and the run kwargs are passed
to DataImage.moresane together with RUN_DEFAULTS.
"""
import numpy as np

MORESANE_CASES = {
    # name: (problem kwargs, run kwargs)
    "lin_double": (dict(n=128, psf_factor=2, seed=31), dict(scale_count=4, conv_mode="linear")),
    "circ_pos": (dict(n=128, psf_factor=1, seed=32), dict(scale_count=4, conv_mode="circular",
                                                         enforce_positivity=True)),
    "lin_same_edge": (dict(n=128, psf_factor=1, seed=33), dict(scale_count=4, conv_mode="linear",
                                                              edge_suppression=True)),
    "lin_subregion": (dict(n=128, psf_factor=2, seed=34), dict(scale_count=4, conv_mode="linear", subregion=64)),
    "neg_excl": (dict(n=128, psf_factor=2, seed=35), dict(scale_count=5, conv_mode="linear", neg_comp=True,
                                                         edge_excl=6, int_excl=10, edge_offset=3)),
}
RUN_DEFAULTS = dict(sigma_level=4, loop_gain=0.2, tolerance=0.75, accuracy=1e-6, major_loop_miter=12,
                    minor_loop_miter=30)


def problem(n, psf_factor, seed):
    from pymoresane_gb300 import synthetic
    w = synthetic.Workload(n=n, psf_factor=psf_factor, n_uv=int(3000 * (n / 512) ** 2 * psf_factor ** 2 / 4) + 200,
                           n_points=10, n_gauss=2, sigma_range=(2.0, 5.0), noise=1e-3, seed=seed)
    return synthetic.make_problem(w)


def restore_inputs():
    """Seeded PSFs (3 sizes) and model / residual pairs of the restore fixtures (shared with the tests)."""
    from pymoresane_gb300.synthetic import make_psf
    psfs = {tag: make_psf(m, n_uv, np.random.default_rng(m)).astype(np.float32)
            for tag, m, n_uv in (("p256", 256, 400), ("p512", 512, 900), ("p1024", 1024, 2500))}
    rng = np.random.default_rng(7)
    cases = {}
    for tag, n, ptag in (("same", 256, "p256"), ("double", 256, "p512"), ("double512", 512, "p1024")):
        model = np.zeros((n, n), np.float32)
        idx = rng.integers(8, n - 8, (30, 2))
        model[idx[:, 0], idx[:, 1]] = rng.uniform(0.1, 2.0, 30).astype(np.float32)
        residual = (0.01 * rng.standard_normal((n, n))).astype(np.float32)
        cases[tag] = (ptag, model, residual)
    return psfs, cases


# Benchmark-size problems run end to end by the reference (make_golden.py
# gen_baseline_*): the 512^2 problem with its full run parameters, and the
# 2048^2 problem that bench.py times, bounded to a few major iterations and
# also run to completion.
BASELINE_RUN = dict(scale_count=5, sigma_level=4, loop_gain=0.2, tolerance=0.75, accuracy=1e-6,
                    major_loop_miter=100, minor_loop_miter=30, conv_mode="linear")
BASELINE_2048_RUN = dict(BASELINE_RUN, scale_count=7)


def parse_major_log(lines):
    """Per-major-iteration records from the INFO log lines of a MORESANE run.

    Works on the reference's log text (pymoresane/main.py:316-507) and on this
    package's identical text. Each record: the list of maximum scales and
    minor-loop counts of the minor loops run in that major iteration (more
    than one when the minimum scale is incremented), the last 'Scale k is
    empty' adjust, and whether the step was reverted.
    """
    recs, cur = [], None

    def fresh():
        return {"max_scale": [], "minor": [], "scale_adjust": [], "reverted": False}

    for ln in lines:
        if cur is None:
            cur = fresh()
        if ln.startswith("Maximum scale = "):
            cur["max_scale"].append(int(ln.split("=")[1]))
            cur["scale_adjust"].append(0)
        elif ln.startswith("Scale ") and " is empty." in ln:
            cur["scale_adjust"][-1] = int(ln.split()[1])
        elif ln.endswith("minor loop iterations performed."):
            cur["minor"].append(int(ln.split()[0]))
        elif ln.startswith("Residual has worsened"):
            cur["reverted"] = True
        elif ln.endswith("major loop iterations performed."):
            recs.append(cur)
            cur = None
    return recs

"""DataImage.restore on the GPU.

The restoring convolution is checked against the reference's restored images
with the reference's own clean beams (tolerance 1e-5 of the peak); the beam fit
itself is pinned on the host by tests/test_restore.py. End to end, restore()
is checked against the float64 oracle given the beam this host's scipy fits
(scipy versions may land a poorly constrained fit on slightly different
parameters).
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from cases import restore_inputs  # noqa: E402

pytestmark = pytest.mark.gpu
G = np.load(os.path.join(HERE, "golden", "restore.npz"))


def reference_beam(tag, shape):
    r0, r1, c0, c1 = G[f"{tag}_beam_box"]
    beam = np.zeros(shape, np.float32)
    beam[r0:r1, c0:c1] = G[f"{tag}_beam_crop"]
    return beam


@pytest.mark.parametrize("tag", ["same", "double", "double512"])
def test_restore_convolution_matches_reference(cuda, tag):
    from pymoresane_gb300.main import DataImage
    psfs, cases = restore_inputs()
    ptag, model, residual = cases[tag]
    img = DataImage(np.zeros_like(model), psfs[ptag], None, 0.5, 0.25)
    img.model, img.residual = model, residual
    got = img.restore_with(reference_beam(ptag, psfs[ptag].shape))
    want = G[f"{tag}_restored"]
    assert got.dtype == np.float32 and got.shape == want.shape
    assert np.max(np.abs(got - want)) <= 1e-5 * np.max(np.abs(want))


@pytest.mark.parametrize("tag,n,m", [("double512", 512, 1024), ("full", 1024, 2048)])
def test_restore_end_to_end_against_oracle(cuda, tag, n, m):
    from oracle import restore as OR
    from pymoresane_gb300.beam_fit import beam_fit
    from pymoresane_gb300.main import DataImage
    from pymoresane_gb300.synthetic import make_psf
    rng = np.random.default_rng(n)
    psf = make_psf(m, 2 * m, np.random.default_rng(m))
    model = np.zeros((n, n), np.float32)
    idx = rng.integers(16, n - 16, (100, 2))
    model[idx[:, 0], idx[:, 1]] = rng.uniform(0.01, 1.0, 100).astype(np.float32)
    residual = (1e-3 * rng.standard_normal((n, n))).astype(np.float32)
    img = DataImage(np.zeros_like(model), psf, None, 1.0, 1.0)
    img.model, img.residual = model, residual
    params = img.restore()
    beam, want_params = beam_fit(psf, 1.0, 1.0)
    assert np.allclose(params, want_params, rtol=1e-12, atol=0)
    want = OR.restore(model, residual, beam)
    assert np.max(np.abs(img.restored - want)) <= 1e-5 * np.max(np.abs(want))

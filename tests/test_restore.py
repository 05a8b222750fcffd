"""Restore step on the host: the beam fit and the oracle restore against the reference's own outputs."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from cases import restore_inputs  # noqa: E402
from oracle import restore as OR  # noqa: E402
from pymoresane_gb300.beam_fit import beam_fit  # noqa: E402

G = np.load(os.path.join(HERE, "golden", "restore.npz"))


def reference_beam(tag, shape):
    r0, r1, c0, c1 = G[f"{tag}_beam_box"]
    beam = np.zeros(shape, np.float32)
    beam[r0:r1, c0:c1] = G[f"{tag}_beam_crop"]
    return beam


@pytest.mark.parametrize("tag", ["p256", "p512", "p1024"])
def test_beam_fit_matches_reference(tag):
    # p256 pins the Python-2 window quirk (rows / columns 128..255 of a 256 x 256 PSF)
    psf = restore_inputs()[0][tag]
    beam, params = beam_fit(psf, 0.5, 0.25)
    assert beam.dtype == np.float32
    ref = reference_beam(tag, psf.shape)
    assert np.allclose(beam, ref, rtol=0, atol=1e-7)
    assert np.allclose(params, G[f"{tag}_params"], rtol=1e-9, atol=0)


@pytest.mark.parametrize("tag", ["same", "double", "double512"])
def test_oracle_restore_matches_reference(tag):
    psfs, cases = restore_inputs()
    ptag, model, residual = cases[tag]
    got = OR.restore(model, residual, reference_beam(ptag, psfs[ptag].shape))
    want = G[f"{tag}_restored"]
    assert got.dtype == np.float32
    assert np.max(np.abs(got - want)) <= 1e-5 * np.max(np.abs(want))

"""FITS reader / writer (host only) on the reference's TART fixture pair."""
import os

import numpy as np

from pymoresane_gb300 import fits

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_read_tart_fixture():
    data, hdr = fits.read(os.path.join(GOLDEN, "tart_dirty.fits"))
    assert data.shape == (256, 256) and data.dtype == np.float64
    assert hdr["BITPIX"] == -64 and hdr["CTYPE1"] == "RA---TAN" and hdr["CDELT1"] == 0.703125
    assert 1.5e-5 < data.min() < 1.6e-5 and 15.0 < data.max() < 15.1
    beam, _ = fits.read(os.path.join(GOLDEN, "tart_beam.fits"))
    assert np.unravel_index(np.argmax(beam), beam.shape) == (128, 128)


def test_write_roundtrip(tmp_path):
    data, hdr = fits.read(os.path.join(GOLDEN, "tart_dirty.fits"))
    out = tmp_path / "x.fits"
    fits.write(str(out), data.reshape(1, 1, 256, 256), hdr)
    back, h2 = fits.read(str(out))
    assert back.shape == (1, 1, 256, 256) and h2["NAXIS"] == 4 and h2["CTYPE2"] == "DEC--TAN"
    assert np.array_equal(back[0, 0], data.astype(np.float32))
    assert os.path.getsize(out) % 2880 == 0

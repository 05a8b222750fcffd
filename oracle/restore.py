"""Oracle for the restore step (test infrastructure only; never imported by the package).

Restates pymoresane/main.py:601-616 in float64 numpy: the model convolved with
the clean beam -- pad to the PSF's size, rfft2 product, irfft2, fftshift and a
centre crop for a double-size PSF (main.py:608-611), the plain circular product
for a same-size PSF (main.py:613) -- plus the residual, cast to float32. The
clean beam itself comes from the reference's beam_fit (beam_fit.py:6-69); its
pinned values are the golden fixture tests/golden/restore.npz.
"""
import numpy as np


def restore(model, residual, clean_beam):
    model = np.asarray(model, np.float64)
    beam = np.asarray(clean_beam, np.float64)
    n = model.shape[0]
    if beam.shape[0] == 2 * n:
        padded = np.zeros(beam.shape, np.float64)
        padded[n // 2:n // 2 + n, n // 2:n // 2 + n] = model
        full = np.fft.fftshift(np.fft.irfft2(np.fft.rfft2(padded) * np.fft.rfft2(beam), s=beam.shape))
        out = full[n // 2:-(n // 2), n // 2:-(n // 2)]
    else:
        out = np.fft.fftshift(np.fft.irfft2(np.fft.rfft2(model) * np.fft.rfft2(beam), s=beam.shape))
    return (out + np.asarray(residual, np.float64)).astype(np.float32)

"""Oracle: FFT convolution with a precomputed PSF spectrum.

Restates pymoresane/iuwt_convolution.py (CPU device):

* ``pad_array``     -- pymoresane/iuwt_convolution.py:142-158: zero-pad an
                       N x N image into the centre [N/2, 3N/2) of a 2N x 2N
                       float64 grid.
* ``fft_convolve``  -- pymoresane/iuwt_convolution.py:62-73:
      linear:   float32 C-contiguous
                crop_centre(fftshift(irfft2(H * rfft2(pad_array(x)))))
      circular: fftshift(irfft2(H * rfft2(x)))            (float64)
* ``psf_spectra``   -- the PSF-spectrum set-up of DataImage.moresane,
                       pymoresane/main.py:118-213 (CPU branches, 8 cases:
                       conv_mode x double-size PSF x full-image subregion),
                       returning (psf_subregion_fft, psf_data_fft,
                       psf_subregion, subregion_slice).
"""
import numpy as np


def pad_array(in1):
    n0, n1 = in1.shape
    out = np.zeros((2 * n0, 2 * n1))
    out[n0 // 2:3 * n0 // 2, n1 // 2:3 * n1 // 2] = in1
    return out


def fft_convolve(in1, in2, conv_mode="linear"):
    if conv_mode == "linear":
        full = np.fft.fftshift(np.fft.irfft2(in2 * np.fft.rfft2(pad_array(in1))))
        sl = tuple(slice(int(0.5 * sz), int(1.5 * sz)) for sz in in1.shape)
        return np.require(full[sl], np.float32, "C")
    if conv_mode == "circular":
        return np.fft.fftshift(np.fft.irfft2(in2 * np.fft.rfft2(in1)))
    raise ValueError(conv_mode)


def subregion_slice(shape, subregion):
    """Central subregion x subregion slice (pymoresane/main.py:121-122)."""
    return (slice(shape[0] // 2 - subregion // 2, shape[0] // 2 + subregion // 2),
            slice(shape[1] // 2 - subregion // 2, shape[1] // 2 + subregion // 2))


def psf_spectra(psf, dirty_shape, subregion, conv_mode):
    """(psf_subregion_fft, psf_data_fft, psf_subregion, subregion_slice) per main.py:118-213."""
    psf_shape = psf.shape
    sub_sl = subregion_slice(dirty_shape, subregion)
    double = all(p == 2 * d for p, d in zip(psf_shape, dirty_shape))
    if double:
        psf_sub = psf[psf_shape[0] // 2 - subregion // 2:psf_shape[0] // 2 + subregion // 2,
                      psf_shape[1] // 2 - subregion // 2:psf_shape[1] // 2 + subregion // 2]
    else:
        psf_sub = psf[sub_sl]
    full_image = all(d == subregion for d in dirty_shape)
    if conv_mode == "circular":
        if double:
            sub_fft = np.fft.rfft2(psf_sub)
            sl = (slice(psf_shape[0] // 2 - dirty_shape[0] // 2, psf_shape[0] // 2 + dirty_shape[0] // 2),
                  slice(psf_shape[1] // 2 - dirty_shape[1] // 2, psf_shape[1] // 2 + dirty_shape[1] // 2))
            data_fft = np.fft.rfft2(psf[sl])
        else:
            sub_fft = np.fft.rfft2(psf_sub)
            data_fft = sub_fft if psf_sub.shape == psf_shape else np.fft.rfft2(psf)
    elif conv_mode == "linear":
        if double:
            if full_image:
                sub_fft = np.fft.rfft2(psf)
                data_fft = sub_fft
            else:
                sl = (slice(psf_shape[0] // 2 - subregion, psf_shape[0] // 2 + subregion),
                      slice(psf_shape[1] // 2 - subregion, psf_shape[1] // 2 + subregion))
                sub_fft = np.fft.rfft2(psf[sl])
                data_fft = np.fft.rfft2(psf)
        else:
            if full_image:
                sub_fft = np.fft.rfft2(pad_array(psf))
                data_fft = sub_fft
            else:
                sl = (slice(psf_shape[0] // 2 - subregion, psf_shape[0] // 2 + subregion),
                      slice(psf_shape[1] // 2 - subregion, psf_shape[1] // 2 + subregion))
                sub_fft = np.fft.rfft2(psf[sl])
                data_fft = np.fft.rfft2(pad_array(psf))
    else:
        raise ValueError(conv_mode)
    return sub_fft, data_fft, psf_sub, sub_sl

"""Drop-in for pymoresane.iuwt_convolution (conv_device='gpu').

Signatures follow pymoresane/iuwt_convolution.py. The FFTs are libmsn's own
shared-memory Stockham kernels (no cuFFT); fft_convolve runs as three fused
kernels (row R2C, column FFT x PSF spectrum x inverse column FFT, row C2R
with the 1/M^2 scale, fft-shift and centre crop folded in).

``in2`` of fft_convolve may be the PsfSpectrum returned by
``psf_spectrum`` (no conversion) or a standard rfft2 spectrum [M, M/2+1]
(CUDA tensor or numpy array, e.g. from gpu_r2c_fft), which is converted to the
packed layout on every call.

Differences from the reference: only
conv_device='gpu' is implemented; pad_array stays a host (numpy) helper as
in the reference; device arrays are torch CUDA tensors.
"""
import numpy as np
import torch

from . import device as dev


def _check_device(conv_device):
    if conv_device != "gpu":
        raise ValueError(f"fft_convolve: conv_device={conv_device!r} is not available in pymoresane_gb300, which "
                         f"implements the GPU path only (use conv_device='gpu')")


def _host(t):
    return t.detach().cpu().numpy()


def fft_convolve(in1, in2, conv_device="gpu", conv_mode="linear", store_on_gpu=False):
    """Convolution of in1 with the PSF whose rfft2 spectrum is in2.

    Reference: pymoresane/iuwt_convolution.py:18-61 (gpu branch). Returns a
    float32 array (host) or a CUDA tensor when store_on_gpu.
    """
    _check_device(conv_device)
    if conv_mode not in ("linear", "circular"):
        raise ValueError(f"fft_convolve: unknown conv_mode {conv_mode!r}")
    out = dev.fft_convolve(in1, in2, linear=(conv_mode == "linear"))
    return out if store_on_gpu else _host(out)


def psf_spectrum(psf, m=None):
    """Packed device spectrum of ``psf`` zero-padded (centred) to an m x m grid."""
    return dev.psf_spectrum(psf, m)


def gpu_r2c_fft(in1, is_gpuarray=False, store_on_gpu=False):
    """rfft2 of a square real array; reference pymoresane/iuwt_convolution.py:76-106."""
    out = dev.rfft2(in1)
    return out if store_on_gpu else _host(out)


def gpu_c2r_ifft(in1, is_gpuarray=False, store_on_gpu=False):
    """irfft2 (divided by rows*cols); reference pymoresane/iuwt_convolution.py:108-139."""
    out = dev.irfft2(in1)
    return out if store_on_gpu else _host(out)


def pad_array(in1):
    """Zero-pad into the centre of a 2x grid (host float64), pymoresane/iuwt_convolution.py:142-158."""
    in1 = np.asarray(in1)
    n0, n1 = in1.shape
    out = np.zeros((2 * n0, 2 * n1))
    out[n0 // 2:3 * n0 // 2, n1 // 2:3 * n1 // 2] = in1
    return out


def fft_shift(in1):
    """In-place quadrant swap of a square device array; pymoresane/iuwt_convolution.py:161-201."""
    return dev.fft_shift_(in1)


def contiguous_slice(in1):
    """Centre crop [m/4, 3m/4)^2 of a device array; pymoresane/iuwt_convolution.py:204-239."""
    return dev.crop_centre(in1)


def scale_fft(in1):
    """In-place division by the element count; pymoresane/iuwt_convolution.py:242-265."""
    if not isinstance(in1, torch.Tensor) or not in1.is_cuda:
        raise TypeError("scale_fft operates in place on a CUDA tensor")
    dev.scale_(in1, in1.shape[0] * in1.shape[1])

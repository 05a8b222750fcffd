"""GPU parity of libmsn's hand-written FFTs and the fused PSF convolution.

Reference numbers: numpy's pocketfft (float64) and the oracle restatement of
pymoresane/iuwt_convolution.py. Tolerances (float32 FFTs): spectra within
2e-6 * sum|x| per bin; convolutions within 1e-5 of the output's peak.
"""
import os

import numpy as np
import pytest
import torch

from oracle import convolution as OC
from pymoresane_gb300 import device as dev
from pymoresane_gb300 import iuwt_convolution as G
from pymoresane_gb300.synthetic import make_psf

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CONV_TOL = 1e-5   # max abs error / max |reference output|

SIZES = [32, 64, 96, 128, 192, 256, 384, 512, 768, 1024, 1536, 2048, 3072, 4096, 6144, 8192]


@pytest.mark.parametrize("m", SIZES)
def test_rfft2_matches_numpy(cuda, m):
    rng = np.random.default_rng(m)
    x = rng.standard_normal((m, m)).astype(np.float32)
    got = G.gpu_r2c_fft(x)
    ref = np.fft.rfft2(x.astype(np.float64))
    assert got.dtype == np.complex64 and got.shape == ref.shape
    err = np.max(np.abs(got - ref))
    assert err <= 2e-6 * np.sum(np.abs(x)) / np.sqrt(m), err


@pytest.mark.parametrize("m", [32, 96, 256, 1536, 4096, 8192])
def test_irfft2_matches_numpy(cuda, m):
    rng = np.random.default_rng(m + 1)
    x = rng.standard_normal((m, m))
    spec = np.fft.rfft2(x)
    got = G.gpu_c2r_ifft(spec.astype(np.complex64))
    ref = np.fft.irfft2(spec)
    assert got.dtype == np.float32 and got.shape == (m, m)
    assert np.max(np.abs(got - ref)) <= 1e-5 * np.max(np.abs(ref))


@pytest.mark.parametrize("n,mode", [(32, "linear"), (64, "linear"), (96, "linear"), (128, "circular"),
                                    (256, "linear"), (256, "circular"), (768, "linear"), (1536, "circular")])
def test_fft_convolve_matches_oracle(cuda, n, mode):
    rng = np.random.default_rng(n)
    x = rng.standard_normal((n, n)).astype(np.float32)
    m = 2 * n if mode == "linear" else n
    psf = make_psf(m, max(50, m), rng)
    spec = np.fft.rfft2(psf.astype(np.float64))
    ref = OC.fft_convolve(x.astype(np.float64), spec, mode)
    packed = dev.psf_spectrum(psf)          # library packed layout
    got = G.fft_convolve(x, packed, "gpu", mode)
    got_std = G.fft_convolve(x, spec.astype(np.complex64), "gpu", mode)   # standard-layout spectrum
    scale = np.max(np.abs(ref))
    assert got.dtype == np.float32 and got.shape == (n, n)
    assert np.max(np.abs(got - ref)) <= CONV_TOL * scale
    assert np.max(np.abs(got_std - ref)) <= CONV_TOL * scale


def test_fft_convolve_golden(cuda):
    g = np.load(os.path.join(GOLDEN, "conv.npz"))
    lin = G.fft_convolve(g["x"], np.fft.rfft2(g["psf2"]), "gpu", "linear")
    assert np.max(np.abs(lin - g["linear"])) <= CONV_TOL * np.max(np.abs(g["linear"]))
    circ = G.fft_convolve(g["x"], np.fft.rfft2(g["psf1"]), "gpu", "circular")
    assert np.max(np.abs(circ - g["circular"])) <= CONV_TOL * np.max(np.abs(g["circular"]))


def test_psf_spectrum_offsets_match_pad_array(cuda):
    # rfft2(pad_array(psf)) -- the same-size-PSF linear branch of main.py:203-206.
    rng = np.random.default_rng(3)
    psf = make_psf(64, 100, rng)
    ref = np.fft.rfft2(OC.pad_array(psf))
    spec = dev.psf_spectrum(psf, m=128)
    x = rng.standard_normal((64, 64)).astype(np.float32)
    got = dev.fft_convolve(x, spec, linear=True).cpu().numpy()
    want = OC.fft_convolve(x.astype(np.float64), ref, "linear")
    assert np.max(np.abs(got - want)) <= CONV_TOL * np.max(np.abs(want))


def test_shift_crop_scale(cuda):
    rng = np.random.default_rng(4)
    a = rng.standard_normal((64, 64)).astype(np.float32)
    t = torch.from_numpy(a).cuda()
    G.fft_shift(t)
    assert np.array_equal(t.cpu().numpy(), np.fft.fftshift(a))
    c = G.contiguous_slice(torch.from_numpy(a).cuda())
    assert np.array_equal(c.cpu().numpy(), a[16:48, 16:48])
    s = torch.from_numpy(a).cuda()
    G.scale_fft(s)
    assert np.array_equal(s.cpu().numpy(), a / np.float32(64 * 64))


def test_invalid_sizes(cuda):
    with pytest.raises(ValueError):
        G.gpu_r2c_fft(np.zeros((40, 40), np.float32))          # 40 = 5 * 8 unsupported
    with pytest.raises(ValueError):
        G.fft_convolve(np.zeros((64, 64), np.float32), dev.psf_spectrum(np.zeros((64, 64), np.float32)),
                       "gpu", "linear")                          # linear needs m == 2n
    with pytest.raises(ValueError):
        G.fft_convolve(np.zeros((64, 64), np.float32), None, "cpu", "linear")


def test_full_size_convolution_2048_linear(cuda):
    # 2048^2 image, 4096^2 PSF: the single-image MORESANE configuration.
    rng = np.random.default_rng(2048)
    psf = make_psf(4096, 20000, rng)
    x = np.zeros((2048, 2048), np.float32)
    idx = rng.integers(0, 2048, (200, 2))
    x[idx[:, 0], idx[:, 1]] = rng.uniform(0.01, 1.0, 200).astype(np.float32)
    ref = OC.fft_convolve(x.astype(np.float64), np.fft.rfft2(psf.astype(np.float64)), "linear")
    got = G.fft_convolve(x, dev.psf_spectrum(psf), "gpu", "linear")
    assert np.max(np.abs(got - ref)) <= CONV_TOL * np.max(np.abs(ref))
    # linearity: conv(a + b) == conv(a) + conv(b)
    y = rng.standard_normal((2048, 2048)).astype(np.float32)
    spec = dev.psf_spectrum(psf)
    s = dev.fft_convolve(torch.from_numpy(x + y).cuda(), spec)
    a = dev.fft_convolve(torch.from_numpy(x).cuda(), spec) + dev.fft_convolve(torch.from_numpy(y).cuda(), spec)
    assert torch.max(torch.abs(s - a)).item() <= 1e-5 * torch.max(torch.abs(s)).item()
    # the persistent kernels' bounded waits never gave up
    import ctypes
    from pymoresane_gb300 import _native
    status = ctypes.c_uint(99)
    _native.call("msn_fft_status", ctypes.byref(status))
    assert status.value == 0


def test_full_size_convolution_2048_dense_random(cuda):
    # dense random image and PSF through the four-step 4096-point path, against float64 numpy
    rng = np.random.default_rng(4096)
    psf = rng.random((4096, 4096)).astype(np.float32)
    x = rng.standard_normal((2048, 2048)).astype(np.float32)
    ref = OC.fft_convolve(x.astype(np.float64), np.fft.rfft2(psf.astype(np.float64)), "linear")
    got = G.fft_convolve(x, dev.psf_spectrum(psf), "gpu", "linear")
    assert np.max(np.abs(got - ref)) <= CONV_TOL * np.max(np.abs(ref))


def test_unaligned_pointers_take_the_stockham_path(cuda):
    # the four-step kernels' bulk copies need 16-byte aligned addresses; an image, output or
    # spectrum that is only 8-byte aligned is convolved by the Stockham kernels instead
    from pymoresane_gb300 import _native
    rng = np.random.default_rng(77)
    x = rng.standard_normal((2048, 2048)).astype(np.float32)
    spec = dev.psf_spectrum(make_psf(4096, 3000, rng))
    ref = dev.fft_convolve(torch.from_numpy(x).cuda(), spec)
    base = torch.empty(2048 * 2048 + 4, dtype=torch.float32, device="cuda")
    xu = base[2:2 + 2048 * 2048]                         # 8 bytes past a 16-byte boundary
    xu.copy_(torch.from_numpy(x).cuda().reshape(-1))
    assert xu.data_ptr() % 16 == 8
    obase = torch.empty(2048 * 2048 + 4, dtype=torch.float32, device="cuda")
    ou = obase[2:2 + 2048 * 2048]
    work = dev.fft_workspace(2048, 4096, xu.device)
    _native.call("msn_fft_convolve", xu.data_ptr(), 2048, 4096, spec.packed.data_ptr(), ou.data_ptr(), 1,
                 work.data_ptr(), work.numel(), dev.stream_handle())
    got = ou.reshape(2048, 2048)
    assert torch.max(torch.abs(got - ref)).item() <= 1e-5 * torch.max(torch.abs(ref)).item()


@pytest.mark.parametrize("n", [2048, 512])
def test_row_flags_give_the_dense_result(cuda, n):
    # an image that is zero outside bands of rows, convolved with the flags of its possibly
    # non-zero rows: the same result as the dense convolution (the 2048^2 linear case skips the
    # row transforms of pairs of zero rows; other sizes ignore the flags). Flag patterns: bands
    # with odd edges (pairs with one live row), everything, nothing, a single row
    rng = np.random.default_rng(n)
    spec = dev.psf_spectrum(make_psf(2 * n, 2000, rng))
    patterns = []
    rows = np.zeros(n, np.uint8)
    rows[n // 16 + 1:n // 8] = 1
    rows[n // 2:n // 2 + n // 5 + 1] = 1
    rows[n - 3:] = 1
    patterns.append(rows)
    patterns.append(np.ones(n, np.uint8))
    patterns.append(np.zeros(n, np.uint8))
    one = np.zeros(n, np.uint8)
    one[n // 3] = 1
    patterns.append(one)
    work = dev.fft_workspace(n, 2 * n, torch.device("cuda"))
    for flags in patterns:
        x = rng.standard_normal((n, n)).astype(np.float32) * flags[:, None].astype(np.float32)
        xd = torch.from_numpy(x).cuda()
        dense = dev.fft_convolve(xd, spec, work=work).clone()
        # stale values in the workspace must not leak into skipped rows
        work.fill_(7)
        got = dev.fft_convolve(xd, spec, work=work, rows=torch.from_numpy(flags).cuda())
        assert torch.equal(got, dense), int(flags.sum())
    with pytest.raises(ValueError):
        dev.fft_convolve(xd, spec, rows=torch.zeros(n, dtype=torch.int32, device="cuda"))

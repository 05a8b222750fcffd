"""Tensor-level entry points: torch CUDA tensors in, torch CUDA tensors out.

PyTorch provides device memory and the current stream only; all arithmetic is
done by libmsn's CUDA kernels through the C ABI (include/msn.h). Every
function requires float32 CUDA tensors and raises if CUDA or the library is
unavailable -- there is no CPU path.
"""
import torch

from . import _native


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("pymoresane_gb300 requires a CUDA device (no CPU fallback)")


def stream_handle(stream=None):
    s = torch.cuda.current_stream() if stream is None else stream
    return s.cuda_stream


def as_f32_cuda(x, device=None):
    """Return a contiguous float32 CUDA tensor holding ``x`` (numpy or torch)."""
    require_cuda()
    if isinstance(x, torch.Tensor):
        t = x
        if not t.is_cuda:
            t = t.to(device or "cuda", non_blocking=False)
    else:
        t = torch.as_tensor(x).to(device or "cuda")
    if t.dtype != torch.float32:
        t = t.to(torch.float32)
    if not t.is_contiguous() or t.data_ptr() % 16:
        t = t.contiguous().clone() if t.data_ptr() % 16 else t.contiguous()
    return t


def _ptr(t):
    return None if t is None else t.data_ptr()


def iuwt_workspace(ny, nx, device):
    nbytes = _native.query("msn_iuwt_workspace_bytes", ny, nx)
    return torch.empty(max(nbytes, 16), dtype=torch.uint8, device=device)


def iuwt_decompose(x, scale_count, scale_adjust=0, store_smoothed=False, out=None, smoothed_out=None,
                   work=None):
    """Detail stack [scale_count - scale_adjust, ny, nx] and (optionally) the smoothest plane."""
    x = as_f32_cuda(x)
    if x.dim() != 2:
        raise ValueError("iuwt_decompose expects a 2-D image")
    ny, nx = x.shape
    planes = scale_count - scale_adjust
    if out is None:
        out = torch.empty((max(planes, 0), ny, nx), dtype=torch.float32, device=x.device)
    sm = None
    if store_smoothed:
        sm = smoothed_out if smoothed_out is not None else torch.empty((ny, nx), dtype=torch.float32,
                                                                       device=x.device)
    if work is None:
        work = iuwt_workspace(ny, nx, x.device)
    _native.call("msn_iuwt_decompose", x.data_ptr(), out.data_ptr() if planes > 0 else None, _ptr(sm), ny, nx,
                 scale_count, scale_adjust, work.data_ptr(), work.numel(), stream_handle())
    return out, sm


def iuwt_recompose(w, scale_adjust=0, smoothed=None, out=None, work=None):
    """Inverse transform of a detail stack [planes, ny, nx] (+ optional smoothest plane)."""
    w = as_f32_cuda(w)
    if w.dim() != 3:
        raise ValueError("iuwt_recompose expects a 3-D coefficient stack")
    planes, ny, nx = w.shape
    if smoothed is not None:
        smoothed = as_f32_cuda(smoothed, device=w.device)
        if tuple(smoothed.shape) != (ny, nx):
            raise ValueError("smoothed_array shape does not match the coefficient planes")
    if out is None:
        out = torch.empty((ny, nx), dtype=torch.float32, device=w.device)
    if work is None:
        work = iuwt_workspace(ny, nx, w.device)
    _native.call("msn_iuwt_recompose", w.data_ptr() if planes > 0 else None, planes, _ptr(smoothed),
                 out.data_ptr(), ny, nx, scale_adjust, work.data_ptr(), work.numel(), stream_handle())
    return out


# ---------------------------------------------------------------------------
# FFTs and the PSF convolution
# ---------------------------------------------------------------------------

def fft_workspace(n, m, device):
    nbytes = _native.query("msn_fft_workspace_bytes", n, m)
    if nbytes == 0:
        raise ValueError(f"unsupported FFT size m={m} (need 2^a in [32, 8192] or 3*2^a in [24, 6144])")
    return torch.empty(nbytes, dtype=torch.uint8, device=device)


class PsfSpectrum:
    """rfft2 of a PSF on an m x m grid, held on the device in libmsn's packed layout."""

    def __init__(self, packed, m):
        self.packed = packed
        self.m = m

    @property
    def device(self):
        return self.packed.device


def psf_spectrum(psf, m=None, off_r=None, off_c=None, work=None):
    """Packed spectrum of ``psf`` placed at (off_r, off_c) (default: centred) in an m x m zero grid."""
    psf = as_f32_cuda(psf)
    rows, cols = psf.shape
    m = rows if m is None else int(m)
    off_r = (m - rows) // 2 if off_r is None else int(off_r)
    off_c = (m - cols) // 2 if off_c is None else int(off_c)
    elems = _native.query("msn_spectrum_elems", m)
    if elems == 0:
        raise ValueError(f"unsupported FFT size m={m}")
    packed = torch.empty(elems, dtype=torch.complex64, device=psf.device)
    if work is None:
        work = fft_workspace(m, m, psf.device)
    _native.call("msn_psf_spectrum", psf.data_ptr(), rows, cols, m, off_r, off_c, packed.data_ptr(),
                 work.data_ptr(), work.numel(), stream_handle())
    return PsfSpectrum(packed, m)


def pack_spectrum(spec):
    """Convert a standard rfft2 spectrum [m, m/2+1] (torch or numpy) into a PsfSpectrum."""
    require_cuda()
    if isinstance(spec, PsfSpectrum):
        return spec
    t = spec if isinstance(spec, torch.Tensor) else torch.as_tensor(spec)
    t = t.to(device="cuda", dtype=torch.complex64).contiguous()
    if t.dim() != 2 or t.shape[1] != t.shape[0] // 2 + 1:
        raise ValueError("a PSF spectrum must have shape [m, m/2 + 1]")
    m = t.shape[0]
    elems = _native.query("msn_spectrum_elems", m)
    if elems == 0:
        raise ValueError(f"unsupported FFT size m={m}")
    packed = torch.empty(elems, dtype=torch.complex64, device=t.device)
    _native.call("msn_spectrum_pack", t.data_ptr(), m, packed.data_ptr(), stream_handle())
    return PsfSpectrum(packed, m)


def fft_convolve(x, spec, linear=True, out=None, work=None):
    """Convolution of the n x n image ``x`` with the PSF of ``spec`` (linear: m == 2n, circular: m == n)."""
    x = as_f32_cuda(x)
    spec = pack_spectrum(spec)
    n = x.shape[0]
    if x.dim() != 2 or x.shape[1] != n:
        raise ValueError("fft_convolve expects a square image")
    if out is None:
        out = torch.empty((n, n), dtype=torch.float32, device=x.device)
    if work is None:
        work = fft_workspace(n, spec.m, x.device)
    _native.call("msn_fft_convolve", x.data_ptr(), n, spec.m, spec.packed.data_ptr(), out.data_ptr(),
                 1 if linear else 0, work.data_ptr(), work.numel(), stream_handle())
    return out


def rfft2(x, work=None):
    x = as_f32_cuda(x)
    m = x.shape[0]
    if x.dim() != 2 or x.shape[1] != m:
        raise ValueError("rfft2 expects a square image")
    out = torch.empty((m, m // 2 + 1), dtype=torch.complex64, device=x.device)
    if work is None:
        work = fft_workspace(m, m, x.device)
    _native.call("msn_rfft2", x.data_ptr(), m, out.data_ptr(), work.data_ptr(), work.numel(), stream_handle())
    return out


def irfft2(spec, work=None):
    require_cuda()
    t = spec if isinstance(spec, torch.Tensor) else torch.as_tensor(spec)
    t = t.to(device="cuda", dtype=torch.complex64).contiguous()
    m = t.shape[0]
    if t.dim() != 2 or t.shape[1] != m // 2 + 1:
        raise ValueError("irfft2 expects a spectrum of shape [m, m/2 + 1]")
    out = torch.empty((m, m), dtype=torch.float32, device=t.device)
    if work is None:
        work = fft_workspace(m, m, t.device)
    _native.call("msn_irfft2", t.data_ptr(), m, out.data_ptr(), work.data_ptr(), work.numel(), stream_handle())
    return out


def fft_shift_(x):
    x = as_f32_cuda(x)
    _native.call("msn_fft_shift", x.data_ptr(), x.shape[0], stream_handle())
    return x


def crop_centre(x):
    x = as_f32_cuda(x)
    m = x.shape[0]
    out = torch.empty((m // 2, m // 2), dtype=torch.float32, device=x.device)
    _native.call("msn_crop_centre", x.data_ptr(), m, out.data_ptr(), stream_handle())
    return out


def scale_(x, divisor):
    x = as_f32_cuda(x)
    _native.call("msn_scale", x.data_ptr(), x.numel(), float(divisor), stream_handle())
    return x

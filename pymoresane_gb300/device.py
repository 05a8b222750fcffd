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


def iuwt_decompose_masked(x, mask, scale_count, scale_adjust=0, out=None, work=None):
    """mask * detail stack, the mask applied inside the detail pass."""
    x = as_f32_cuda(x)
    ny, nx = x.shape
    planes = scale_count - scale_adjust
    if out is None:
        out = torch.empty((max(planes, 0), ny, nx), dtype=torch.float32, device=x.device)
    if work is None:
        work = iuwt_workspace(ny, nx, x.device)
    _native.call("msn_iuwt_decompose_masked", x.data_ptr(), mask.data_ptr(), out.data_ptr() if planes > 0 else None,
                 ny, nx, scale_count, scale_adjust, work.data_ptr(), work.numel(), stream_handle())
    return out


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


def fft_convolve(x, spec, linear=True, out=None, work=None, rows=None):
    """Convolution of the n x n image ``x`` with the PSF of ``spec`` (linear: m == 2n, circular: m == n).

    ``rows`` (optional, n uint8 on the device): non-zero where row r of ``x`` may be
    non-zero; rows flagged zero must hold zeros (msn_fft_convolve_rows).
    """
    x = as_f32_cuda(x)
    spec = pack_spectrum(spec)
    n = x.shape[0]
    if x.dim() != 2 or x.shape[1] != n:
        raise ValueError("fft_convolve expects a square image")
    if out is None:
        out = torch.empty((n, n), dtype=torch.float32, device=x.device)
    if work is None:
        work = fft_workspace(n, spec.m, x.device)
    if rows is None:
        _native.call("msn_fft_convolve", x.data_ptr(), n, spec.m, spec.packed.data_ptr(), out.data_ptr(),
                     1 if linear else 0, work.data_ptr(), work.numel(), stream_handle())
    else:
        if rows.dtype != torch.uint8 or rows.numel() < n or not rows.is_cuda:
            raise ValueError("fft_convolve: rows must be n uint8 flags on the device")
        _native.call("msn_fft_convolve_rows", x.data_ptr(), n, spec.m, spec.packed.data_ptr(), out.data_ptr(),
                     1 if linear else 0, rows.data_ptr(), work.data_ptr(), work.numel(), stream_handle())
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


# ---------------------------------------------------------------------------
# Noise estimate, thresholding, labelling, extraction
# ---------------------------------------------------------------------------

def toolbox_workspace(planes, ny, nx, device):
    nbytes = _native.query("msn_toolbox_workspace_bytes", planes, ny, nx)
    return torch.empty(max(nbytes, 16), dtype=torch.uint8, device=device)


def noise_rects(ny, nx, edge_excl=0, int_excl=0):
    """Pixel set of estimate_threshold as include / exclude rectangles.

    Follows pymoresane/iuwt_toolbox.py:26-43 with Python slice semantics:
    include [e:-e, e:-e] when edge_excl != 0 (else everything), exclude
    [mid-i:mid+i, mid-i:mid+i] with mid = nx // 2 on both axes when int_excl != 0.
    """
    y0, y1, x0, x1 = 0, ny, 0, nx
    ey0 = ey1 = ex0 = ex1 = 0
    if edge_excl != 0:
        y0, y1 = slice(edge_excl, -edge_excl).indices(ny)[:2]
        x0, x1 = slice(edge_excl, -edge_excl).indices(nx)[:2]
    if int_excl != 0:
        mid = nx // 2
        ey0, ey1 = slice(mid - int_excl, mid + int_excl).indices(ny)[:2]
        ex0, ex1 = slice(mid - int_excl, mid + int_excl).indices(nx)[:2]
    return (y0, y1, x0, x1, ey0, ey1, ex0, ex1)


def mad_sigma(w, edge_excl=0, int_excl=0, out=None, work=None):
    """Per-plane MAD noise estimate (float64 device tensor [planes])."""
    import ctypes
    w = as_f32_cuda(w)
    if w.dim() == 2:
        w = w.unsqueeze(0)
    planes, ny, nx = w.shape
    rects = (ctypes.c_int * 8)(*noise_rects(ny, nx, edge_excl, int_excl))
    if out is None:
        out = torch.empty(planes, dtype=torch.float64, device=w.device)
    if work is None:
        work = toolbox_workspace(planes, ny, nx, w.device)
    _native.call("msn_mad_sigma", w.data_ptr(), planes, ny, nx, rects, out.data_ptr(), work.data_ptr(),
                 work.numel(), stream_handle())
    return out


def apply_threshold(w, sigma, sigma_level=4, supp_rects=None, out=None, want_max=False, work=None):
    """w * (|w| > sigma_level * sigma) per plane (+ optional suppression rectangles and plane maxima)."""
    w = as_f32_cuda(w)
    squeeze = w.dim() == 2
    if squeeze:
        w = w.unsqueeze(0)
    planes, ny, nx = w.shape
    if not isinstance(sigma, torch.Tensor) or sigma.dtype != torch.float64 or not sigma.is_cuda:
        sigma = torch.as_tensor(sigma, dtype=torch.float64).reshape(-1).to(w.device)
    if sigma.numel() == 1 and planes > 1:
        sigma = sigma.expand(planes).contiguous()
    if out is None:
        out = torch.empty_like(w)
    pmax = torch.empty(planes, dtype=torch.float32, device=w.device) if want_max else None
    if work is None and want_max:
        work = torch.empty(max(16, 4 * planes), dtype=torch.uint8, device=w.device)
    _native.call("msn_apply_threshold", w.data_ptr(), planes, ny, nx, sigma.data_ptr(), float(sigma_level),
                 _ptr(supp_rects), out.data_ptr(), _ptr(pmax), _ptr(work), 0 if work is None else work.numel(),
                 stream_handle())
    if squeeze:
        out = out[0]
    return (out, pmax) if want_max else out


def source_extraction(w, tolerance, neg_comp=False, mask=None, extracted=None, work=None):
    """Kept-island mask (float32 0/1) and mask * w for a coefficient stack."""
    w = as_f32_cuda(w)
    planes, ny, nx = w.shape
    if mask is None:
        mask = torch.empty_like(w)
    if extracted is None:
        extracted = torch.empty_like(w)
    if work is None:
        work = toolbox_workspace(planes, ny, nx, w.device)
    _native.call("msn_source_extraction", w.data_ptr(), planes, ny, nx, float(tolerance), 1 if neg_comp else 0,
                 mask.data_ptr(), extracted.data_ptr(), work.data_ptr(), work.numel(), stream_handle())
    return mask, extracted


def label(img, work=None):
    """scipy.ndimage.label-compatible 8-connected labelling of img != 0: (int32 labels, count)."""
    img = as_f32_cuda(img)
    ny, nx = img.shape
    labels = torch.empty((ny, nx), dtype=torch.int32, device=img.device)
    count = torch.zeros(1, dtype=torch.int32, device=img.device)
    if work is None:
        work = toolbox_workspace(1, ny, nx, img.device)
    _native.call("msn_label", img.data_ptr(), ny, nx, labels.data_ptr(), count.data_ptr(), work.data_ptr(),
                 work.numel(), stream_handle())
    return labels, int(count.item())


# ---------------------------------------------------------------------------
# Reductions and CG vector work
# ---------------------------------------------------------------------------

def reduce_workspace(device):
    """Reduction scratch, zeroed once (its completion counter must start at zero)."""
    return torch.zeros(_native.query("msn_reduce_workspace_bytes"), dtype=torch.uint8, device=device)


def dot2(a, b, c=None, d=None, out=None, work=None):
    out = torch.empty(2, dtype=torch.float64, device=a.device) if out is None else out
    work = reduce_workspace(a.device) if work is None else work
    _native.call("msn_dot2", a.data_ptr(), b.data_ptr(), _ptr(c), _ptr(d), a.numel(), out.data_ptr(),
                 work.data_ptr(), work.numel(), stream_handle())
    return out


def snr_sums(a, b, out=None, work=None):
    out = torch.empty(2, dtype=torch.float64, device=a.device) if out is None else out
    work = reduce_workspace(a.device) if work is None else work
    _native.call("msn_snr_sums", a.data_ptr(), b.data_ptr(), a.numel(), out.data_ptr(), work.data_ptr(),
                 work.numel(), stream_handle())
    return out


def snr_sums_f64(a, b, out=None, work=None):
    """sum a^2, sum (a - b)^2 of two contiguous float64 CUDA tensors, all in float64."""
    out = torch.empty(2, dtype=torch.float64, device=a.device) if out is None else out
    work = reduce_workspace(a.device) if work is None else work
    _native.call("msn_snr_sums_f64", a.data_ptr(), b.data_ptr(), a.numel(), out.data_ptr(), work.data_ptr(),
                 work.numel(), stream_handle())
    return out


def mul(a, b, out):
    _native.call("msn_mul", a.data_ptr(), b.data_ptr(), out.data_ptr(), a.numel(), stream_handle())
    return out


def sub(a, b, out):
    _native.call("msn_sub", a.data_ptr(), b.data_ptr(), out.data_ptr(), a.numel(), stream_handle())
    return out


def plane_max(w, use_abs=False, out=None, work=None):
    """Per-plane maximum (float32 device tensor)."""
    w = as_f32_cuda(w)
    planes = 1 if w.dim() == 2 else w.shape[0]
    per = w.numel() // planes
    out = torch.empty(planes, dtype=torch.float32, device=w.device) if out is None else out
    work = torch.empty(max(16, 4 * planes), dtype=torch.uint8, device=w.device) if work is None else work
    _native.call("msn_plane_max", w.data_ptr(), planes, per, 1 if use_abs else 0, out.data_ptr(), work.data_ptr(),
                 work.numel(), stream_handle())
    return out

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

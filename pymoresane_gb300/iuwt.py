"""Drop-in for pymoresane.iuwt (mode='gpu'): IUWT decomposition / recomposition.

Signatures follow pymoresane/iuwt.py:17 (iuwt_decomposition) and
pymoresane/iuwt.py:43 (iuwt_recomposition). Host (numpy) inputs are uploaded
as float32 and results come back as float32 numpy arrays; CUDA tensors are
accepted as inputs (the reference accepts pycuda gpuarrays,
pymoresane/iuwt.py:428-431) and ``store_on_gpu=True`` returns CUDA tensors.

Differences from the reference:
* only mode='gpu' is implemented; 'ser' and 'mp' raise ValueError (this
  package is the GPU path and has no CPU implementation);
* with store_on_gpu=True and store_smoothed=True the smoothed plane is
  returned as well (the reference drops it, pymoresane/iuwt.py:494-495).
"""
import numpy as np
import torch

from . import device as dev

GPU_MODES = ("gpu",)


def check_mode(mode, what):
    if mode not in GPU_MODES:
        raise ValueError(f"{what}: mode={mode!r} is not available in pymoresane_gb300, which implements "
                         f"the GPU path only (use mode='gpu')")


def to_host(t):
    return t.detach().cpu().numpy()


def iuwt_decomposition(in1, scale_count, scale_adjust=0, mode='gpu', core_count=2, store_smoothed=False,
                       store_on_gpu=False):
    """IUWT decomposition of ``in1`` into ``scale_count - scale_adjust`` detail planes.

    Reference: pymoresane/iuwt.py:17-41 -> gpu_iuwt_decomposition :384-499.
    ``core_count`` is accepted for signature compatibility and ignored.
    """
    check_mode(mode, "iuwt_decomposition")
    w, c = dev.iuwt_decompose(in1, int(scale_count), int(scale_adjust), store_smoothed=store_smoothed)
    if store_on_gpu:
        return (w, c) if store_smoothed else w
    if store_smoothed:
        return to_host(w), to_host(c)
    return to_host(w)


def iuwt_recomposition(in1, scale_adjust=0, mode='gpu', core_count=1, store_on_gpu=False, smoothed_array=None):
    """Inverse IUWT of a detail stack (plus the smoothest plane when given).

    Reference: pymoresane/iuwt.py:43-64 -> gpu_iuwt_recomposition :501-581.
    """
    check_mode(mode, "iuwt_recomposition")
    rec = dev.iuwt_recompose(in1, int(scale_adjust), smoothed=smoothed_array)
    return rec if store_on_gpu else to_host(rec)

"""The allocation-free IUWT decomposition entry point (msn_iuwt_decompose_static).

Some callers cannot give the library device scratch memory: a host imaging
pipeline whose own pool allocator owns all GPU memory, or a loop that must
never call cudaMalloc because it can block, fail under memory pressure or
synchronise the device. msn_iuwt_decompose_static serves them by keeping its
two scratch planes in a fixed device array inside libmsn.so (images up to
1,048,576 pixels). These tests call it through the C ABI and check that two
calls in a row give exactly what the workspace-based msn_iuwt_decompose gives
(the IUWT is deterministic and bit-exact, so the tolerance is zero), and that
larger images are refused with a clear error.

This file is collected last on purpose, so that a run stopping at the first
failure has already run every other test.
"""
import numpy as np
import pytest
import torch

from pymoresane_gb300 import _native
from pymoresane_gb300 import device as dev
from pymoresane_gb300 import synthetic

pytestmark = pytest.mark.gpu
MAX_PIXELS = 1 << 20


def decompose_static(x, scale_count, scale_adjust):
    ny, nx = x.shape
    detail = torch.empty((scale_count - scale_adjust, ny, nx), dtype=torch.float32, device=x.device)
    smoothed = torch.empty((ny, nx), dtype=torch.float32, device=x.device)
    args = ("msn_iuwt_decompose_static", x.data_ptr(), detail.data_ptr(), smoothed.data_ptr(), ny, nx,
            scale_count, scale_adjust, torch.cuda.current_stream().cuda_stream)
    # A first call with these arguments loads the kernels it uses: with lazy module
    # loading the driver may reserve device memory for them (and for the static array)
    # at that point. The call after it is the one checked.
    _native.call(*args)
    # torch's allocator counter sees allocations made through torch; the device's free
    # memory (cudaMemGetInfo) also sees a cudaMalloc made inside libmsn.so itself.
    torch.cuda.synchronize()
    before = torch.cuda.memory_allocated()
    free_before = torch.cuda.mem_get_info()[0]
    _native.call(*args)
    torch.cuda.synchronize()
    assert torch.cuda.memory_allocated() == before
    assert torch.cuda.mem_get_info()[0] == free_before
    return detail, smoothed


def test_static_matches_workspace_entry_point_on_two_calls(cuda):
    cases = [((1024, 1024), 8, 0, 11), ((256, 512), 6, 2, 12)]   # the second call reuses the array
    for shape, scales, adj, seed in cases:
        img = synthetic.iuwt_image(shape[0], 40, seed=seed)[:, :shape[1]] if shape[0] == shape[1] else \
            np.random.default_rng(seed).standard_normal(shape).astype(np.float32)
        x = torch.from_numpy(np.ascontiguousarray(img)).to(cuda)
        got_w, got_c = decompose_static(x, scales, adj)
        ref_w, ref_c = dev.iuwt_decompose(x, scales, adj, store_smoothed=True)
        torch.cuda.synchronize()
        assert torch.equal(got_w, ref_w)
        assert torch.equal(got_c, ref_c)


def test_static_refuses_images_beyond_the_limit(cuda):
    x = torch.zeros((1024, 1028), dtype=torch.float32, device=cuda)   # 1,052,672 pixels
    assert x.numel() > MAX_PIXELS
    with pytest.raises(ValueError, match="static scratch limit"):
        decompose_static(x, 4, 0)

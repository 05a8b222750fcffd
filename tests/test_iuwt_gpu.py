"""GPU parity of the IUWT (msn_iuwt_decompose / msn_iuwt_recompose) against the oracle.

* bit-exact against the FP32 restatement of the reference's pyCUDA kernels
  (``oracle.iuwt`` with arith='f32fma') on small images;
* within 2e-6 x max|x| of the FP64 reference path ('ser');
* against the committed golden vectors of the reference itself;
* full-size (4096^2, 8 scales) size-independent properties: perfect
  reconstruction and linearity.
"""
import os

import numpy as np
import pytest
import torch

from oracle import iuwt as O
from pymoresane_gb300 import device as dev
from pymoresane_gb300 import iuwt as G
from pymoresane_gb300 import synthetic

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
F64_TOL = 2e-6   # max abs error / max |input| vs the FP64 oracle


def rand(shape, seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(shape).astype(np.float32)
    x[shape[0] // 3, shape[1] // 4] += 30.0
    return x


@pytest.mark.parametrize("shape,scales,adj", [((64, 64), 4, 0), ((64, 64), 5, 2), ((48, 96), 4, 1),
                                              ((128, 32), 5, 0), ((40, 52), 2, 0), ((256, 256), 7, 3)])
def test_decompose_bit_exact_vs_f32_oracle(cuda, shape, scales, adj):
    x = rand(shape, 1)
    d, c = G.iuwt_decomposition(x, scales, adj, mode="gpu", store_smoothed=True)
    od, oc = O.decompose(x, scales, adj, store_smoothed=True, arith="f32fma")
    assert d.dtype == np.float32 and d.shape == od.shape
    assert np.array_equal(d.view(np.uint32), od.view(np.uint32))
    assert np.array_equal(c.view(np.uint32), oc.view(np.uint32))


@pytest.mark.parametrize("adj,with_smoothed", [(0, True), (0, False), (2, True), (2, False)])
def test_recompose_bit_exact_vs_f32_oracle(cuda, adj, with_smoothed):
    x = rand((64, 128), 2)
    od, oc = O.decompose(x, 5, adj, store_smoothed=True, arith="f32fma")
    sm = oc if with_smoothed else None
    r = G.iuwt_recomposition(od, adj, mode="gpu", smoothed_array=sm)
    orr = O.recompose(od, adj, smoothed_array=sm, arith="f32fma")
    assert np.array_equal(r.view(np.uint32), orr.view(np.uint32))


def test_recompose_signed_zero_start(cuda):
    w = np.zeros((2, 16, 16), np.float32)
    w[0, 3, 3] = -0.0
    w[1] = -0.0
    r = G.iuwt_recomposition(w, 0, mode="gpu")
    orr = O.recompose(w, 0, arith="f32fma")
    assert np.array_equal(r.view(np.uint32), orr.view(np.uint32))


def test_against_reference_golden(cuda):
    g = np.load(os.path.join(GOLDEN, "iuwt.npz"))
    x = g["x"]
    scale = np.max(np.abs(x))
    for adj in (0, 1, 2):
        d, c = G.iuwt_decomposition(x, 4, adj, mode="gpu", store_smoothed=True)
        assert np.max(np.abs(d - g[f"ser_detail_adj{adj}"])) <= F64_TOL * scale
        assert np.max(np.abs(c - g[f"ser_smoothed_adj{adj}"])) <= F64_TOL * scale
        r = G.iuwt_recomposition(g[f"ser_detail_adj{adj}"], adj, mode="gpu",
                                 smoothed_array=g[f"ser_smoothed_adj{adj}"])
        assert np.max(np.abs(r - g[f"ser_recomp_smoothed_adj{adj}"])) <= F64_TOL * scale


def test_max_scale_equals_side(cuda):
    # 2^scale_count == N: the largest dilation the mirror rule allows.
    x = rand((32, 32), 3)
    d = G.iuwt_decomposition(x, 5, 0, mode="gpu")
    od = O.decompose(x, 5, 0, arith="f32fma")
    assert np.array_equal(d, od)


def test_device_inputs_and_store_on_gpu(cuda):
    x = rand((64, 64), 4)
    xt = torch.from_numpy(x).cuda()
    w, c = G.iuwt_decomposition(xt, 3, 0, mode="gpu", store_smoothed=True, store_on_gpu=True)
    assert w.is_cuda and c.is_cuda
    r = G.iuwt_recomposition(w, 0, mode="gpu", store_on_gpu=True, smoothed_array=c)
    assert r.is_cuda
    assert torch.max(torch.abs(r - xt)).item() < 1e-4


def test_empty_detail_stack(cuda):
    x = rand((32, 32), 5)
    d, c = G.iuwt_decomposition(x, 2, 2, mode="gpu", store_smoothed=True)
    assert d.shape == (0, 32, 32)
    oc = O.a_trous(O.a_trous(x, 0, "f32fma"), 1, "f32fma")
    assert np.array_equal(c, oc)


def test_invalid_arguments(cuda):
    with pytest.raises(ValueError):
        G.iuwt_decomposition(np.zeros((32, 30), np.float32), 2, mode="gpu")     # nx % 4
    with pytest.raises(ValueError):
        G.iuwt_decomposition(np.zeros((32, 32), np.float32), 6, mode="gpu")     # 2^6 > 32
    with pytest.raises(ValueError):
        G.iuwt_decomposition(np.zeros((32, 32), np.float32), 2, 3, mode="gpu")  # adjust > count
    with pytest.raises(ValueError):
        G.iuwt_decomposition(np.zeros((32, 32), np.float32), 2, mode="ser")


def test_full_size_reconstruction_and_linearity(cuda):
    # 4096^2, 8 scales (the IUWT benchmark workload): size-independent properties.
    x = torch.from_numpy(synthetic.iuwt_image(4096, 500, seed=11)).cuda()
    y = torch.from_numpy(synthetic.iuwt_image(4096, 500, seed=12)).cuda()
    wx, cx = dev.iuwt_decompose(x, 8, 0, store_smoothed=True)
    rx = dev.iuwt_recompose(wx, 0, smoothed=cx)
    assert torch.max(torch.abs(rx - x)).item() <= 1e-5 * torch.max(torch.abs(x)).item()
    wy, cy = dev.iuwt_decompose(y, 8, 0, store_smoothed=True)
    ws, cs = dev.iuwt_decompose(x + y, 8, 0, store_smoothed=True)
    lin = torch.max(torch.abs(ws - (wx + wy))).item()
    assert lin <= 1e-5 * torch.max(torch.abs(x + y)).item()
    # per-plane sums of detail coefficients vanish up to rounding (the B3 filter preserves the mean)
    assert torch.allclose(cx.double().mean(), x.double().mean(), rtol=0, atol=1e-4)


def test_full_size_rows_match_f32_oracle(cuda):
    # A band of rows of the 4096^2 decomposition is checked bit-exactly against the oracle.
    x = synthetic.iuwt_image(1024, 50, seed=3)
    d = G.iuwt_decomposition(x, 8, 0, mode="gpu")
    od = O.decompose(x, 8, 0, arith="f32fma")
    assert np.array_equal(d, od)


@pytest.mark.parametrize("shape,scales,adj", [((64, 64), 4, 0), ((128, 96), 5, 2)])
def test_masked_decomposition_equals_product(cuda, shape, scales, adj):
    # msn_iuwt_decompose_masked == mask * msn_iuwt_decompose, bit for bit (main.py:381-383)
    x = torch.from_numpy(rand(shape, 7)).cuda()
    rng = np.random.default_rng(8)
    mask = torch.from_numpy((rng.random((scales - adj,) + shape) < 0.3).astype(np.float32)).cuda()
    w, _ = dev.iuwt_decompose(x, scales, adj)
    got = dev.iuwt_decompose_masked(x, mask, scales, adj)
    want = w * mask
    assert torch.equal(got.view(torch.int32), want.view(torch.int32))


@pytest.mark.parametrize("n,scales,adj,blobs", [(64, 4, 0, 3), (256, 6, 1, 10), (128, 5, 0, 0), (512, 7, 2, 30),
                                                 (96, 2, 1, 4)])
def test_decompose_masked_rows_matches_dense(cuda, n, scales, adj, blobs):
    """Skipping the mask's empty rows leaves exactly the dense masked decomposition (zeros compare equal)."""
    from pymoresane_gb300 import _native
    rng = np.random.default_rng(n + scales + blobs)
    planes = scales - adj
    mask = np.zeros((planes, n, n), np.float32)
    for _ in range(blobs):
        p, y, x = rng.integers(0, planes), rng.integers(0, n - 8), rng.integers(0, n - 8)
        mask[p, y:y + rng.integers(1, 8), x:x + rng.integers(1, 8)] = 1.0
    x = torch.from_numpy(rng.standard_normal((n, n)).astype(np.float32)).cuda()
    m = torch.from_numpy(mask).cuda()
    dense = dev.iuwt_decompose_masked(x, m, scales, adj)
    flags = torch.empty(planes * n, dtype=torch.uint8, device="cuda")
    st = dev.stream_handle()
    _native.call("msn_row_flags", m.data_ptr(), planes * n, n, flags.data_ptr(), st)
    assert np.array_equal(flags.cpu().numpy().astype(bool), (mask != 0).any(axis=2).reshape(-1))
    out = torch.zeros_like(dense)
    work = dev.iuwt_workspace(n, n, x.device)
    _native.call("msn_iuwt_decompose_masked_rows", x.data_ptr(), m.data_ptr(), flags.data_ptr(), out.data_ptr(), n, n,
                 scales, adj, work.data_ptr(), work.numel(), st)
    assert np.array_equal(out.cpu().numpy(), dense.cpu().numpy())


@pytest.mark.parametrize("n,planes,adj,blobs", [(64, 4, 0, 3), (256, 6, 1, 10), (128, 5, 0, 0), (512, 7, 2, 25),
                                                 (96, 1, 1, 4)])
def test_recompose_rows_matches_dense(cuda, n, planes, adj, blobs):
    """Recomposition restricted to the active rows equals the dense one on a row-sparse stack (zeros compare equal)."""
    from pymoresane_gb300 import _native
    rng = np.random.default_rng(3 * n + planes + blobs)
    w = np.zeros((planes, n, n), np.float32)
    for _ in range(blobs):
        p, y, x = rng.integers(0, planes), rng.integers(0, n - 8), rng.integers(0, n - 8)
        h, wd = rng.integers(1, 8), rng.integers(1, 8)
        w[p, y:y + h, x:x + wd] = rng.standard_normal((h, wd)).astype(np.float32)
    wt = torch.from_numpy(w).cuda()
    dense = dev.iuwt_recompose(wt, adj)
    st = dev.stream_handle()
    flags = torch.empty(planes * n, dtype=torch.uint8, device="cuda")
    _native.call("msn_row_flags", wt.data_ptr(), planes * n, n, flags.data_ptr(), st)
    act = torch.empty((planes + adj) * n, dtype=torch.uint8, device="cuda")
    _native.call("msn_recompose_row_activity", flags.data_ptr(), planes, n, adj, act.data_ptr(), st)
    out = torch.full((n, n), 7.0, device="cuda")          # stale contents must be overwritten
    work = dev.iuwt_workspace(n, n, wt.device)
    work.fill_(0x7f)
    _native.call("msn_iuwt_recompose_rows", wt.data_ptr(), planes, act.data_ptr(), out.data_ptr(), n, n, adj,
                 work.data_ptr(), work.numel(), st)
    d = dense.cpu().numpy()
    assert np.array_equal(out.cpu().numpy(), d)
    # the activity covers every non-zero row of the result
    rows = (d != 0).any(axis=1)
    assert not np.any(rows & ~act.cpu().numpy()[:n].astype(bool))
    # the variant that never touches inactive rows: cleared output and recomposition planes, two calls
    # in a row with one activity map (as the minor loop calls it), and a second stack on the same map
    out2 = torch.zeros((n, n), device="cuda")
    work.zero_()
    for stack in (wt, wt * 0.5):
        _native.call("msn_iuwt_recompose_active_rows", stack.data_ptr(), planes, act.data_ptr(), out2.data_ptr(), n,
                     n, adj, work.data_ptr(), work.numel(), st)
        work[:2 * ((n * n * 4 + 255) // 256 * 256)].fill_(0x7f)   # planes 0 and 1 are free scratch
        assert np.array_equal(out2.cpu().numpy(), dev.iuwt_recompose(stack, adj).cpu().numpy())

"""GPU parity of the noise estimate, thresholding, labelling, extraction and CG reductions.

Integer / mask / selection work is checked bit-exactly against the oracle
(and scipy.ndimage.label); float64 reductions within 1e-12 relative.
"""
import os

import numpy as np
import pytest
import torch

from oracle import iuwt as OI
from oracle import toolbox as T
from pymoresane_gb300 import device as dev
from pymoresane_gb300 import iuwt_toolbox as G

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def golden():
    return np.load(os.path.join(GOLDEN, "toolbox.npz"))


@pytest.mark.parametrize("ee,ie", [(0, 0), (3, 0), (0, 5), (4, 7), (0, 70)])
def test_estimate_threshold_golden(cuda, ee, ie):
    g = golden()
    got = G.estimate_threshold(g["decomp"], ee, ie)
    assert got.dtype == np.float64
    assert np.array_equal(got, g[f"thr_{ee}_{ie}"])


@pytest.mark.parametrize("shape,ee,ie", [((3, 64, 64), 0, 0), ((2, 63, 64), 0, 0), ((2, 64, 60), 5, 3),
                                         ((1, 256, 256), 0, 10), ((4, 512, 512), 17, 0)])
def test_estimate_threshold_random(cuda, shape, ee, ie):
    rng = np.random.default_rng(sum(shape) + ee + ie)
    w = (rng.standard_normal(shape) * rng.uniform(0.1, 3, (shape[0], 1, 1))).astype(np.float32)
    w[0, :3, :3] = 0.0            # ties and zeros
    w[-1, 5, :] = w[-1, 5, 0]
    assert np.array_equal(G.estimate_threshold(w, ee, ie), T.estimate_threshold(w, ee, ie))


def test_estimate_threshold_full_size(cuda):
    # 2048^2 x 7 planes of Laplacian noise: the exact median must match numpy's.
    rng = np.random.default_rng(77)
    w = rng.laplace(0, 1, (7, 2048, 2048)).astype(np.float32)
    assert np.array_equal(G.estimate_threshold(w), T.estimate_threshold(w))


def test_apply_threshold_golden_bit_exact(cuda):
    g = golden()
    got = G.apply_threshold(g["decomp"], g["thr_0_0"], 4)
    assert np.array_equal(got.view(np.uint32), g["thresh"].view(np.uint32))
    got2 = G.apply_threshold(g["decomp"][1], g["thr_0_0"][1], 3)
    assert np.array_equal(got2.view(np.uint32), g["thresh_2d"].view(np.uint32))


def test_threshold_suppression_and_max(cuda):
    g = golden()
    d = torch.from_numpy(g["decomp"]).cuda()
    sig = torch.from_numpy(g["thr_0_0"]).cuda()
    rects = torch.tensor([[4, 124, 6, 120]] * d.shape[0], dtype=torch.int32, device="cuda")
    out, pmax = dev.apply_threshold(d, sig, 4, supp_rects=rects, want_max=True)
    ref = T.apply_threshold(g["decomp"], g["thr_0_0"], 4)
    supp = np.zeros(g["decomp"].shape[1:], np.float32)
    supp[4:124, 6:120] = 1
    ref = ref * supp
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(pmax.cpu().numpy(), ref.reshape(ref.shape[0], -1).max(axis=1))


@pytest.mark.parametrize("neg", [False, True])
def test_source_extraction_golden(cuda, neg):
    g = golden()
    src, msk = G.source_extraction(g["thresh"][1:4], 0.75, mode="gpu", neg_comp=neg)
    assert src.dtype == np.float64 and msk.dtype == np.int32
    assert np.array_equal(msk, g[f"mask_neg{int(neg)}"])
    assert np.array_equal(src.view(np.uint64), g[f"src_neg{int(neg)}"].view(np.uint64))


@pytest.mark.parametrize("n,planes,density,tol", [(64, 3, 0.05, 0.75), (128, 4, 0.2, 0.5), (256, 5, 0.02, 0.9),
                                                  (512, 2, 0.4, 0.3)])
def test_source_extraction_random(cuda, n, planes, density, tol):
    rng = np.random.default_rng(n * planes)
    w = rng.standard_normal((planes, n, n)).astype(np.float32)
    w[rng.random((planes, n, n)) > density] = 0.0
    for neg in (False, True):
        src, msk = G.source_extraction(w, tol, mode="gpu", neg_comp=neg)
        osrc, omsk = T.source_extraction(w, tol, neg, semantics="gpu")
        assert np.array_equal(msk, omsk)
        assert np.array_equal(src.view(np.uint64), osrc.view(np.uint64))


def test_source_extraction_store_on_gpu(cuda):
    g = golden()
    src, msk = G.source_extraction(g["thresh"][1:4], 0.75, mode="gpu", store_on_gpu=True)
    assert isinstance(msk, torch.Tensor) and msk.is_cuda and msk.dtype == torch.float32
    assert np.array_equal(msk.cpu().numpy().astype(np.int32), g["mask_neg0"])


@pytest.mark.parametrize("shape,density", [((1, 1), 1.0), ((7, 12), 0.5), ((64, 64), 0.3), ((100, 256), 0.6),
                                           ((256, 256), 0.45), ((1024, 1024), 0.5), ((2048, 2048), 0.03)])
def test_label_matches_scipy(cuda, shape, density):
    rng = np.random.default_rng(shape[0] * 7 + shape[1])
    img = (rng.random(shape) < density).astype(np.float32) * rng.standard_normal(shape).astype(np.float32)
    got, cnt = G.label(img)
    ref, rcnt = T.label(img)
    assert cnt == rcnt
    assert np.array_equal(got, ref)


def test_label_worst_case_snake(cuda):
    # one long serpentine component + isolated pixels: deep union-find chains
    n = 512
    img = np.zeros((n, n), np.float32)
    img[::2, :] = 1.0
    img[1::4, -1] = 1.0
    img[3::4, 0] = 1.0
    img[1::4, 5] = 2.0   # isolated-ish bridges too
    got, cnt = G.label(img)
    ref, rcnt = T.label(img)
    assert cnt == rcnt and np.array_equal(got, ref)


def test_snr_ratio(cuda):
    g = golden()
    a = g["thresh"][1:4]
    b = g["decomp"][1:4]
    # float64 accumulation of four-element float32 partials: ~1e-7 relative on the norms
    assert abs(G.snr_ratio(a, b) - T.snr_ratio(a.astype(np.float64), b)) <= 1e-6 * abs(T.snr_ratio(a, b))


def test_snr_ratio_float64_inputs(cuda):
    # float64 inputs reduce in float64 (np.linalg.norm, iuwt_toolbox.py:304): the reference's golden value
    g = golden()
    a = g["thresh"][1:4].astype(np.float64)
    b = g["decomp"][1:4]
    want = float(g["snr"])
    assert abs(G.snr_ratio(a, b) - want) <= 1e-12 * abs(want)
    assert abs(G.snr_ratio(torch.as_tensor(a).cuda(), torch.as_tensor(b).cuda()) - want) <= 1e-12 * abs(want)


def test_cg_vector_kernels(cuda):
    from pymoresane_gb300 import _native
    rng = np.random.default_rng(5)
    n = 300_004
    x, p, r, ap = (rng.standard_normal(n).astype(np.float32) for _ in range(4))
    t = {k: torch.from_numpy(v).cuda() for k, v in dict(x=x, p=p, r=r, ap=ap).items()}
    scal = torch.zeros(8, dtype=torch.float64, device="cuda")
    work = dev.reduce_workspace(t["x"].device)
    dev.dot2(t["r"], t["r"], t["p"], t["ap"], out=scal[0:2], work=work)
    rr, pap = np.dot(r.astype(np.float64), r), np.dot(p.astype(np.float64), ap)
    s = scal.cpu().numpy()
    assert abs(s[0] - rr) <= 1e-9 * rr and abs(s[1] - pap) <= 1e-9 * abs(abs(pap) + rr)
    xn = torch.empty_like(t["x"])
    neg = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    _native.call("msn_cg_alpha_x", t["x"].data_ptr(), t["p"].data_ptr(), scal.data_ptr(), xn.data_ptr(), n,
                 neg.data_ptr(), st)
    alpha = s[0] / s[1]
    af = np.float32(alpha)
    want = x + af * p                     # the reference's float32 expression with a float32 alpha
    assert np.array_equal(xn.cpu().numpy(), want)
    assert neg.item() == int(np.sum(want < 0))
    rn = torch.empty_like(t["r"])
    _native.call("msn_cg_residual", t["r"].data_ptr(), t["ap"].data_ptr(), scal.data_ptr(), rn.data_ptr(), n,
                 work.data_ptr(), work.numel(), st)
    rn_ref = r - af * ap
    assert np.array_equal(rn.cpu().numpy(), rn_ref)
    s = scal.cpu().numpy()
    rnrn = np.dot(rn_ref.astype(np.float64), rn_ref)
    assert abs(s[3] - rnrn) <= 1e-9 * rnrn and s[4] == s[3] / s[0]
    pp = t["p"].clone()
    _native.call("msn_cg_direction", rn.data_ptr(), pp.data_ptr(), scal.data_ptr(), n, st)
    assert np.array_equal(pp.cpu().numpy(), rn_ref + np.float32(s[4]) * p)
    # positivity
    xpos = xn.clone()
    ppos = t["p"].clone()
    _native.call("msn_cg_positivity", t["x"].data_ptr(), xpos.data_ptr(), ppos.data_ptr(), scal.data_ptr(), n, st)
    clamped = np.where(want < 0, np.float32(0), want)
    assert np.array_equal(xpos.cpu().numpy(), clamped)
    assert np.array_equal(ppos.cpu().numpy(), (clamped - x) / af)
    # the fused step equals cg_alpha_x followed by cg_residual bit for bit (vectors and scalars)
    scal2 = torch.zeros(8, dtype=torch.float64, device="cuda")
    scal2[0:2] = scal[0:2]
    xn2, rn2 = torch.empty_like(xn), torch.empty_like(rn)
    _native.call("msn_cg_step", t["x"].data_ptr(), t["p"].data_ptr(), t["r"].data_ptr(), t["ap"].data_ptr(),
                 scal2.data_ptr(), xn2.data_ptr(), rn2.data_ptr(), n, work.data_ptr(), work.numel(), st)
    assert torch.equal(xn2, xn) and torch.equal(rn2, rn)
    assert torch.equal(scal2[2:5], scal[2:5])
    # r.r of the next iteration equals this iteration's rn.rn bit for bit (carried in the minor loop)
    rr_next = torch.zeros(2, dtype=torch.float64, device="cuda")
    dev.dot2(rn.reshape(-1), rn.reshape(-1), out=rr_next, work=work)
    assert rr_next[0].item() == scal[3].item()


def test_region_std_and_model_update(cuda):
    from pymoresane_gb300 import _native
    rng = np.random.default_rng(9)
    img = rng.standard_normal((96, 96)).astype(np.float32)
    t = torch.from_numpy(img).cuda()
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    work = dev.reduce_workspace(t.device)
    st = torch.cuda.current_stream().cuda_stream
    _native.call("msn_region_std", t.data_ptr(), 96, 64, 64, 16, 16, out.data_ptr(), work.data_ptr(), work.numel(), st)
    ref = img[16:80, 16:80].astype(np.float64)
    o = out.cpu().numpy()
    # float64 accumulation of four-element float32 partials
    assert abs(o[2] - ref.mean()) <= 1e-7 and abs(o[3] - ref.std()) <= 1e-7 * ref.std()
    x = rng.standard_normal((64, 64)).astype(np.float32)
    xt = torch.from_numpy(x).cuda()
    model = torch.zeros((96, 96), dtype=torch.float32, device="cuda")
    _native.call("msn_model_update", model.data_ptr(), 96, xt.data_ptr(), 64, 16, 16, 0.2, 1, st)
    m = np.zeros((96, 96), np.float32)
    m[16:80, 16:80] += np.float32(0.2) * x
    assert np.array_equal(model.cpu().numpy(), m)


@pytest.mark.parametrize("planes,n,blobs", [(3, 64, 2), (5, 256, 6), (2, 100, 0), (7, 512, 40)])
def test_snr_update_masked_matches_dense(cuda, planes, n, blobs):
    """The segment-skipping SNR pass gives the dense pass's running sum and norms bit for bit."""
    from pymoresane_gb300 import _native
    rng = np.random.default_rng(planes * n + blobs)
    mask = np.zeros((planes, n, n), np.float32)
    for _ in range(blobs):
        p, y, x = rng.integers(0, planes), rng.integers(0, n - 8), rng.integers(0, n - 8)
        mask[p, y:y + rng.integers(1, 8), x:x + rng.integers(1, 8)] = 1.0
    w = rng.standard_normal(mask.shape).astype(np.float32)
    e = torch.from_numpy(mask * w).cuda()                     # extracted sources (signed zeros outside)
    q = torch.from_numpy(mask * rng.standard_normal(mask.shape).astype(np.float32)).cuda()
    ms0 = torch.from_numpy(mask * rng.standard_normal(mask.shape).astype(np.float32)).cuda()
    scal = torch.tensor([1.0, 2.0, -0.37, 0.0, 0.0, 0, 0, 0], dtype=torch.float64, device="cuda")
    work = dev.reduce_workspace(e.device)
    st = dev.stream_handle()
    n_el = e.numel()
    flags = torch.empty(max(1, _native.query("msn_segment_flags_bytes", n_el)), dtype=torch.uint8, device="cuda")
    _native.call("msn_segment_flags", torch.from_numpy(mask).cuda().data_ptr(), n_el, flags.data_ptr(), st)
    seg = mask.reshape(-1)
    pad = (-seg.size) % 128
    want = (np.concatenate([seg, np.zeros(pad, np.float32)]).reshape(-1, 128) != 0).any(axis=1)
    assert np.array_equal(flags.cpu().numpy()[:want.size].astype(bool), want)
    outs = []
    for masked in (False, True):
        ms = ms0.clone()
        out2 = torch.zeros(2, dtype=torch.float64, device="cuda")
        if masked:
            _native.call("msn_snr_update_masked", e.data_ptr(), ms.data_ptr(), q.data_ptr(), scal.data_ptr(), n_el,
                         flags.data_ptr(), out2.data_ptr(), work.data_ptr(), work.numel(), st)
        else:
            _native.call("msn_snr_update", e.data_ptr(), ms.data_ptr(), q.data_ptr(), scal.data_ptr(), n_el,
                         out2.data_ptr(), work.data_ptr(), work.numel(), st)
        outs.append((ms.cpu().numpy(), out2.cpu().numpy()))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])
    # and the running sum is ms + (float32)alpha * q as in the reference's float32 update
    a = np.float32(-0.37)
    assert np.array_equal(outs[1][0], ms0.cpu().numpy() + a * q.cpu().numpy())

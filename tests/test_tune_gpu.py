"""The autotuner on the GPU: it picks values, and no value changes a result."""
import numpy as np
import pytest
import torch

from pymoresane_gb300 import device as dev
from pymoresane_gb300 import synthetic, tune

pytestmark = pytest.mark.gpu


def test_autotune_choices_do_not_change_results(cuda, tmp_path):
    rng = np.random.default_rng(11)
    x = torch.from_numpy(rng.standard_normal((2048, 2048)).astype(np.float32)).cuda()
    spec = dev.psf_spectrum(synthetic.make_psf(4096, 3000, rng))
    tune.reset()
    try:
        ref = dev.fft_convolve(x, spec).clone()
        w_ref = dev.iuwt_decompose(x, 6, 0)[0].clone()
        res = tune.autotune(n=2048, reps=3, path=str(tmp_path / "tune.json"))
        assert set(res["values"]) == set(tune.KNOBS)
        assert "iuwt_threads_wide" not in res["tuned"] and "fft_four_step" in res["tuned"]
        cached = tune.load_cache(str(tmp_path / "tune.json"))[tune.device_key()]["values"]
        assert all(cached[k] == v for k, v in res["tuned"].items())
        # every candidate of every knob gives the same convolution (within the FFT tolerance) and the
        # same wavelet coefficients (bit for bit)
        for four_step in (0, 1):
            for ctas in (0, 2):
                tune.set_values({"fft_four_step": four_step, "fft_sq_col_ctas": ctas, "fft_sq_fwd_ctas": ctas,
                                 "fft_sq_inv_ctas": ctas})
                got = dev.fft_convolve(x, spec)
                if four_step:
                    grids = tune.sq_grids()
                    sms = torch.cuda.get_device_properties(0).multi_processor_count
                    assert all(0 < g for g in grids) and (ctas == 0 or max(grids) <= ctas * sms), grids
                assert torch.max(torch.abs(got - ref)).item() <= 1e-5 * torch.max(torch.abs(ref)).item()
        for threads in (64, 128, 256):
            tune.set_values({"iuwt_threads": threads})
            assert torch.equal(dev.iuwt_decompose(x, 6, 0)[0], w_ref)
        # wide rows have their own parameter
        xw = torch.from_numpy(rng.standard_normal((64, 4096)).astype(np.float32)).cuda()
        ww_ref = dev.iuwt_decompose(xw, 5, 0)[0].clone()
        for threads in (64, 128, 256):
            tune.set_values({"iuwt_threads_wide": threads})
            assert torch.equal(dev.iuwt_decompose(xw, 5, 0)[0], ww_ref)
    finally:
        tune.reset()


def test_autotune_times_the_cta_size_on_a_given_workload(cuda, tmp_path):
    # with workload=, the a trous CTA size is timed on the caller's operation (every candidate
    # runs it); the convolution parameters still on the convolution
    rng = np.random.default_rng(5)
    x = torch.from_numpy(rng.standard_normal((2048, 2048)).astype(np.float32)).cuda()
    calls = []

    def work():
        calls.append(tune.get("iuwt_threads"))
        dev.iuwt_decompose(x, 4, 0)

    tune.reset()
    try:
        res = tune.autotune(n=2048, reps=1, path=str(tmp_path / "tune.json"), workload=work)
        assert "iuwt_threads" in res["tuned"] and "fft_four_step" in res["tuned"]
        assert sorted(set(calls)) == sorted(tune.CANDIDATES["iuwt_threads"])
    finally:
        tune.reset()

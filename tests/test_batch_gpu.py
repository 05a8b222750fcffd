"""Batched / served deconvolution on one GPU: every result is the same alone and in the mix."""
import numpy as np
import pytest

from pymoresane_gb300 import synthetic

KW = dict(sigma_level=4, loop_gain=0.2, tolerance=0.75, accuracy=1e-6, major_loop_miter=30, minor_loop_miter=20,
          conv_mode="linear")


def _jobs():
    from pymoresane_gb300.batch import Job
    jobs = []
    for i, n in enumerate((128, 256, 128, 192, 256, 128)):
        w = synthetic.scaled(n, seed=100 + i)
        w.n_uv = max(w.n_uv, 400)
        dirty, psf, _ = synthetic.make_problem(w)
        jobs.append(Job(dirty, psf, kwargs=dict(KW, scale_count=max(2, int(np.log2(n)) - 3)), tag=i))
    return jobs


@pytest.mark.gpu
def test_results_same_alone_and_in_the_mix(cuda):
    import torch

    from pymoresane_gb300.batch import DeconvolutionExecutor
    from pymoresane_gb300.main import Deconvolver
    jobs = _jobs()
    alone = []
    for j in jobs:
        eng = Deconvolver(j.psf)
        model, residual, major = eng.moresane(torch.from_numpy(j.dirty).cuda(), **j.kwargs)
        alone.append((model.cpu().numpy(), residual.cpu().numpy(), major))
    for order in ("largest", "fifo"):
        with DeconvolutionExecutor(workers=4, order=order) as ex:
            mixed = ex.map(jobs)
        assert len({r.worker for r in mixed}) > 1
        for (m, r, k), res in zip(alone, mixed):
            assert res.major == k
            assert np.array_equal(res.model, m)
            assert np.array_equal(res.residual, r)


@pytest.mark.gpu
def test_serve_reports_latency(cuda):
    from pymoresane_gb300.batch import serve
    jobs = _jobs()[:4]
    arrivals = [0.0, 0.01, 0.02, 0.5]
    results, wall = serve(jobs, arrivals, workers=2)
    assert all(r is not None for r in results)
    assert all(r.t_start >= r.t_submit and r.t_end > r.t_start for r in results)
    assert wall >= 0.5


@pytest.mark.gpu
def test_failing_job_reports_and_releases(cuda):
    # an odd-sized image is rejected (main.py:101-103); the error reaches the caller's future,
    # the job's memory reservation is returned and the other jobs still complete
    from pymoresane_gb300.batch import DeconvolutionExecutor, Job
    jobs = _jobs()[:2]
    bad = Job(np.zeros((127, 127), np.float32), jobs[0].psf, kwargs=dict(KW, scale_count=3), tag="bad")
    with DeconvolutionExecutor(workers=2) as ex:
        futs = [ex.submit(j) for j in (jobs[0], bad, jobs[1])]
        with pytest.raises(ValueError, match="uneven"):
            futs[1].result(timeout=300)
        assert futs[0].result(timeout=300).major >= 0 and futs[2].result(timeout=300).major >= 0
    # every reservation (jobs' transients, workers' cached buffers) is returned at shutdown
    assert ex.gate.used == 0

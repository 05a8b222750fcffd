"""CPU oracle for the PyMORESANE deconvolution hot path.

TEST INFRASTRUCTURE ONLY. This package restates the reference algorithms in
numpy so that the CUDA implementation in ``pymoresane_gb300`` can be checked
against them. Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU-baseline / reference legs may import it, and there only as the checker or
the timed CPU baseline. The product package never imports it and has no CPU
fallback.

Parity pinning: every restated function is checked against golden vectors
produced by running the reference's own Python code (loaded under Python 3 by
``tests/golden/refshim.py``) with ``tests/golden/make_golden.py``; the
fixtures are committed under ``tests/golden/`` and exercised by
``tests/test_oracle_golden.py``.

Modules:
  iuwt         -- a trous smoothing, IUWT decomposition / recomposition
  convolution  -- FFT convolution (linear / circular), PSF spectra
  toolbox      -- MAD threshold, thresholding, source extraction, SNR
  moresane     -- the MORESANE major / minor loops
"""

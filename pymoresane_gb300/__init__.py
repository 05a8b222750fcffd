"""pymoresane_gb300 -- GB300 (sm_103a) implementation of the PyMORESANE deconvolution hot path.

The modules mirror the reference package's public functions for mode='gpu':

* ``pymoresane_gb300.iuwt``              -- iuwt_decomposition / iuwt_recomposition
* ``pymoresane_gb300.iuwt_convolution``  -- fft_convolve and helpers
* ``pymoresane_gb300.iuwt_toolbox``      -- estimate_threshold, apply_threshold,
                                            source_extraction, snr_ratio
* ``pymoresane_gb300.main``              -- DataImage / FitsImage (moresane, moresane_by_scale)

All arithmetic runs in libmsn.so (hand-written CUDA, C ABI in include/msn.h);
``device`` holds the torch-tensor level wrappers.
"""
__version__ = "0.1.0"

"""ctypes binding of libmsn.so (declared in include/msn.h).

The library is loaded from the package directory; there is no fallback: if it
is missing or CUDA is unavailable every entry point raises.
"""
import ctypes
import os
import threading

_LIB = None
_LOCK = threading.Lock()
LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libmsn.so")

c_int, c_size_t, c_void_p, c_float, c_double = (ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p,
                                                ctypes.c_float, ctypes.c_double)

# name -> (restype, [argtypes]); kept in the order of include/msn.h.
SIGNATURES = {
    "msn_last_error": (ctypes.c_char_p, []),
    "msn_version": (c_int, []),
    "msn_launch_count": (ctypes.c_ulonglong, [c_int]),
    "msn_iuwt_workspace_bytes": (c_size_t, [c_int, c_int]),
    "msn_iuwt_decompose": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_size_t,
                                   c_void_p]),
    "msn_iuwt_decompose_masked": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_void_p,
                                          c_size_t, c_void_p]),
    "msn_iuwt_decompose_masked_rows": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int,
                                               c_void_p, c_size_t, c_void_p]),
    "msn_recompose_row_activity": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p]),
    "msn_iuwt_recompose_rows": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_size_t,
                                        c_void_p]),
    "msn_iuwt_recompose_active_rows": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_int, c_int, c_int, c_void_p,
                                               c_size_t, c_void_p]),
    "msn_iuwt_recompose": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_size_t,
                                   c_void_p]),
    "msn_iuwt_decompose_static": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_void_p]),
    "msn_fft_workspace_bytes": (c_size_t, [c_int, c_int]),
    "msn_spectrum_elems": (c_size_t, [c_int]),
    "msn_psf_spectrum": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_size_t,
                                 c_void_p]),
    "msn_spectrum_pack": (c_int, [c_void_p, c_int, c_void_p, c_void_p]),
    "msn_fft_convolve": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_size_t, c_void_p]),
    "msn_fft_convolve_rows": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_size_t,
                                      c_void_p]),
    "msn_fft_status": (c_int, [c_void_p]),
    "msn_fft_sq_grids": (c_int, [c_void_p]),
    "msn_rfft2": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_size_t, c_void_p]),
    "msn_irfft2": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_size_t, c_void_p]),
    "msn_fft_shift": (c_int, [c_void_p, c_int, c_void_p]),
    "msn_crop_centre": (c_int, [c_void_p, c_int, c_void_p, c_void_p]),
    "msn_scale": (c_int, [c_void_p, c_size_t, c_float, c_void_p]),
    "msn_toolbox_workspace_bytes": (c_size_t, [c_int, c_int, c_int]),
    "msn_mad_sigma": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "msn_apply_threshold": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_double, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_size_t, c_void_p]),
    "msn_source_extraction": (c_int, [c_void_p, c_int, c_int, c_int, c_float, c_int, c_void_p, c_void_p, c_void_p,
                                      c_size_t, c_void_p]),
    "msn_plane_max": (c_int, [c_void_p, c_int, c_size_t, c_int, c_void_p, c_void_p, c_size_t, c_void_p]),
    "msn_label": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "msn_reduce_workspace_bytes": (c_size_t, []),
    "msn_set_reduction_precision": (c_int, [c_int]),
    "msn_reduction_precision": (c_int, []),
    "msn_tune_set": (c_int, [ctypes.c_char_p, c_int]),
    "msn_tune_get": (c_int, [ctypes.c_char_p, c_void_p]),
    "msn_tune_reset": (c_int, []),
    "msn_tune_epoch": (ctypes.c_uint, []),
    "msn_dot2": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p, c_void_p, c_size_t, c_void_p]),
    "msn_snr_sums": (c_int, [c_void_p, c_void_p, c_size_t, c_void_p, c_void_p, c_size_t, c_void_p]),
    "msn_snr_sums_f64": (c_int, [c_void_p, c_void_p, c_size_t, c_void_p, c_void_p, c_size_t, c_void_p]),
    "msn_snr_update": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p, c_void_p, c_size_t,
                               c_void_p]),
    "msn_segment_flags_bytes": (c_size_t, [c_size_t]),
    "msn_segment_flags": (c_int, [c_void_p, c_size_t, c_void_p, c_void_p]),
    "msn_row_flags": (c_int, [c_void_p, c_size_t, c_int, c_void_p, c_void_p]),
    "msn_snr_update_masked": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p, c_void_p, c_void_p,
                                      c_size_t, c_void_p]),
    "msn_cg_alpha_x": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p, c_void_p]),
    "msn_cg_positivity": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "msn_cg_residual": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p, c_size_t, c_void_p]),
    "msn_cg_step": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p,
                            c_size_t, c_void_p]),
    "msn_cg_direction": (c_int, [c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "msn_model_update": (c_int, [c_void_p, c_int, c_void_p, c_int, c_int, c_int, c_float, c_int, c_void_p]),
    "msn_sub": (c_int, [c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "msn_add": (c_int, [c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "msn_mul": (c_int, [c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "msn_region_std": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_size_t, c_void_p]),
    "msn_minor_engine_create": (c_int, [ctypes.POINTER(c_void_p)]),
    "msn_minor_engine_destroy": (c_int, [c_void_p]),
    "msn_minor_loop": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    "msn_moresane_run": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p]),
}

MINOR_RUNNING, MINOR_FALSE_DETECTION, MINOR_CONVERGED, MINOR_STALLED, MINOR_ITERATION_CAP = range(5)


class MinorArgs(ctypes.Structure):
    """msn_minor_args of include/msn.h."""
    _fields_ = [("n", c_int), ("m", c_int), ("linear", c_int), ("max_scale", c_int), ("scale_adjust", c_int),
                ("minor_loop_miter", c_int), ("enforce_positivity", c_int), ("reserved", c_int),
                ("spec", c_void_p), ("rec", c_void_p), ("x", c_void_p), ("xn", c_void_p), ("r", c_void_p),
                ("rn", c_void_p), ("p", c_void_p), ("ap", c_void_p), ("tmp", c_void_p), ("planes", c_void_p),
                ("emask", c_void_p), ("esrc", c_void_p), ("ms", c_void_p), ("scal", c_void_p), ("snr2", c_void_p),
                ("neg", c_void_p), ("seg_flags", c_void_p), ("row_flags", c_void_p), ("rec_rows", c_void_p),
                ("fft_work", c_void_p),
                ("fft_work_bytes", c_size_t),
                ("iuwt_work", c_void_p),
                ("iuwt_work_bytes", c_size_t), ("red_work", c_void_p), ("red_work_bytes", c_size_t)]


class MinorResult(ctypes.Structure):
    """msn_minor_result of include/msn.h."""
    _fields_ = [("minor", c_int), ("outcome", c_int), ("positivity_runs", c_int), ("reserved", c_int),
                ("snr_current", c_double), ("snr_last", c_double)]


class MsnError(RuntimeError):
    """A libmsn entry point returned a non-zero status."""

    def __init__(self, fn, code, msg):
        super().__init__(f"{fn} failed with status {code}: {msg}")
        self.code = code


def load():
    """Load libmsn.so once and declare every entry point's signature."""
    global _LIB
    if _LIB is not None:
        return _LIB
    with _LOCK:
        if _LIB is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"libmsn.so not found at {LIB_PATH}; build it first with "
                    "`python -m pymoresane_gb300.build` (the GPU path has no CPU fallback)")
            lib = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _LIB = lib
    return _LIB


def call(name, *args):
    """Invoke entry point ``name``; raise MsnError on a non-zero status."""
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != 0:
        msg = lib.msn_last_error().decode(errors="replace")
        if rc == -1:
            raise ValueError(f"{name}: {msg}")
        raise MsnError(name, rc, msg)
    return rc


def query(name, *args):
    return getattr(load(), name)(*args)


(EV_MINIMUM_SCALE, EV_MAXIMUM_SCALE, EV_SCALE_EMPTY, EV_NO_COEFFICIENTS, EV_MINOR_DONE, EV_ALL_SCALES_POOR,
 EV_REVERTED, EV_MAJOR_DONE, EV_NO_WORK) = range(1, 10)


class Event(ctypes.Structure):
    """msn_event of include/msn.h."""
    _fields_ = [("code", c_int), ("a", c_int), ("b", c_int), ("reserved", c_int), ("v", c_double)]


class MajorRecord(ctypes.Structure):
    """msn_major_record of include/msn.h."""
    _fields_ = [("major", c_int), ("max_scale", c_int), ("scale_adjust", c_int), ("minor", c_int),
                ("outcome", c_int), ("reverted", c_int), ("snr", c_double), ("std", c_double)]


class MoresaneArgs(ctypes.Structure):
    """msn_moresane_args of include/msn.h."""
    _fields_ = ([(k, c_int) for k in ("n", "ns", "off", "scale_count", "m_sub", "m_data", "linear",
                                      "major_loop_miter", "minor_loop_miter", "enforce_positivity", "neg_comp")]
                + [("noise_rects", c_int * 8), ("reserved", c_int)]
                + [(k, c_double) for k in ("sigma_level", "tolerance", "accuracy", "flux_threshold")]
                + [("loop_gain", c_float), ("reserved_f", c_float)]
                + [(k, c_void_p) for k in ("dirty", "mask_sub", "supp_rects", "energies", "spec_sub", "spec_data",
                                           "model", "residual", "dec", "thr", "emask", "esrc", "planes", "ms", "x",
                                           "xn", "r", "rn", "p", "ap", "tmp", "rec", "masked", "sub", "conv_full",
                                           "sigma", "pmax", "scal", "snr2", "std4", "neg", "seg_flags",
                                           "row_flags", "rec_rows", "fmax", "small")]
                + [("small_bytes", c_size_t)]
                + [f for k in ("iuwt_work", "fft_work", "fft_work_full", "tool_work", "red_work")
                   for f in ((k, c_void_p), (k + "_bytes", c_size_t))])


class MoresaneResult(ctypes.Structure):
    """msn_moresane_result of include/msn.h."""
    _fields_ = [(k, c_int) for k in ("major", "complete", "have_residual", "n_records", "n_events",
                                     "events_dropped")]

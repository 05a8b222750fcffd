"""The C-ABI library loads and exports every entry point include/msn.h declares.

No compute calls are made here (no GPU is needed): only symbol presence, the
ctypes signature table and the pure-host queries.
"""
import ctypes
import os
import re

import pytest

from pymoresane_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "msn.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(msn_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_native.LIB_PATH):
        from pymoresane_gb300 import build
        build.build()
    return ctypes.CDLL(_native.LIB_PATH)


def test_header_declares_entry_points():
    fns = declared_functions()
    assert "msn_iuwt_decompose" in fns and "msn_last_error" in fns


def test_every_declared_symbol_exported(lib):
    missing = [f for f in declared_functions() if not hasattr(lib, f)]
    assert not missing, missing


def test_signature_table_matches_header():
    assert sorted(_native.SIGNATURES) == declared_functions()


def test_host_queries(lib):
    _native.load()
    assert _native.query("msn_version") >= 100
    assert _native.query("msn_iuwt_workspace_bytes", 64, 64) == 4 * 64 * 64 * 4
    assert _native.query("msn_iuwt_workspace_bytes", 0, 64) == 0
    assert _native.query("msn_last_error") == b""


def test_minor_structs_match_header(tmp_path):
    """The ctypes mirrors of the engine structs have the C layout (gcc on the header)."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    structs = {"msn_minor_args": _native.MinorArgs, "msn_minor_result": _native.MinorResult,
               "msn_moresane_args": _native.MoresaneArgs, "msn_moresane_result": _native.MoresaneResult,
               "msn_major_record": _native.MajorRecord, "msn_event": _native.Event}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "msn.h"', "int main(void) {"]
    for cname, cls in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    for line in filter(None, out):
        cname, field, value = line.split()
        cls = structs[cname]
        got = ctypes.sizeof(cls) if field == "size" else getattr(cls, field).offset
        assert got == int(value), (cname, field, got, value)


def test_native_run_log_replay(caplog):
    """The events of msn_moresane_run become the reference's log messages, in order (no GPU involved)."""
    import logging

    from pymoresane_gb300 import main as M
    N = _native
    evs = (N.Event * 9)()
    spec = [(N.EV_MINIMUM_SCALE, 0, 0, 0.0), (N.EV_MAXIMUM_SCALE, 3, 0, 0.0), (N.EV_SCALE_EMPTY, 1, 0, 0.0),
            (N.EV_MINOR_DONE, 7, N.MINOR_CONVERGED, 41.0), (N.EV_MINOR_DONE, 1, N.MINOR_FALSE_DETECTION, 45.0),
            (N.EV_REVERTED, 0, 0, 0.0), (N.EV_MAJOR_DONE, 2, 0, 0.0), (N.EV_ALL_SCALES_POOR, 0, 0, 0.0),
            (N.EV_NO_WORK, 0, 0, 0.0)]
    for e, (c, a, b, v) in zip(evs, spec):
        e.code, e.a, e.b, e.v = c, a, b, v
    with caplog.at_level(logging.INFO, logger="pymoresane_gb300.main"):
        M._replay(evs)
    assert [r.getMessage() for r in caplog.records] == [
        "Minimum scale = 0", "Maximum scale = 3", "Scale 1 is empty. Ignoring scales <= 1",
        "Model has reached <1% error - exiting minor loop.", "7 minor loop iterations performed.",
        "SNR too large on first iteration - false detection. Incrementing the minimum scale.",
        "1 minor loop iterations performed.", "Residual has worsened - reverting changes.",
        "2 major loop iterations performed.", "All scales are performing poorly - stopping.",
        "Current MORESANE iteration did no work - finished."]


def test_engine_entry_points_reject_null_engine(lib):
    """Argument checks that run before any CUDA call: a null engine is an invalid argument."""
    args, res = _native.MinorArgs(), _native.MinorResult()
    with pytest.raises(ValueError, match="null engine"):
        _native.call("msn_minor_loop", None, ctypes.byref(args), ctypes.byref(res), None, 0, None)
    margs, mres = _native.MoresaneArgs(), _native.MoresaneResult()
    with pytest.raises(ValueError, match="null engine"):
        _native.call("msn_moresane_run", None, ctypes.byref(margs), ctypes.byref(mres), None, 0, None, 0, None)
    assert _native.query("msn_minor_engine_destroy", None) == 0


def test_float4_entry_points_reject_unaligned_planes(lib):
    """Argument checks that run before any CUDA call: the plane passes read float4, so planes that
    are not 16-byte aligned are refused instead of faulting (addresses are never dereferenced)."""
    bad = ctypes.c_void_p(0x1008)   # 8 bytes past a 16-byte boundary
    good = ctypes.c_void_p(0x2000)
    with pytest.raises(ValueError, match="16-byte aligned"):
        _native.call("msn_source_extraction", bad, 2, 64, 64, ctypes.c_float(0.75), 0, good, None, good, 1 << 30,
                     None)
    with pytest.raises(ValueError, match="16-byte aligned"):
        _native.call("msn_plane_max", bad, 2, 64 * 64, 0, good, good, 1 << 20, None)
    with pytest.raises(ValueError, match="null row flags"):
        _native.call("msn_fft_convolve_rows", good, 2048, 4096, good, good, 1, None, good, 1 << 30, None)

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
    assert _native.query("msn_iuwt_workspace_bytes", 64, 64) == 2 * 64 * 64 * 4
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

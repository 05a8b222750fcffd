"""Build libmsn.so (the CUDA C-ABI library) in-tree for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled in parallel with nvcc
(``-gencode arch=compute_103a,code=sm_103a``) and linked into
``pymoresane_gb300/libmsn.so``. Object files go to ``pymoresane_gb300/_build``.
Run as ``python -m pymoresane_gb300.build`` or through ``__graft_entry__.build()``.
"""
import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build", platform.machine())
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(PKG, "libmsn.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = shutil.which("nvcc")
    if cand:
        return cand
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    return os.path.join(cuda, "bin", "nvcc")


def _cuda_lib_dir():
    nvcc = os.path.realpath(_nvcc())
    home = os.path.dirname(os.path.dirname(nvcc))
    for sub in ("lib64", "lib", os.path.join("targets", "sbsa-linux", "lib"),
                os.path.join("targets", "x86_64-linux", "lib")):
        p = os.path.join(home, sub)
        if os.path.exists(os.path.join(p, "libcudart.so")):
            return p
    return os.path.join(home, "lib64")


TWIDDLE_N = 24576  # 2^13 * 3: every supported FFT length divides it


def write_twiddles():
    """Generate msn_twiddles.inc: exp(-2 pi i k / TWIDDLE_N) rounded from float64 to float32.

    Emitted as exact hexadecimal float literals; included by csrc/fft_core.cuh.
    """
    import numpy as np

    path = os.path.join(BUILD, "msn_twiddles.inc")
    k = np.arange(TWIDDLE_N, dtype=np.float64)
    ang = -2.0 * np.pi * k / TWIDDLE_N
    c = np.cos(ang).astype(np.float32)
    s = np.sin(ang).astype(np.float32)
    lines = [f"{{{float(a).hex()}f, {float(b).hex()}f}}," for a, b in zip(c, s)]
    text = "\n".join(lines) + "\n"
    if not os.path.exists(path) or open(path).read() != text:
        with open(path, "w") as fh:
            fh.write(text)
    return path


def _flags(extra=()):
    return ["-O3", "-std=c++20", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-O3", "-I", INCLUDE, "-I", CSRC,
            "-I", BUILD, "--expt-relaxed-constexpr", *extra]


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    return res.stdout + res.stderr


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def build(verbose=False, extra_flags=(), force=False):
    """Compile every csrc/*.cu and link libmsn.so. Returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    write_twiddles()
    nvcc = _nvcc()
    srcs = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    headers += [os.path.join(BUILD, "msn_twiddles.inc")]
    newest_header = max((os.path.getmtime(h) for h in headers), default=0.0)

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        if (not force and os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src)
                and os.path.getmtime(obj) >= newest_header):
            return obj, ""
        out = _run([nvcc, "-c", src, "-o", obj, *_flags(extra_flags)])
        return obj, out

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as pool:
        results = list(pool.map(compile_one, srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, out in results:
            if out:
                sys.stdout.write(out)
    libdir = _cuda_lib_dir()
    _run([nvcc, "-shared", *ARCH, "-o", LIB, *objs, "-cudart", "shared", "-L", libdir,
          "-Xlinker", "-rpath=" + libdir])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))

"""Loader that imports the reference PyMORESANE (Python 2 sources) under Python 3.

Used ONLY by ``make_golden.py`` in a checkout that has the reference sources
available; nothing in the test suite, the package or the benchmark imports it.
The reference files are never modified: each module's source text is read,
patched in memory and executed into a fresh module object.

Patches (all syntactic, none changes the arithmetic):

* ``print "..."``  -> ``print("...")``  (pymoresane/iuwt.py:14,
  iuwt_convolution.py:15, iuwt_toolbox.py:13).
* ``pylab`` (iuwt_toolbox.py:15) and ``astropy.io.fits`` (main.py:4) are
  stubbed; neither is used on the deconvolution path.
* Python 2 integer ``/`` in index arithmetic becomes ``//``:
  main.py slice bounds (``/2``, ``/4``), iuwt_toolbox.py:29
  (``mid = in1.shape[1]/2``), iuwt_convolution.py:156 (``/4`` in pad_array)
  and iuwt_convolution.py:68 (``slice(0.5*sz, 1.5*sz)`` -> ints).
* beam_fit.py:16 ``if psf.shape>512:`` compares a tuple with an int, which
  Python 2 evaluates as True for every shape (a tuple sorts after an int) and
  Python 3 rejects; it becomes ``if True:``, and the window bounds
  ``psf.shape[i]/2-256`` use ``//`` (beam_fit.py:17), as Python 2 computed them.
* The pycuda / scikits.cuda imports fail into the reference's own
  ``except`` blocks, so only the 'ser' / 'mp' / 'cpu' paths are usable.
"""
import io
import os
import re
import sys
import types
import contextlib

# Root of a reference PyMORESANE checkout (the directory holding pymoresane/); required.
REF_ROOT = os.environ.get("PYMORESANE_REF", "")


def _patch(name, src):
    src = re.sub(r'print "([^"]*)"', r'print("\1")', src)
    if name == "main":
        src = re.sub(r"/(2|4)\b", r"//\1", src)
    if name == "iuwt_toolbox":
        src = src.replace("mid = in1.shape[1]/2", "mid = in1.shape[1]//2")
    if name == "beam_fit":
        src = src.replace("if psf.shape>512:", "if True:")
        src = re.sub(r"psf\.shape\[(\d)\]/2", r"psf.shape[\1]//2", src)
    if name == "iuwt_convolution":
        src = src.replace("slice(0.5*sz,1.5*sz)", "slice(int(0.5*sz),int(1.5*sz))")
        src = src.replace("padded_size[0]/4:3*padded_size[0]/4,padded_size[1]/4:3*padded_size[1]/4",
                          "padded_size[0]//4:3*padded_size[0]//4,padded_size[1]//4:3*padded_size[1]//4")
    return src


def load_reference():
    """Return the patched reference package ``pymoresane`` (a module object)."""
    if not REF_ROOT or not os.path.isdir(os.path.join(REF_ROOT, "pymoresane")):
        raise RuntimeError("set PYMORESANE_REF to the root of a reference PyMORESANE checkout")
    if "pymoresane" in sys.modules and getattr(sys.modules["pymoresane"], "_shimmed", False):
        return sys.modules["pymoresane"]
    pylab = types.ModuleType("pylab")
    sys.modules.setdefault("pylab", pylab)
    astropy = types.ModuleType("astropy")
    astropy_io = types.ModuleType("astropy.io")
    astropy_fits = types.ModuleType("astropy.io.fits")
    astropy.io = astropy_io
    astropy_io.fits = astropy_fits
    sys.modules.setdefault("astropy", astropy)
    sys.modules.setdefault("astropy.io", astropy_io)
    sys.modules.setdefault("astropy.io.fits", astropy_fits)

    pkg = types.ModuleType("pymoresane")
    pkg.__path__ = [os.path.join(REF_ROOT, "pymoresane")]
    pkg._shimmed = True
    sys.modules["pymoresane"] = pkg
    for name in ["iuwt", "iuwt_convolution", "iuwt_toolbox", "parser", "beam_fit", "main"]:
        path = os.path.join(REF_ROOT, "pymoresane", name + ".py")
        with open(path) as fh:
            src = _patch(name, fh.read())
        mod = types.ModuleType("pymoresane." + name)
        mod.__file__ = path
        sys.modules["pymoresane." + name] = mod
        # The reference prints a traceback when pycuda is missing; keep it quiet.
        with contextlib.redirect_stderr(io.StringIO()), contextlib.redirect_stdout(io.StringIO()):
            exec(compile(src, path, "exec"), mod.__dict__)
        setattr(pkg, name, mod)
    return pkg

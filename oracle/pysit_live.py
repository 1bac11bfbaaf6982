"""TEST INFRASTRUCTURE: import the unmodified reference package (PySIT) in-process.

Only tests/ and tests/golden/make_golden.py use this module, as a checker.  It
runs only where the reference tree exists, and the product (pysit_gb300) never
imports it.

What it does, without writing to the read-only reference tree:
  * adds the numpy aliases removed in numpy >= 1.24 that the reference still uses
    (``np.int`` etc., e.g. pysit/core/mesh_representation.py:157,177);
  * installs empty stand-ins for optional third-party modules the reference
    imports at package import time but that are absent here (matplotlib via
    pysit/util/wrappers/petsc.py:4, pyamg via pysit/util/derivatives/derivatives.py:6,
    obspy via pysit/util/io.py:3, petsc4py); mpi4py is left absent so that
    pysit/util/parallel.py:1-5 takes its own no-MPI path;
  * maps the SWIG extension
    ``pysit.solvers.constant_density_acoustic.time.scalar._constant_density_acoustic_time_scalar_cpp``
    onto the module that oracle/Makefile compiled into oracle/_ref/ from the
    reference's own solvers_wrap.cxx.
"""
from __future__ import annotations

import importlib.abc
import importlib.machinery
import os
import sys
import types
import warnings

_HERE = os.path.dirname(os.path.abspath(__file__))
_REF_DIR = os.path.join(_HERE, "_ref")


def _reference_root():
    """The reference tree: PYSIT_REFERENCE_ROOT, else the tree that oracle/Makefile built
    oracle/_ref from (recorded in _ref/reference_root.txt), else None."""
    env = os.environ.get("PYSIT_REFERENCE_ROOT")
    if env:
        return env
    try:
        with open(os.path.join(_REF_DIR, "reference_root.txt")) as f:
            return f.read().strip() or None
    except OSError:
        return None


REFERENCE_ROOT = _reference_root() or ""
_SWIG_FULLNAME = ("pysit.solvers.constant_density_acoustic.time.scalar."
                  "_constant_density_acoustic_time_scalar_cpp")


class _SwigFinder(importlib.abc.MetaPathFinder):
    def find_spec(self, fullname, path=None, target=None):
        if fullname != _SWIG_FULLNAME:
            return None
        suffix = importlib.machinery.EXTENSION_SUFFIXES[0]
        so = os.path.join(_REF_DIR, "_constant_density_acoustic_time_scalar_cpp" + suffix)
        if not os.path.exists(so):
            return None
        loader = importlib.machinery.ExtensionFileLoader(fullname, so)
        return importlib.machinery.ModuleSpec(fullname, loader, origin=so)


def _absent(*args, **kwargs):
    raise RuntimeError("optional dependency is absent in this environment")


def _stub_getattr(attr):
    # dunder names (__file__, __spec__ ...) stay absent, so that tools walking
    # sys.modules (inspect.getmodule) see an ordinary module without a file
    if attr.startswith("__") and attr.endswith("__"):
        raise AttributeError(attr)
    return _absent


def _stub(name):
    if name in sys.modules:
        return sys.modules[name]
    mod = types.ModuleType(name)
    mod.__path__ = []  # behave as a package so submodule stubs can hang off it
    # any attribute (e.g. pyamg.gallery.stencil_grid) resolves to a callable that
    # raises only if the reference actually uses it on the path under test
    mod.__getattr__ = _stub_getattr
    sys.modules[name] = mod
    parent, _, child = name.rpartition(".")
    if parent and parent in sys.modules:
        setattr(sys.modules[parent], child, mod)
    return mod


def available() -> bool:
    """True when the reference tree and the compiled SWIG module are both present."""
    suffix = importlib.machinery.EXTENSION_SUFFIXES[0]
    so = os.path.join(_REF_DIR, "_constant_density_acoustic_time_scalar_cpp" + suffix)
    return os.path.isdir(os.path.join(REFERENCE_ROOT, "pysit")) and os.path.exists(so)


def import_pysit():
    """Import and return the reference ``pysit`` package (raises ImportError if absent)."""
    if "pysit" in sys.modules:
        return sys.modules["pysit"]
    if not available():
        raise ImportError("reference pysit tree or its compiled SWIG module is absent")
    import numpy as np
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        for alias, typ in (("int", int), ("float", float), ("complex", complex),
                           ("object", object), ("bool", bool)):
            if alias not in np.__dict__:
                setattr(np, alias, typ)
    for name in ("matplotlib", "matplotlib.pyplot", "matplotlib.cm", "matplotlib.colors",
                 "matplotlib.animation", "matplotlib.gridspec", "matplotlib.ticker",
                 "matplotlib.sphinxext", "matplotlib.sphinxext.plot_directive",
                 "obspy", "obspy.segy", "obspy.segy.core", "obspy.io", "obspy.io.segy",
                 "obspy.io.segy.core", "pyamg", "pyamg.gallery", "pyamg.krylov",
                 "petsc4py", "petsc4py.PETSc"):
        _stub(name)
    if not any(isinstance(f, _SwigFinder) for f in sys.meta_path):
        sys.meta_path.insert(0, _SwigFinder())
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(0, REFERENCE_ROOT)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        import pysit  # noqa: F401
    return sys.modules["pysit"]

"""Import the reference (Python) solver unchanged, behind harness-side shims.

Only the fixture generator in this folder uses this module, and only on a
machine where the reference checkout is present (``REF_ROOT`` below).  Nothing
in the package, the GPU tests, ``smoke()`` or ``bench.py`` imports it.

Shims (all installed in ``sys.modules`` before the reference is imported; the
reference tree itself is never modified):

* ``cupy``   -- a stub whose ``asarray`` is ``numpy.asarray`` (the reference
  copies its tables to the GPU at construction time,
  ``src/collision/inelastic_collisions.py:125-137``).
* ``pyfftw`` -- ``builders.fftn/ifftn`` mapped onto ``scipy.fft.fftn/ifftn``
  (same convention: unnormalised forward, 1/N inverse), used by
  ``src/collision/inelastic_collisions.py:139-162``.
* ``np.float = float`` -- removed from NumPy >= 1.24, used by
  ``src/collision/spherical_design/__init__.py:39-40``.
* ``tqdm.tnrange = range`` -- the notebook progress bar breaks under current
  tqdm (``src/solver.py:131``, ``src/boltzmann.py:124-149``).
* ``matplotlib`` -- an empty stub; ``src/utility.py:5`` imports pyplot for
  plotting helpers that the iterative solver (``src/iter_solver.py:6``) does
  not call.
"""
import os
import sys
import types

import numpy as np
import scipy.fft

# the reference checkout: required, no default (only the fixture scripts need it)
REF_ROOT = os.environ.get("PII_REFERENCE_ROOT", "")


def _install_shims(workers=None):
    workers = workers or os.cpu_count()
    if not hasattr(np, "float"):
        np.float = float  # noqa: NPY001 - the reference uses the removed alias

    cp = types.ModuleType("cupy")
    cp.asarray = np.asarray
    sys.modules["cupy"] = cp

    pyfftw = types.ModuleType("pyfftw")

    class _Config:
        NUM_THREADS = 1
        PLANNER_EFFORT = "FFTW_ESTIMATE"

    pyfftw.config = _Config()

    def empty_aligned(shape, dtype="complex128"):
        return np.empty(shape, dtype=dtype)

    pyfftw.empty_aligned = empty_aligned

    builders = types.ModuleType("pyfftw.builders")

    def fftn(arr, axes=None):
        return lambda x: scipy.fft.fftn(x, axes=axes, workers=workers)

    def ifftn(arr, axes=None):
        return lambda x: scipy.fft.ifftn(x, axes=axes, workers=workers)

    builders.fftn = fftn
    builders.ifftn = ifftn
    pyfftw.builders = builders
    sys.modules["pyfftw"] = pyfftw
    sys.modules["pyfftw.builders"] = builders

    import tqdm

    tqdm.tnrange = lambda n, *a, **k: range(n)

    try:
        import matplotlib  # noqa: F401
    except ImportError:
        mpl = types.ModuleType("matplotlib")
        plt = types.ModuleType("matplotlib.pyplot")
        mpl.pyplot = plt
        sys.modules["matplotlib"] = mpl
        sys.modules["matplotlib.pyplot"] = plt


def load_reference(workers=None):
    """Return a namespace with the reference modules used by the fixtures."""
    if not REF_ROOT:
        raise RuntimeError("set PII_REFERENCE_ROOT to the reference checkout (the directory holding src/)")
    if not os.path.isdir(os.path.join(REF_ROOT, "src")):
        raise RuntimeError(f"reference checkout not found under PII_REFERENCE_ROOT={REF_ROOT}")
    _install_shims(workers)
    if REF_ROOT not in sys.path:
        sys.path.insert(0, REF_ROOT)
    import importlib

    ns = types.SimpleNamespace()
    ns.spectral_mesh = importlib.import_module("src.collision.spectral_mesh")
    ns.inelastic = importlib.import_module("src.collision.inelastic_collisions")
    ns.spherical_design = importlib.import_module("src.collision.spherical_design")
    ns.boltzmann = importlib.import_module("src.boltzmann")
    ns.solver = importlib.import_module("src.solver")
    ns.advection_1D = importlib.import_module("src.riemann.advection_1D")
    ns.tvd = importlib.import_module("src.limiters.tvd")
    ns.iter_solver = importlib.import_module("src.iter_solver")
    return ns

"""Import name for the package directory ``proj-int-inelastic_gb300/``.

The directory name is not a Python identifier, so ``import
proj_int_inelastic_gb300`` loads it from there through this module.
"""
import importlib.util
import os
import sys

_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "proj-int-inelastic_gb300")
_spec = importlib.util.spec_from_file_location(__name__, os.path.join(_DIR, "__init__.py"),
                                               submodule_search_locations=[_DIR])
_mod = importlib.util.module_from_spec(_spec)
sys.modules[__name__] = _mod
_spec.loader.exec_module(_mod)

"""Import name for the package in ``sci-algorithms_gb300/``.

The package directory's name contains a hyphen, which ``import`` cannot
spell; this module loads that directory as the package
``sci_algorithms_gb300`` and replaces itself with it, so
``import sci_algorithms_gb300`` works from the repository root.
"""
import importlib.util
import os
import sys

_PKG_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "sci-algorithms_gb300")
_spec = importlib.util.spec_from_file_location(
    __name__, os.path.join(_PKG_DIR, "__init__.py"),
    submodule_search_locations=[_PKG_DIR])
_module = importlib.util.module_from_spec(_spec)
sys.modules[__name__] = _module
_spec.loader.exec_module(_module)

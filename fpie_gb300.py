"""Import name for the package directory ``fast-poisson-image-editing_gb300``.

A directory whose name holds hyphens cannot be imported with ``import``; this
module loads that directory as the package ``fpie_gb300`` and puts it in
``sys.modules`` in its own place, so ``import fpie_gb300`` and
``from fpie_gb300.process import GridProcessor`` work from the repository root.
"""

import importlib.util
import pathlib
import sys

_PKG_DIR = pathlib.Path(__file__).resolve().parent / "fast-poisson-image-editing_gb300"
_spec = importlib.util.spec_from_file_location(
    __name__, _PKG_DIR / "__init__.py", submodule_search_locations=[str(_PKG_DIR)]
)
_pkg = importlib.util.module_from_spec(_spec)
sys.modules[__name__] = _pkg
_spec.loader.exec_module(_pkg)

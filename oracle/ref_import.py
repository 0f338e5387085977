"""ORACLE (test infrastructure only): import the reference fpie for checking.

Loads the reference's pure-Python package from its source tree (the
``root`` argument, else $FPIE_REFERENCE) as the module ``fpie``, with the
compiled reference solver modules that oracle/build_ref.sh puts in
oracle/_ref/fpie on its search path.  Returns None when no tree is given or
it is absent, so callers skip.
"""

from __future__ import annotations

import importlib.util
import os
import pathlib
import sys

_HERE = pathlib.Path(__file__).resolve().parent


def import_reference(root=None):
    """Return the reference ``fpie.process`` module, or None if unavailable."""
    root = root or os.environ.get("FPIE_REFERENCE")
    if not root:
        return None
    pkg = pathlib.Path(root) / "fpie"
    if not (pkg / "process.py").exists():
        return None
    if "fpie" not in sys.modules:
        spec = importlib.util.spec_from_file_location(
            "fpie", pkg / "__init__.py",
            submodule_search_locations=[str(pkg), str(_HERE / "_ref" / "fpie")],
        )
        mod = importlib.util.module_from_spec(spec)
        sys.modules["fpie"] = mod
        spec.loader.exec_module(mod)
    import fpie.process  # noqa: E402

    return fpie.process

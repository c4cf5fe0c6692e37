"""sys.path helper for importing the compiled reference CyLag (test oracle).

Test infrastructure only.  ``use_reference()`` puts ``oracle/_ref`` and the
import stubs on ``sys.path`` and returns the imported ``cylag`` package, or
raises ImportError if the reference has not been built (``oracle/build_ref.py``).
"""
from __future__ import annotations

import importlib
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def available() -> bool:
    pkg = HERE / "_ref" / "cylag" / "core"
    return pkg.is_dir() and any(pkg.glob("solver*.so"))


def use_reference():
    if not available():
        raise ImportError("reference CyLag not built (run oracle/build_ref.py)")
    for p in (str(HERE / "ref_stubs"), str(HERE / "_ref")):
        if p not in sys.path:
            sys.path.insert(0, p)
    return importlib.import_module("cylag")

"""Import the reference package with its compiled modules taken from ``oracle/_ref``.

Test infrastructure only.  The reference's pure-Python modules are loaded from the
reference tree where they lie (``$RBG_REFERENCE_ROOT``, default the mounted reference);
its extension modules, which :mod:`oracle.ref_build` compiled from that tree, are loaded
from ``oracle/_ref/redblackgraph``.  Used to pin the oracle and to generate golden
fixtures in a container that has the reference; never on the product path.
"""
from __future__ import annotations

import importlib.abc
import importlib.machinery
import importlib.util
import os
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_ROOT = Path(os.environ.get("RBG_REFERENCE_ROOT", "/root/reference"))
BUILT = HERE / "_ref" / "redblackgraph"


class _RefExtFinder(importlib.abc.MetaPathFinder):
    """Resolve ``redblackgraph.<...>._ext`` to the module compiled into ``oracle/_ref``."""

    def find_spec(self, fullname, path=None, target=None):
        if not fullname.startswith("redblackgraph."):
            return None
        parts = fullname.split(".")
        if not parts[-1].startswith("_") or parts[-1] == "__init__":
            return None
        rel = Path(*parts[1:-1])
        for suffix in importlib.machinery.EXTENSION_SUFFIXES:
            cand = BUILT / rel / (parts[-1] + suffix)
            if cand.exists():
                loader = importlib.machinery.ExtensionFileLoader(fullname, str(cand))
                return importlib.util.spec_from_file_location(fullname, str(cand), loader=loader)
        return None


def available() -> bool:
    return (REF_ROOT / "redblackgraph").is_dir() and (HERE / "_ref" / ".built").exists()


def load():
    """Return the reference ``redblackgraph`` package (raises if it is not available)."""
    if not available():
        raise ImportError("reference tree or its compiled modules are not available")
    if not any(isinstance(f, _RefExtFinder) for f in sys.meta_path):
        sys.meta_path.insert(0, _RefExtFinder())
    if str(REF_ROOT) not in sys.path:
        sys.path.insert(0, str(REF_ROOT))
    import redblackgraph  # noqa: F401  (the reference package)
    return redblackgraph

"""Load the reference pyfds package from its source tree for validation only.

This module is test infrastructure: it is imported by the golden-vector generator
(``tests/golden/make_golden.py``) and by CPU tests that cross-check the oracle
against the live reference where the reference source tree is available. Nothing
in the product package imports it.

Two harness-side shims make the unmodified reference importable here:

1. ``pyfds/__init__.py:6`` star-imports ``gfx``, which imports matplotlib
   (``pyfds/gfx.py:1-2``). Matplotlib is not installed, so empty stub modules
   ``matplotlib``, ``matplotlib.pyplot``, ``matplotlib.patches`` and
   ``matplotlib.animation`` are registered in ``sys.modules`` first.
2. ``Dimension.get_index`` (``pyfds/fields.py:557-571``) ends in ``int(index)``
   on a one-element 1-D array, which numpy 2 rejects. The shim replaces the method
   with one that performs the same snap search and returns ``int(index[0])``.

The reference source itself is never modified.
"""
import os
import sys
import types

import numpy as np

# The reference tree is found through PYFDS_REFERENCE_ROOT, else as a directory
# named ``reference`` beside this repository's checkout.
_SIBLING = os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(
    os.path.abspath(__file__)))), "reference")
DEFAULT_REFERENCE_ROOT = os.environ.get("PYFDS_REFERENCE_ROOT", _SIBLING)


def reference_available(root=DEFAULT_REFERENCE_ROOT):
    return os.path.isfile(os.path.join(root, "pyfds", "fields.py"))


def _install_matplotlib_stub():
    if "matplotlib" in sys.modules:
        return
    mpl = types.ModuleType("matplotlib")
    mpl.__path__ = []
    for sub in ("pyplot", "patches", "animation", "colors", "cm"):
        m = types.ModuleType("matplotlib." + sub)
        sys.modules["matplotlib." + sub] = m
        setattr(mpl, sub, m)
    mpl.use = lambda *a, **k: None
    sys.modules["matplotlib"] = mpl


def load_reference(root=DEFAULT_REFERENCE_ROOT):
    """Import and return the reference ``pyfds`` package with the two shims applied."""
    if "pyfds" in sys.modules and getattr(sys.modules["pyfds"], "_oracle_shimmed", False):
        return sys.modules["pyfds"]
    if not reference_available(root):
        raise ImportError("reference pyfds source tree not found at %r" % root)
    _install_matplotlib_stub()
    # the reference writes no bytecode into its read-only tree
    sys.dont_write_bytecode = True
    if root not in sys.path:
        sys.path.insert(0, root)
    import pyfds  # noqa: E402
    import pyfds.fields as ref_fields

    def get_index(self, value):
        index, = np.where(np.abs(self.vector - value) <= self.snap_radius)
        assert len(index) < 2, "Multiple points found within snap radius of given value."
        assert len(index) > 0, "No point found within snap radius of given value."
        return int(index[0])

    ref_fields.Dimension.get_index = get_index
    pyfds._oracle_shimmed = True
    return pyfds

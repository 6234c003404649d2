"""Digest of a scenario spec (shared by the golden generator and the tests).

Sequences of numbers and arrays hash by their float64 values, so a spec whose
lists were replaced by equal arrays (``golden_inputs.apply_inputs``) keeps its digest.
"""
import hashlib

import numpy as np


def spec_digest(spec):
    """Stable digest of a scenario spec's numbers (detects generator drift)."""
    h = hashlib.sha256()

    def numeric_seq(x):
        return isinstance(x, np.ndarray) or (
            isinstance(x, (list, tuple)) and all(
                isinstance(v, (int, float, np.integer, np.floating)) and not isinstance(v, bool)
                for v in x))

    def feed(x):
        if isinstance(x, dict):
            for k in sorted(x):
                h.update(str(k).encode())
                feed(x[k])
        elif numeric_seq(x):
            h.update(b"A")
            h.update(np.ascontiguousarray(np.asarray(x, dtype=np.float64)).tobytes())
        elif isinstance(x, (list, tuple)):
            h.update(b"[")
            for v in x:
                feed(v)
            h.update(b"]")
        elif x is None:
            h.update(b"None")
        elif isinstance(x, bool):
            h.update(repr(x).encode())
        elif isinstance(x, (int, float, np.integer, np.floating)):
            h.update(repr(float(x)).encode())
        else:
            h.update(repr(x).encode())
    feed(spec)
    return h.hexdigest()[:16]

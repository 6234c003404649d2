"""Digest of a scenario spec (shared by the golden generator and the tests)."""
import hashlib

import numpy as np


def spec_digest(spec):
    """Stable digest of a scenario spec's numbers (detects generator drift)."""
    h = hashlib.sha256()

    def feed(x):
        if isinstance(x, dict):
            for k in sorted(x):
                h.update(str(k).encode())
                feed(x[k])
        elif isinstance(x, (list, tuple)):
            h.update(b"[")
            for v in x:
                feed(v)
            h.update(b"]")
        elif isinstance(x, np.ndarray):
            h.update(np.ascontiguousarray(x, dtype=np.float64).tobytes())
        elif x is None:
            h.update(b"None")
        else:
            h.update(repr(float(x) if isinstance(x, (int, float, np.floating, np.integer))
                          and not isinstance(x, bool) else x).encode())
    feed(spec)
    return h.hexdigest()[:16]

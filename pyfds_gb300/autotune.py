"""Autotuner for the batched step: tile shape, pipeline depth and temporal blocking
(one or two steps per tile and launch) per size class.

Candidates are timed on the real batch for a few steps (CUDA events on the
launching stream, warm-up first); the winner is cached in a JSON file keyed by
field class, precision and size class (PYFDS_GB300_AUTOTUNE overrides the path).
The fields' state is restored after the trials.
"""
import json
import math
import os

from . import _capi
from ._engine import require_cuda

# (tile, stages): one step per tile and launch (1), the persistent two-stage pipeline
# (2), two steps per tile and launch (3: temporal blocking)
CANDIDATES = [((64, 16), 1), ((32, 32), 1), ((128, 8), 1), ((64, 32), 1), ((128, 16), 1),
              ((64, 16), 2), ((32, 32), 2), ((128, 8), 2),
              ((64, 16), 3), ((64, 12), 3), ((32, 32), 3), ((64, 8), 3)]


def cache_path():
    return os.environ.get("PYFDS_GB300_AUTOTUNE",
                          os.path.join(os.path.expanduser("~"), ".cache", "pyfds_gb300",
                                       "autotune.json"))


def _load():
    try:
        with open(cache_path()) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _save(cache):
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as fh:
            json.dump(cache, fh, indent=1, sort_keys=True)
    except OSError:
        pass


def size_key(fields):
    """Field class, precision and a coarse size class of a batch."""
    cells = sum(f.num_points for f in fields)
    mean = cells / max(len(fields), 1)
    return "%s/%s/n%d/mean2^%d" % (type(fields[0]).__name__, fields[0].precision,
                                   int(round(math.log2(max(len(fields), 1)))),
                                   int(round(math.log2(max(mean, 1)))))


def autotune_batch(fields, steps=20, candidates=CANDIDATES, force=False, verbose=False):
    """Pick (tile, stages) for ``simulate_batch(fields, ...)``; returns the choice and
    sets it on every field."""
    from .batch import BatchRunner
    torch = require_cuda()
    key = size_key(fields)
    cache = _load()
    if key in cache and not force:
        tile, stages = tuple(cache[key]["tile"]), int(cache[key]["stages"])
    else:
        steps += (-steps) % 4  # even launches for one or two steps per launch: the
        # ping-pong buffers end where they started
        saved_tile = [getattr(f, "tile", None) for f in fields]
        first = BatchRunner(fields, steps)  # uploads the host state
        snapshot = [{n: b[0].clone() for n, b in f._engine().buffers.items()} for f in fields]
        del first
        results = []
        for tile, stages in candidates:
            try:
                r = BatchRunner(fields, steps, tile=tile, stages=stages)
                r.launch()
                torch.cuda.synchronize()
                s = torch.cuda.current_stream()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(s)
                for _ in range(2):
                    r.launch()
                e1.record(s)
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1) / 2
                results.append((ms, tile, stages))
                if verbose:
                    print("autotune %s tile %s stages %d: %.3f ms" % (key, tile, stages, ms))
            except _capi.FdsError:
                continue
        for f, snap in zip(fields, snapshot):
            for n, t in snap.items():
                f._engine().buffers[n][0].copy_(t)
        for f, t in zip(fields, saved_tile):
            f.tile = t
        if not results:
            raise RuntimeError("no candidate tile shape runs this batch")
        ms, tile, stages = min(results)
        cache[key] = {"tile": list(tile), "stages": stages, "ms": ms, "steps": steps,
                      "trials": [[list(t), s, m] for m, t, s in results]}
        _save(cache)
    for f in fields:
        f.tile = tuple(tile)
        f.stages = stages
    return tuple(tile), stages

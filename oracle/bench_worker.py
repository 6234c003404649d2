"""CPU-baseline worker: runs the oracle's time step on one replica of a workload.

TEST INFRASTRUCTURE: used only by bench.py's CPU-baseline leg and its
``--impl reference`` arm, through a ``spawn`` process pool (one replica per
process; the oracle, like the reference's scipy path, is single-threaded).

The operators run as ``scipy.sparse.dia_matrix`` products built from the oracle's
diagonals: the reference's own call (``dia_matrix.dot``) with the same diagonals in
the same order, so the timed CPU work is the reference's. The oracle's numpy
restatement of that product (``dia_matvec``) computes the same values but makes a
temporary per diagonal, and ran 1.7x slower per step than the reference on the
2048^2 workload.
"""
import os
import time

import numpy as np

from . import fds_oracle as O

_W = {}


def _is_dia(v):
    return (isinstance(v, list) and len(v) > 0
            and all(isinstance(t, tuple) and len(t) == 2 for t in v))


def scipy_operators(ops):
    """A copy of ``ops`` with every DIA operator as a scipy dia_matrix (same diagonals,
    same storage order)."""
    import scipy.sparse as sp
    n = int(ops["n"])
    out = dict(ops)
    for k, v in ops.items():
        if _is_dia(v):
            offsets = np.array([int(off) for off, _ in v])
            data = np.vstack([np.asarray(d, dtype=np.float64) for _, d in v])
            out[k] = sp.dia_matrix((data, offsets), shape=(n, n))
    return out


def _dot(a, x):
    return a.dot(x)


def setup(workload, kwargs):
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    from pyfds_gb300 import workloads
    spec = getattr(workloads, workload)(**kwargs)
    ops = scipy_operators(O.assemble(spec))
    n = ops["n"]
    state = {c: np.zeros(n) for c in O.components_of(spec["kind"])}
    for c, v in (spec.get("init") or {}).items():
        state[c] = np.array(v, dtype=np.float64)
    _W.update(spec=spec, ops=ops, state=state, step=0)
    return os.getpid()


def run(nsteps):
    """Advance this replica by nsteps oracle steps; returns the elapsed seconds."""
    spec, ops, state = _W["spec"], _W["ops"], _W["state"]
    outputs = spec.get("outputs") or {}
    bounds = spec.get("bounds") or {}
    signals = {c: [[[] for _ in idx] for idx in outputs.get(c, [])]
               for c in O.components_of(spec["kind"])}
    kind = spec["kind"]
    periods = O.flow_periods(spec) if kind == "AcousticFlow2D" else None
    step_kind = "Acoustic2D" if periods is not None else kind
    t0 = time.perf_counter()
    for _ in range(nsteps):
        O.sim_step(step_kind, ops, state, bounds, outputs, signals, _W["step"], dt=spec["dt"],
                   matvec=_dot, inplace=True)
        if periods is not None:
            O.apply_flow(state, periods, _W["step"], ops["nx"])
        _W["step"] += 1
    return time.perf_counter() - t0


def cells():
    return int(_W["ops"]["n"])


_BATCH = {}


def run_batch_instance(args):
    """(cells, seconds) of ``nsteps`` oracle steps on instance k of a batch workload."""
    workload, kwargs, k, nsteps = args
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    from pyfds_gb300 import workloads
    if k not in _BATCH:
        spec = getattr(workloads, workload)(**kwargs)[k]
        ops = scipy_operators(O.assemble(spec))
        _BATCH[k] = (spec, ops, {c: np.zeros(ops["n"]) for c in O.components_of(spec["kind"])})
    spec, ops, state = _BATCH[k]
    outputs = spec.get("outputs") or {}
    signals = {c: [[[] for _ in idx] for idx in outputs.get(c, [])] for c in state}
    t0 = time.perf_counter()
    for s in range(nsteps):
        O.sim_step(spec["kind"], ops, state, spec.get("bounds") or {}, outputs, signals, s,
                   dt=spec["dt"], matvec=_dot, inplace=True)
    return int(ops["n"]), time.perf_counter() - t0

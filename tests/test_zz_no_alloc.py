"""The allocation-free batched entry point (fds_stag_batch_run_static).

It exists for callers that cannot allocate device memory themselves, such as a C
or Fortran host code that links libfdsgpu.so directly without a device
allocator: its workspace is a fixed array built into the library. This file runs
last (pytest collects it after the others) and must also pass on its own in a
fresh process. Both entry points are driven through the C ABI on the same
fields, twice in a row, and must agree within the float64 bar of the other
parity tests (relative L2 1e-12; in fact bit for bit, the kernels are the same);
after the two calls the allocation-free run is also held to the oracle's
trajectory at that bar. A call made while its stream is being captured into a
CUDA graph is rejected (the call copies its descriptors from host memory).
"""
import ctypes as C

import numpy as np
import pytest

from oracle import fds_oracle as O
from oracle import scenarios as S
from helpers import build_field, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _fields():
    sizes = [(204, 77), (130, 61), (64, 96)]
    specs = [S.random_scenario(300 + k, "Acoustic2D", nx, ny, steps=24, mu=False)
             for k, (nx, ny) in enumerate(sizes)]
    fields = [build_field(s, tile=(64, 16)) for s in specs]
    for f in fields:
        f.assemble_matrices()  # what simulate() does first
    return specs, fields


def _structs(fields, plans):
    from pyfds_gb300 import _capi
    n = len(fields)
    probs = (_capi.FdsStagProblem * n)(*[p["prob"] for p in plans])
    tables = (_capi.FdsStagTables * n)(*[p["tstruct"] for p in plans])
    states = (_capi.FdsStagState * n)()
    for i, f in enumerate(fields):
        for k, name in enumerate(f._stag_components):
            cur, nxt = f._engine().buffers[name]
            states[i].cur[k] = cur.data_ptr()
            states[i].nxt[k] = nxt.data_ptr()
    return probs, states, tables


def _run(fields, step0, nsteps, static):
    """One batched call through the C ABI; returns the potentials afterwards."""
    import torch
    from pyfds_gb300 import _capi
    lib = _capi.load()
    plans = [f._engine().prepare(step0, nsteps, batched=True) for f in fields]
    probs, states, tables = _structs(fields, plans)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if static:
        code = lib.fds_stag_batch_run_static(probs, states, tables, len(fields), step0, nsteps, 1,
                                             stream)
    else:
        total = sum(p["geo"].ntiles for p in plans)
        ws = torch.empty(lib.fds_stag_batch_workspace_bytes(len(fields), total),
                         dtype=torch.uint8, device="cuda")
        code = lib.fds_stag_batch_run(probs, states, tables, len(fields),
                                      C.c_void_p(ws.data_ptr()), ws.numel(), step0, nsteps, 1,
                                      _capi.BATCH_UPLOAD | _capi.BATCH_LAUNCH, stream)
    _capi.check(code)
    torch.cuda.synchronize()
    out = []
    for i, f in enumerate(fields):
        eng = f._engine()
        for k, name in enumerate(f._stag_components):
            bufs = eng.buffers[name]
            if states[i].cur[k] != bufs[0].data_ptr():
                bufs.reverse()
            getattr(f, name)._where = "device"
        out.append(eng.buffers["pressure"][0].double().cpu().numpy().copy())
    return out


def test_static_scratch_matches_workspace_entry_point(gpu):
    specs, ref_fields = _fields()
    _, st_fields = _fields()
    for step0, n in ((0, 11), (11, 13)):  # two calls in a row
        a = _run(ref_fields, step0, n, static=False)
        b = _run(st_fields, step0, n, static=True)
        for x, y in zip(a, b):
            assert rel_l2(y, x) <= TOL
            assert np.array_equal(x, y)
    # the allocation-free trajectory against the oracle's, 24 steps
    for spec, y in zip(specs, b):
        st_o, _ = O.simulate(spec, 24)
        assert rel_l2(y, st_o["pressure"]) <= TOL


def test_static_scratch_rejects_a_capturing_stream(gpu):
    import torch
    from pyfds_gb300 import _capi
    lib = _capi.load()
    _, fields = _fields()
    plans = [f._engine().prepare(0, 1, batched=True) for f in fields]
    probs, states, tables = _structs(fields, plans)
    side = torch.cuda.Stream()
    scratch = torch.zeros(16, device="cuda")
    graph = torch.cuda.CUDAGraph()
    codes = []
    with torch.cuda.stream(side):
        with torch.cuda.graph(graph, stream=side):
            scratch.add_(1.0)  # the capture holds one node
            codes.append(lib.fds_stag_batch_run_static(
                probs, states, tables, len(fields), 0, 1, 1,
                C.c_void_p(side.cuda_stream)))
    torch.cuda.synchronize()
    assert codes == [_capi.FDS_E_ARG]
    assert "captur" in _capi.last_error()


def test_static_scratch_rejects_oversized_batches(gpu):
    from pyfds_gb300 import _capi
    lib = _capi.load()
    specs, fields = _fields()
    plans = [f._engine().prepare(0, 1, batched=True) for f in fields]
    probs, states, tables = _structs(fields, plans)
    # a batch far larger than the built-in scratch (repeat one field many times)
    n = 4000
    big_p = (_capi.FdsStagProblem * n)(*([plans[0]["prob"]] * n))
    big_s = (_capi.FdsStagState * n)(*([states[0]] * n))
    big_t = (_capi.FdsStagTables * n)(*([tables[0]] * n))
    code = lib.fds_stag_batch_run_static(big_p, big_s, big_t, n, 0, 1, 1, None)
    assert code == _capi.FDS_E_SIZE
    assert "scratch" in _capi.last_error()

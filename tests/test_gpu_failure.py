"""Failure detection on the GPU, without a fault or a hang.

* Bounded waits: fds_selftest_bounded_wait runs the stepping kernels' wait helpers
  (mbar_wait on an mbarrier that no copy targets, wait_counters on a tile-row
  counter that nothing increments) with a small poll limit. The waits give up, the
  kernel ORs FDS_STATUS_TMA_TIMEOUT into the status word and returns; the engine's
  finish() turns that word into FdsError, and the context stays usable.
* Divergence: a time step above the explicit scheme's stability limit (the
  reference's is_stable(), pyfds/acoustics.py:54-63, returns False) makes the field
  blow up; the kernels flag the non-finite potential on the call's last step and
  simulate() raises FieldDiverged (a FloatingPointError) after recording the
  outputs and advancing the step, or warns, as set_nonfinite_action chooses.
"""
import ctypes as C
import warnings

import numpy as np
import pytest

import pyfds_gb300 as fds
from oracle import scenarios as S
from helpers import build_field
from pyfds_gb300 import _capi, _engine

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [0, 1])
def test_bounded_wait_gives_up_and_the_host_raises(gpu, mode):
    import torch
    lib = _capi.load()
    spec = S.random_scenario(51, "Acoustic2D", 64, 40, steps=4, mu=False)
    f = build_field(spec)
    f.simulate(2)
    eng = f._engine()
    counter = torch.zeros(4, dtype=torch.int32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _capi.check(lib.fds_selftest_bounded_wait(mode, C.c_void_p(eng.status.data_ptr()),
                                              C.c_void_p(counter.data_ptr()), 2000, stream))
    torch.cuda.synchronize()
    assert int(eng.status.item()) & _capi.STATUS_TMA_TIMEOUT
    with pytest.raises(_capi.FdsError, match="bounded wait"):
        eng.finish(eng._last)
    # the status word was cleared and the context still steps correctly
    assert int(eng.status.item()) == 0
    f2 = build_field(spec)
    f2.simulate(4)
    f.simulate(2)
    for c in ("pressure", "velocity_x", "velocity_y"):
        assert np.array_equal(getattr(f, c).values, getattr(f2, c).values)


def _unstable(kind="Acoustic2D", nx=64, ny=64, steps=400):
    spec = S.random_scenario(52, kind, nx, ny, steps=steps, mu=False)
    spec["dt"] = spec["dt"] * 40.0  # far beyond the CFL limit
    return spec


@pytest.mark.parametrize("precision,stages", [("f64", 0), ("f64", 4), ("f32", 0), ("dw", 0),
                                              ("f64", 3)])
def test_diverging_field_raises(gpu, precision, stages):
    spec = _unstable()
    f = build_field(spec, precision=precision)
    assert not f.is_stable()
    f.stages = stages
    with pytest.raises(_capi.FieldDiverged) as e:
        f.simulate(spec["steps"])
    assert isinstance(e.value, FloatingPointError)
    assert f.step == spec["steps"]  # the call completed; the step counter advanced
    assert not np.all(np.isfinite(f.pressure.values))


def test_stable_field_does_not_raise(gpu):
    spec = S.random_scenario(53, "Acoustic2D", 64, 64, steps=50, mu=False)
    f = build_field(spec)
    assert f.is_stable()
    f.simulate(50)
    assert np.all(np.isfinite(f.pressure.values))


def test_diverging_field_warns_when_asked(gpu):
    spec = _unstable(kind="Thermal2D", steps=1000)  # slower growth than the acoustic case
    f = build_field(spec)
    _engine.set_nonfinite_action("warn")
    try:
        with warnings.catch_warnings(record=True) as w:
            warnings.simplefilter("always")
            f.simulate(spec["steps"])
        assert any(issubclass(x.category, RuntimeWarning) and "diverged" in str(x.message)
                   for x in w)
        _engine.set_nonfinite_action("ignore")
        f.simulate(3)  # no warning, no exception
    finally:
        _engine.set_nonfinite_action("raise")
    assert f.step == spec["steps"] + 3
    with pytest.raises(ValueError):
        _engine.set_nonfinite_action("abort")


def test_diverging_instance_of_a_batch_raises(gpu):
    from pyfds_gb300.batch import simulate_batch
    good = build_field(S.random_scenario(54, "Acoustic2D", 96, 64, steps=200, mu=False))
    bad = build_field(_unstable(nx=96, steps=200))
    with pytest.raises(_capi.FieldDiverged):
        simulate_batch([good, bad], 200)
    assert good.step == bad.step == 200
    assert np.all(np.isfinite(good.pressure.values))

"""The product path has no CPU fallback: without a visible GPU, or without the built
library, every entry that would step a field raises instead of computing on the
host. Runs on CPU (the GPU case is skipped where a GPU is visible)."""
import numpy as np
import pytest
import torch

from oracle import scenarios as S
from pyfds_gb300 import _capi, batch, workloads
from pyfds_gb300.fields import FieldComponent


def test_missing_library_raises(tmp_path, monkeypatch):
    monkeypatch.setattr(_capi, "_lib", None)
    with pytest.raises(RuntimeError, match="not built"):
        _capi.load(str(tmp_path / "libfdsgpu.so"))


needs_no_gpu = pytest.mark.skipif(torch.cuda.is_available(),
                                  reason="checks the behaviour without a visible GPU")


@needs_no_gpu
@pytest.mark.parametrize("kind", ["Acoustic1D", "Acoustic2D", "Acoustic3DAxi", "Thermal2D"])
def test_simulate_without_gpu_raises(kind):
    nx, ny = (9, None) if kind.endswith("1D") else (9, 5)
    spec = S.random_scenario(3, kind, nx, ny, steps=4, mu=True)
    f = workloads.build_field(spec)
    comps = [c for c in dir(f) if isinstance(getattr(f, c, None), FieldComponent)]
    assert comps
    before = {c: np.array(getattr(f, c).values, copy=True) for c in comps}
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        f.simulate(spec["steps"])
    for c, v in before.items():  # nothing was stepped on the host
        assert np.array_equal(np.asarray(getattr(f, c).values), v)


@needs_no_gpu
def test_batch_without_gpu_raises():
    specs = [S.random_scenario(k, "Acoustic2D", 9, 5, steps=4, mu=False) for k in range(2)]
    fields = [workloads.build_field(s) for s in specs]
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        batch.simulate_batch(fields, 4)

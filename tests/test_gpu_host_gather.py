"""fds_host_gather (csrc/dw_convert.cu): one kernel reads float64 host arrays where they
are (pageable memory the device reads through the host's page tables, as a Grace host
offers) and writes them to the device as float64, float32 or double words. Every
value must be what the per-array copies give: the same bits as torch's float64 ->
float32 rounding and as split_dw. Also the uploads of a batch and of a single field go
through it and match the copy path's results (HostUpload)."""
import ctypes as C

import numpy as np
import pytest

from pyfds_gb300 import _capi
from pyfds_gb300._engine import split_dw

pytestmark = pytest.mark.gpu


def test_gather_matches_the_copies(gpu):
    import torch
    lib = _capi.load()
    if not lib.fds_host_access():
        pytest.skip("the device does not read pageable host memory")
    rng = np.random.default_rng(3)
    arrays = []
    for n in (1, 7, 1000, 262147, 1 << 20):
        a = rng.standard_normal(n) * 10.0 ** rng.integers(-40, 40, n)
        a[: min(n, 4)] = [0.0, -0.0, 1e-310, -3.5][: min(n, 4)]
        arrays.append(a)
    dsts, items = [], []
    for a in arrays:
        for kind in (_capi.GATHER_F64, _capi.GATHER_F32, _capi.GATHER_DW):
            if kind == _capi.GATHER_F64:
                d = torch.empty(a.size, dtype=torch.float64, device="cuda")
            elif kind == _capi.GATHER_F32:
                d = torch.empty(a.size, dtype=torch.float32, device="cuda")
            else:
                d = torch.empty((a.size, 2), dtype=torch.float32, device="cuda")
            dsts.append((a, kind, d))
            items.append((a.ctypes.data, d.data_ptr(), a.size, kind, 0))
    table = np.array(items, dtype=_capi.GATHER_ITEM_DTYPE)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _capi.check(lib.fds_host_gather(C.c_void_p(table.ctypes.data), len(items), stream))
    torch.cuda.synchronize()
    for a, kind, d in dsts:
        got = d.cpu().numpy()
        if kind == _capi.GATHER_F64:
            want = a
        elif kind == _capi.GATHER_F32:
            want = torch.from_numpy(a).to(torch.float32).numpy()
        else:
            with np.errstate(over="ignore"):  # magnitudes past float32's range: inf, as the kernel
                want = split_dw(a)
        assert got.tobytes() == want.tobytes(), (a.size, kind)


def test_uploads_through_the_gather_equal_the_copies(gpu, monkeypatch):
    """A float32 and a double-word field stepped after an upload through the gather and
    after one through per-array copies: identical states and outputs."""
    from pyfds_gb300 import _engine
    from oracle import scenarios as S
    from helpers import build_field, field_results
    if not _capi.load().fds_host_access():
        pytest.skip("the device does not read pageable host memory")
    spec = S.random_scenario(41, "Acoustic2D", 420, 400, steps=20, mu=True)  # arrays > 1 MiB
    for precision in ("f32", "dw", "f64"):
        res = []
        for access in (True, False):
            monkeypatch.setattr(_engine, "_host_access", lambda a=access: a)
            f = build_field(spec, precision=precision)
            f.simulate(20)
            res.append(field_results(f))
        (sa, ga), (sb, gb) = res
        for c in sa:
            assert np.array_equal(sa[c], sb[c]), (precision, c)
            for x, y in zip(ga[c], gb[c]):
                assert np.array_equal(x, y), (precision, c)

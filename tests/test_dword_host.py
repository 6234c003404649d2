"""Host side of the double-word precision (precision="dw"), without a GPU: the
float64 <-> (hi, lo) float32 split, the ABI constant, the argument check of the C
ABI that rejects exact double words, the temperature-offset policy, and the engine's
automatic choice between one and two steps per tile."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from pyfds_gb300 import _capi
from pyfds_gb300._engine import PRECISIONS, join_dw, split_dw
from oracle import scenarios as S
from helpers import build_field

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_header_constant_matches():
    with open(os.path.join(ROOT, "include", "fds_capi.h")) as fh:
        m = re.search(r"#define FDS_PREC_DW (\d+)", fh.read())
    assert m and int(m.group(1)) == _capi.PREC_DW == PRECISIONS["dw"]


def test_split_is_exact_to_48_bits():
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.standard_normal(10000) * 10.0 ** rng.integers(-20, 20, 10000),
                        [0.0, 1.0, -3.5, 1e30, -1e-25, np.pi]])
    p = split_dw(x)
    assert p.dtype == np.float32 and p.shape == (x.size, 2)
    hi, lo = p[:, 0], p[:, 1]
    assert np.array_equal(hi, x.astype(np.float32))
    # normalised: |lo| <= ulp(hi) / 2
    assert np.all(np.abs(lo.astype(np.float64)) <= np.spacing(np.abs(hi)).astype(np.float64) / 2)
    y = join_dw(p)
    assert np.all(np.abs(y - x) <= 2.0 ** -48 * np.abs(x))
    # values with at most 48 significand bits survive exactly
    z = np.round(x * 2.0 ** 20) / 2.0 ** 20
    z = z[(np.abs(z) < 2.0 ** 27) & (np.abs(z) > 0)]
    assert np.array_equal(join_dw(split_dw(z)), z)


def test_exact_mode_is_float64_only():
    spec = S.random_scenario(1, "Acoustic2D", 8, 4, steps=2)
    with pytest.raises(ValueError):
        build_field(spec, precision="dw", exact=True)
    f = build_field(spec, precision="dw")
    assert f.precision == "dw"


def _fake_problem(precision, flags):
    pr = _capi.FdsStagProblem()
    pr.family = _capi.FAMILY_ACOUSTIC
    pr.precision = precision
    pr.flags = flags
    pr.nx, pr.ny = 64, 16
    pr.tile_x, pr.tile_y = 64, 16
    pr.coefs.bx = pr.coefs.kx = 4096  # never dereferenced: the checks fail first
    st = _capi.FdsStagState()
    for k in range(3):
        st.cur[k] = st.nxt[k] = 4096
    return pr, st


def test_abi_rejects_exact_double_words():
    lib = _capi.load()
    tb = _capi.FdsStagTables()
    pr, st = _fake_problem(_capi.PREC_DW, _capi.FLAG_HAS_V | _capi.FLAG_EXACT)
    assert lib.fds_stag_run(C.byref(pr), C.byref(st), C.byref(tb), 0, 1, 1, None) == \
        _capi.FDS_E_ARG
    assert "float64 only" in _capi.last_error()


@pytest.mark.parametrize("precision,explicit,expected", [
    ("f64", None, 0.0), ("f64", 250.0, 0.0),   # float64 stores the temperature itself
    ("f32_t64", 250.0, 0.0),
    ("f32", None, "mean"), ("f32", 250.0, 250.0),
    ("dw", None, 0.0), ("dw", 250.0, 250.0),    # double words: only when asked for
])
def test_potential_offset_policy(precision, explicit, expected):
    from pyfds_gb300._engine import StagEngine
    spec = S.random_scenario(4, "Thermal2D", 9, 5, steps=2)
    f = build_field(spec, precision=precision)
    f.potential_offset = explicit
    off = StagEngine(f)._potential_offset()
    if expected == "mean":
        expected = float(np.mean(f.temperature.values))
    assert off == expected
    g = build_field(S.random_scenario(4, "Acoustic2D", 9, 5, steps=2), precision=precision
                    if precision in ("f64", "f32", "dw") else "f64")
    g.potential_offset = 5.0
    assert StagEngine(g)._potential_offset() == 0.0  # acoustic: never


@pytest.mark.parametrize("kind,precision,kwargs,stages,batched,expected", [
    ("Acoustic2D", "f32", {}, 0, False, 3),       # float32: two steps per tile
    ("Acoustic2D", "dw", {}, 0, False, 3),        # double-word acoustic: two steps
    ("Thermal2D", "dw", {}, 0, False, 0),         # double-word thermal keeps one
    ("Thermal2D", "f32", {}, 0, False, 3),
    ("Acoustic2D", "f64", {}, 0, False, 4),       # float64 acoustic: the wavefront run
    ("Acoustic3DAxi", "f64", {}, 0, False, 4),    # (lossless axisymmetric steps as planar)
    ("Thermal2D", "f64", {}, 0, False, 0),        # float64 thermal keeps one per launch
    ("Acoustic2D", "f64", {"tile": (32, 32)}, 0, False, 0),  # no wavefront kernel
    ("Acoustic2D", "f64", {"exact": True}, 0, False, 0),
    ("Acoustic2D", "f64", {}, 4, True, 3),        # batches have no wavefront run
    ("Acoustic2D", "f32", {}, 1, False, 1),       # an explicit choice stands
    ("Acoustic2D", "f64", {}, 3, False, 3),
    ("Acoustic2D", "f64", {}, 0, True, 3),        # batches: two steps for every precision
    ("Thermal2D", "f32_t64", {}, 0, True, 0),     # ... with one potential/flux type
    ("Acoustic2D", "f32", {}, 2, True, 2),
    ("Acoustic1D", "f32", {}, 0, False, 0),       # 1-D: no two-step kernel
])
def test_automatic_stages(kind, precision, kwargs, stages, batched, expected):
    """StagEngine.stages: the field's choice when set; otherwise the wavefront run or
    two steps per tile where measured faster and the kernel exists (lossless 2-D,
    not exact, no moving medium, a tile with that kernel)."""
    from pyfds_gb300._engine import StagEngine
    spec = S.random_scenario(6, kind, 40, None if kind.endswith("1D") else 20, steps=2,
                             mu=False)
    f = build_field(spec, precision=precision, **kwargs)
    f.stages = stages
    f.assemble_matrices()
    assert StagEngine(f).stages(batched=batched) == expected


def test_automatic_stages_needs_lossless_fields():
    from pyfds_gb300._engine import StagEngine
    spec = S.random_scenario(6, "Acoustic2D", 40, 20, steps=2, mu=True)
    f = build_field(spec, precision="f32")
    f.assemble_matrices()
    assert f._stag_flags() & _capi.FLAG_ABSORB
    assert StagEngine(f).stages() == 0
    assert StagEngine(f).stages(batched=True) == 0

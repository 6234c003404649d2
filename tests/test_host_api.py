"""The package's host side against the reference's own known answers
(test/test_fields.py, test/test_regions.py, test/test_acoustics.py) and against the
pinned oracle: dimensions and lookups, line and rectangle regions, material vectors,
boundary application and output recording on a bare FieldComponent, the
finite-difference builders kept for inspection, and the assembled operators of
every field kind. numpy / scipy only; no GPU."""
import numpy as np
import pytest

import pyfds_gb300 as fds
from oracle import fds_oracle as O
from oracle import scenarios as S
from pyfds_gb300 import fields as fls
from pyfds_gb300 import regions as reg
from pyfds_gb300 import workloads


def _fwd(n, s=1):
    """Forward difference on the flat index with neighbour offset s."""
    return -np.eye(n) + np.eye(n, k=s)


def _bwd(n, s=1):
    return np.eye(n) - np.eye(n, k=-s)


def _cen(n, s=1):
    return 0.5 * (np.eye(n, k=s) - np.eye(n, k=-s))


def _lap(n, s=1):
    return -2 * np.eye(n) + np.eye(n, k=s) + np.eye(n, k=-s)


# ---- dimensions, lookups, regions (test/test_fields.py:6-9, 110-147)

def test_dimension_vector_and_index():
    d = fls.Dimension(3, 0.1)
    assert np.allclose(d.vector, 0.1 * np.arange(3))
    assert d.get_index(0.1) == 1


def test_index_and_position_round_trip():
    f1 = fls.Field1D(4, 0.1, 1, 1, int(5))
    assert np.isclose(f1.get_position(f1.get_index(0.1)), 0.1)
    f2 = fls.Field2D(4, 0.1, 3, 0.1, 1, 1, int(5))
    i = f2.get_index((0.2, 0.1))
    assert i == 2 + 1 * 4  # x + y * nx
    assert np.allclose(f2.get_position(i), (0.2, 0.1))


def test_line_region_sets_material():
    f = fls.Field1D(4, 0.1, 1, 1, int(5))
    f.material_regions.append(reg.MaterialRegion(f.get_line_region((0.1, 0.2)), int(23)))
    assert np.allclose(f.material_vector('real'), [5, 23, 23, 5])


# a 3 x 4 grid (dx 1, dy 0.5): flat index x + 3 y
@pytest.mark.parametrize("line,cells", [
    ((1, 0, 1, 1.5), [(1, 0), (1, 1), (1, 2), (1, 3)]),   # vertical
    ((0, 0, 2, 0), [(0, 0), (1, 0), (2, 0)]),             # horizontal
    ((0, 0, 2, 1.5), [(0, 0), (1, 1), (1, 2), (2, 3)]),   # rising diagonal
    ((0, 1.5, 2, 0), [(0, 3), (1, 2), (1, 1), (2, 0)]),   # falling diagonal, in line order
])
def test_line_regions_2d(line, cells):
    f = fls.Field2D(3, 1, 4, 0.5, 1, 1, int(5))
    assert list(f.get_line_region(line).indices) == [x + 3 * y for x, y in cells]


@pytest.mark.parametrize("rect,cells", [
    ((0, 0, 1, 1), [(0, 0), (0, 1), (0, 2), (1, 0), (1, 1), (1, 2)]),
    ((2, 1.5, -1, -1), [(1, 1), (1, 2), (1, 3), (2, 1), (2, 2), (2, 3)]),  # negative extent
])
def test_rect_regions_2d(rect, cells):
    f = fls.Field2D(3, 1, 4, 0.5, 1, 1, int(5))
    assert list(f.get_rect_region(rect).indices) == [x + 3 * y for x, y in cells]


# ---- material vectors (test/test_fields.py:50-55, 70-76)

@pytest.mark.parametrize("make,n", [
    (lambda: fls.Field1D(100, 0.1, 100, 0.1, int(5)), 100),
    (lambda: fls.Field2D(100, 0.1, 100, 0.1, 100, 0.1, int(5)), 10000),
])
def test_material_vector_of_the_main_material(make, n):
    v = make().material_vector('real')
    assert np.size(v) == n and np.all(v == 5)


# ---- boundaries and outputs of a bare component (test/test_fields.py:12-47,
# test/test_regions.py:5-8)

@pytest.mark.parametrize("start,value,additive,step,expect", [
    ("random", 23, False, 0, [23, 23, 23]),                       # scalar, Dirichlet
    ("ones", [np.arange(3) * 23, np.arange(3) * 42, np.arange(3) * 23], True, 1,
     [24, 43, 24]),                                              # one signal per point
    ("ones", np.arange(3) * 23, True, 2, [47, 47, 47]),           # one signal for all points
])
def test_component_boundary(start, value, additive, step, expect):
    fc = fls.FieldComponent(100)
    rng = np.random.default_rng(step)
    fc.values = rng.random(100) if start == "random" else np.ones(100)
    before = fc.values.copy()
    fc.boundaries = [reg.Boundary(reg.LineRegion([5, 6, 7], [0, 0.2], 'b'))]
    fc.boundaries[0].value = value
    fc.boundaries[0].additive = additive
    fc.apply_bounds(step=step)
    assert np.allclose(fc.values[[5, 6, 7]], expect)
    rest = np.setdiff1d(np.arange(100), [5, 6, 7])
    assert np.array_equal(fc.values[rest], before[rest])


def test_component_outputs_and_mean_signal():
    fc = fls.FieldComponent(100)
    fc.outputs = [reg.Output(reg.LineRegion([0, 1, 2], [0, 0.2], 'o'))]
    fc.write_outputs()
    fc.write_outputs()
    assert np.shape(fc.outputs[0].signals) == (3, 2)
    assert np.all(np.asarray(fc.outputs[0].signals) == 0)
    assert np.all(np.asarray(fc.outputs[0].mean_signal) == 0)
    out = reg.Output(reg.LineRegion([0, 1, 2], [0, 0.2], 'o'))
    ramp = np.linspace(0, 1)
    out.signals = [ramp * (k + 1) for k in range(3)]
    assert np.allclose(out.mean_signal, 2 * ramp)


# ---- operator builders (test/test_fields.py:57-107)

@pytest.mark.parametrize("variant,build", [(None, _fwd), ("forward", _fwd), ("backward", _bwd),
                                           ("central", _cen)])
def test_difference_builders(variant, build):
    kw = {} if variant is None else {"variant": variant}
    f1 = fls.Field1D(3, 1, 3, 1, int(5))
    assert np.allclose(f1.d_x(**kw).toarray(), build(3))
    f2 = fls.Field2D(2, 1, 2, 1, 10, 1, int(5))
    assert np.allclose(f2.d_x(**kw).toarray(), build(4))       # wraps across the row end
    assert np.allclose(f2.d_y(**kw).toarray(), build(4, 2))


def test_second_difference_builders():
    assert np.allclose(fls.Field1D(3, 1, 3, 1, 5).d_x2().toarray(), _lap(3))
    f2 = fls.Field2D(2, 1, 2, 1, 10, 1, int(5))
    assert np.allclose(f2.d_x2().toarray(), _lap(4))
    assert np.allclose(f2.d_y2().toarray(), _lap(4, 2))


# ---- materials and assembled operators (test/test_acoustics.py:5-66)

def test_acoustic_material_absorption():
    water = fds.AcousticMaterial(1500, 1000)
    water.bulk_viscosity = 1e-3
    water.shear_viscosity = 1e-3
    assert np.isclose(water.absorption_coef, 4 / 3 * 1e-3 + 1e-3)
    water.absorption_coef = 3e-3
    assert np.isclose(water.absorption_coef, 3e-3)
    assert np.isclose(fds.AcousticMaterial(1500, 1000, absorption_coef=2e-3).absorption_coef,
                      2e-3)


def test_acoustic_operators_known_answers():
    # c = 700, rho = 0.01, bulk viscosity 1, dt = dx = 1: rho c^2 = 4900, 1/rho = 100
    mat = fds.AcousticMaterial(700, 0.01, bulk_viscosity=1)
    f1 = fds.Acoustic1D(t_delta=1, t_samples=1, x_delta=1, x_samples=3, material=mat)
    f1.assemble_matrices()
    assert np.allclose(f1.a_p_v.toarray(), 4900 * _fwd(3))
    assert np.allclose(f1.a_v_p.toarray(), 100 * _bwd(3))
    assert np.allclose(f1.a_v_v.toarray(), 100 * _lap(3))
    f2 = fds.Acoustic2D(t_delta=1, t_samples=1, x_delta=1, x_samples=2, y_delta=1, y_samples=2,
                        material=mat)
    f2.assemble_matrices()
    assert np.allclose(f2.a_p_vx.toarray(), 4900 * _fwd(4))
    assert np.allclose(f2.a_p_vy.toarray(), 4900 * _fwd(4, 2))
    assert np.allclose(f2.a_vx_p.toarray(), 100 * _bwd(4))
    assert np.allclose(f2.a_vy_p.toarray(), 100 * _bwd(4, 2))
    for a in (f2.a_vx_vx, f2.a_vy_vy):
        assert np.allclose(a.toarray(), 100 * (_lap(4) + _lap(4, 2)))


OPERATORS = {
    "Acoustic1D": ("a_p_v", "a_v_p", "a_v_v"),
    "Acoustic2D": ("a_p_vx", "a_p_vy", "a_vx_p", "a_vy_p", "a_vx_vx", "a_vy_vy"),
    "Acoustic3DAxi": ("a_p_vx", "a_p_vy", "a_vx_p", "a_vy_p", "a_vx_vx", "a_vy_vy"),
    "Thermal1D": ("a_t_q", "a_q_t"),
    "Thermal2D": ("a_t_qx", "a_t_qy", "a_qx_t", "a_qy_t"),
    "Thermal3DAxi": ("a_t_qx", "a_t_qy", "a_qx_t", "a_qy_t"),
}


@pytest.mark.parametrize("kind", sorted(OPERATORS))
@pytest.mark.parametrize("seed", [1, 2])
def test_assembled_operators_match_the_oracle(kind, seed):
    """The package's assembled operators equal the oracle's (pinned to the reference's
    known answers and trajectories) entry for entry, on random media and sizes."""
    nx, ny = (7 + seed, None) if kind.endswith("1D") else (5 + seed, 4)
    spec = S.random_scenario(seed, kind, nx, ny, steps=2, mu=True)
    f = workloads.build_field(spec)
    f.assemble_matrices()
    ops = O.assemble(spec)
    n = nx * (ny or 1)
    assert set(OPERATORS[kind]) <= set(ops)
    for name in OPERATORS[kind]:
        assert np.array_equal(getattr(f, name).toarray(), O.dia_to_dense(ops[name], n)), name

"""The package's host-side geometry against the live reference, where its source tree
is available (skipped elsewhere): index and position lookups, point / line /
rectangle / triangle / ellipse regions, material vectors from random overlapping
regions, boundary application / output recording of a component with boundaries of
every value form, on random grids, and material objects. Lookups snap to a grid point within an absolute
10-eps radius and fail otherwise, so positions are drawn from the grid coordinates
and the outcomes, failures included, must agree. No GPU."""
import numpy as np
import pytest

from oracle.ref_loader import load_reference, reference_available
from pyfds_gb300 import fields as ours
from pyfds_gb300 import regions as our_reg

pytestmark = pytest.mark.skipif(not reference_available(),
                                reason="the reference source tree is not present")

SEEDS = range(12)


@pytest.fixture(scope="module")
def ref():
    return load_reference()


def _outcome(fn):
    """('ok', value) or ('error', exception type name)."""
    try:
        v = fn()
    except Exception as e:  # the same failure must occur on both sides
        return ("error", type(e).__name__)
    if hasattr(v, "indices"):
        v = np.asarray(v.indices).reshape(-1).tolist()
    elif isinstance(v, tuple):
        v = tuple(float(x) for x in v)
    elif isinstance(v, (np.floating, float)):
        v = float(v)
    return ("ok", v)


def _agree(fo, fr):
    a, b = _outcome(fo), _outcome(fr)
    assert a == b, (a, b)
    return a[0] == "ok"


def _grids(ref, seed):
    rng = np.random.default_rng(seed)
    nx, ny = (int(v) for v in rng.integers(3, 40, size=2))
    dx, dy = (float(v) for v in rng.uniform(0.01, 2.0, size=2))
    args = (nx, dx, ny, dy, 10, 1.0, int(5))
    return rng, ref.fields.Field2D(*args), ours.Field2D(*args)


def _points(rng, f, k):
    """k grid points (x, y) of field f."""
    xs, ys = f.x.vector, f.y.vector
    return [(float(xs[i]), float(ys[j]))
            for i, j in zip(rng.integers(0, len(xs), k), rng.integers(0, len(ys), k))]


@pytest.mark.parametrize("seed", SEEDS)
def test_lookups_2d(ref, seed):
    rng, r, o = _grids(ref, seed)
    ok = 0
    for p in _points(rng, r, 20):
        ok += _agree(lambda: o.get_index(p), lambda: r.get_index(p))
        i = r.get_index(p)
        _agree(lambda: o.get_position(i), lambda: r.get_position(i))
        _agree(lambda: o.get_point_region(p), lambda: r.get_point_region(p))
    assert ok == 20
    off = (float(r.x.vector[1]) * 0.5, float(r.y.vector[0]))    # between two grid points
    assert not _agree(lambda: o.get_index(off), lambda: r.get_index(off))


@pytest.mark.parametrize("seed", SEEDS)
def test_regions_2d(ref, seed):
    rng, r, o = _grids(ref, seed)
    ok = 0
    for _ in range(8):
        (x0, y0), (x1, y1), (x2, y2) = _points(rng, r, 3)
        line = (x0, y0, x1, y1)
        ok += _agree(lambda: o.get_line_region(line), lambda: r.get_line_region(line))
        rect = (x0, y0, x1 - x0, y1 - y0)                        # either sign
        _agree(lambda: o.get_rect_region(rect), lambda: r.get_rect_region(rect))
        tri = (x0, y0, x1, y1, x2, y2)
        _agree(lambda: o.get_tri_region(tri), lambda: r.get_tri_region(tri))
    ellipses = 0
    ys = r.y.vector
    for _ in range(8):
        # the ellipse's y extent is looked up on the grid: centre_y +- r_y must be grid
        # points, so r_y is a whole number of y steps that stays inside the grid
        i, j = int(rng.integers(0, len(r.x.vector))), int(rng.integers(0, len(ys)))
        k = int(rng.integers(0, min(j, len(ys) - 1 - j) + 1))
        centre = (float(r.x.vector[i]), float(ys[j]))
        radii = (float(rng.uniform(0.5, 6.0) * r.x.increment), float(ys[k]))
        if radii[1] == 0:
            continue
        ellipses += _agree(lambda: o.get_ellipse_region(centre, radii),
                           lambda: r.get_ellipse_region(centre, radii))
        _agree(lambda: o.get_ellipse_region(centre, radii[1]),   # scalar: a circle
               lambda: r.get_ellipse_region(centre, radii[1]))
    assert ok == 8  # lines between grid points always resolve
    assert ellipses >= 1


@pytest.mark.parametrize("seed", SEEDS)
def test_lookups_and_lines_1d(ref, seed):
    rng = np.random.default_rng(100 + seed)
    n, dx = int(rng.integers(3, 200)), float(rng.uniform(1e-4, 1.0))
    r = ref.fields.Field1D(n, dx, 10, 1.0, int(5))
    o = ours.Field1D(n, dx, 10, 1.0, int(5))
    xs = r.x.vector
    for k in rng.integers(0, n, 20):
        x = float(xs[k])
        assert _agree(lambda: o.get_index(x), lambda: r.get_index(x))
        _agree(lambda: o.get_position(int(k)), lambda: r.get_position(int(k)))
    for a, b in rng.integers(0, n, (6, 2)):
        lo, hi = float(xs[min(a, b)]), float(xs[max(a, b)])
        assert _agree(lambda: o.get_line_region((lo, hi)), lambda: r.get_line_region((lo, hi)))


@pytest.mark.parametrize("seed", SEEDS)
def test_material_vectors_2d(ref, seed):
    rng, r, o = _grids(ref, seed)
    added = 0
    for _ in range(6):
        (x0, y0), (x1, y1) = _points(rng, r, 2)
        line = (x0, y0, x1, y1)
        value = int(rng.integers(6, 100))
        r.material_regions.append(ref.regions.MaterialRegion(r.get_line_region(line), value))
        o.material_regions.append(our_reg.MaterialRegion(o.get_line_region(line), value))
        added += 1
        tri = (x0, y0, x1, y1) + _points(rng, r, 1)[0]
        ro, oo = _outcome(lambda: r.get_tri_region(tri)), _outcome(lambda: o.get_tri_region(tri))
        assert ro == oo
        if ro[0] == "ok":
            value = int(rng.integers(6, 100))
            r.material_regions.append(ref.regions.MaterialRegion(r.get_tri_region(tri), value))
            o.material_regions.append(our_reg.MaterialRegion(o.get_tri_region(tri), value))
            added += 1
    assert added >= 6
    assert np.array_equal(o.material_vector('real'), r.material_vector('real'))


def _random_boundaries(rng, n, steps, make_boundary, make_region):
    """Boundaries of every value form over random index sets (duplicates included):
    scalar, one signal for all points, one signal per point, [steps][points] array."""
    out = []
    for _ in range(int(rng.integers(2, 7))):
        k = int(rng.integers(1, 6))
        idx = rng.integers(0, n, k).tolist()
        form = int(rng.integers(0, 4))
        if form == 0:
            value = float(rng.normal())
        elif form == 1:
            value = rng.normal(size=steps)
        elif form == 2:
            value = [rng.normal(size=steps) for _ in idx]
        else:
            value = rng.normal(size=(steps, k))
        out.append(make_boundary(make_region(idx), value, bool(rng.integers(0, 2))))
    return out


@pytest.mark.parametrize("seed", SEEDS)
def test_component_bounds_and_outputs(ref, seed):
    """FieldComponent.apply_bounds / write_outputs on host arrays, step by step."""
    rng = np.random.default_rng(300 + seed)
    n, steps = int(rng.integers(5, 60)), 6
    r = ref.fields.FieldComponent(n)
    o = ours.FieldComponent(n)
    init = rng.normal(size=n)
    r.values, o.values = init.copy(), init.copy()
    state = rng.bit_generator.state
    r.boundaries = _random_boundaries(
        rng, n, steps, lambda reg_, v, a: ref.regions.Boundary(reg_, v, a),
        lambda idx: ref.regions.PointRegion(idx, None))
    rng.bit_generator.state = state  # the same boundaries for both
    o.boundaries = _random_boundaries(
        rng, n, steps, lambda reg_, v, a: our_reg.Boundary(reg_, v, a),
        lambda idx: our_reg.PointRegion(idx, None))
    probe = rng.integers(0, n, 4).tolist()
    r.outputs = [ref.regions.Output(ref.regions.PointRegion(probe, None))]
    o.outputs = [our_reg.Output(our_reg.PointRegion(probe, None))]
    for step in range(steps):
        ro = _outcome(lambda: r.apply_bounds(step))
        oo = _outcome(lambda: o.apply_bounds(step))
        assert ro == oo
        if ro[0] == "error":
            return
        assert np.array_equal(o.values, r.values), step
        r.write_outputs()
        o.write_outputs()
    assert np.array_equal(np.asarray(o.outputs[0].signals), np.asarray(r.outputs[0].signals))


@pytest.mark.parametrize("seed", SEEDS)
def test_materials(ref, seed):
    """Material objects: constructor defaults, the absorption coefficient derived from
    the viscosities and heat capacities (and its setter), the thermal conductivity
    (scalar or per direction), and the second-order material's defaults."""
    import pyfds_gb300 as fds
    rng = np.random.default_rng(500 + seed)
    c, rho = rng.uniform(100, 6000), rng.uniform(1, 8000)
    kw = {k: float(rng.uniform(0, 1e-2)) for k in ("shear_viscosity", "bulk_viscosity",
                                                    "thermal_conductivity")}
    kw.update(isobaric_heat_cap=float(rng.uniform(1, 5)), isochoric_heat_cap=float(rng.uniform(1, 5)))
    for args in ({}, kw, {"absorption_coef": float(rng.uniform(0, 1e-2))}):
        r, o = ref.AcousticMaterial(c, rho, **args), fds.AcousticMaterial(c, rho, **args)
        assert o.absorption_coef == r.absorption_coef
        assert (o.sound_velocity, o.density) == (r.sound_velocity, r.density)
        a = float(rng.uniform(0, 1e-2))
        r.absorption_coef, o.absorption_coef = a, a
        assert o.absorption_coef == r.absorption_coef
    conds = [float(rng.uniform(0.1, 300)),
             tuple(float(v) for v in rng.uniform(0.1, 300, 2))]
    for k in conds:
        outs = [_outcome(lambda: m.ThermalMaterial(897.0, 2700.0, k).thermal_conductivity)
                for m in (ref, fds)]
        assert outs[0] == outs[1]
        r, o = ref.ThermalMaterial(897.0, 2700.0, k), fds.ThermalMaterial(897.0, 2700.0, k)
        for name in ("heat_capacity", "density"):
            assert getattr(o, name) == getattr(r, name)
    for d in (2.0, None):  # None: the reference derives it (and fails doing so)
        outs = [_outcome(lambda: (lambda m: (m.d_rho_p, m.d_rho2_p))(
                    mod.AcousticMaterial2ndOrder(d_rho_p=d, sound_velocity=c, density=rho)))
                for mod in (ref, fds)]
        assert outs[0] == outs[1], outs

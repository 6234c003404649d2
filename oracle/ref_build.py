"""Build and run a scenario spec on the unmodified reference pyfds (validation only).

TEST INFRASTRUCTURE ONLY: used by ``tests/golden/make_golden.py`` and by CPU tests
that are skipped where the reference source tree is absent.

A scenario spec is a plain dict (see ``oracle.fds_oracle.simulate``):
``kind, nx, [ny], dx, [dy], dt, nt, materials, [init], [bounds], [outputs]``.
Materials are ``(indices or None, params)`` pairs in insertion order; ``None``
marks the main material that the reference's constructor installs over the
whole grid (``pyfds/fields.py:148-150``, ``:265-267``).
"""
import numpy as np

from .ref_loader import load_reference


def _make_material(pyfds, kind, params):
    if kind.startswith("Acoustic") or kind == "IdealGas1D":
        p = dict(params)
        mat = pyfds.AcousticMaterial(p.pop("sound_velocity"), p.pop("density"))
        for k, v in p.items():
            setattr(mat, k, v)
        return mat
    p = dict(params)
    kx = p.pop("thermal_conductivity_x")
    ky = p.pop("thermal_conductivity_y", kx)
    mat = pyfds.ThermalMaterial(p.pop("heat_capacity"), p.pop("density"), (kx, ky))
    return mat


def build_reference_field(spec):
    pyfds = load_reference()
    import pyfds.regions as reg

    kind = spec["kind"]
    cls = getattr(pyfds, kind)
    mats = spec["materials"]
    assert mats[0][0] is None, "first material must be the main material"
    main = _make_material(pyfds, kind, mats[0][1])
    if kind == "IdealGas1D":
        fld = cls(spec.get("convective", True), spec.get("nl_state", True),
                  x_samples=spec["nx"], x_delta=spec["dx"], t_samples=spec["nt"],
                  t_delta=spec["dt"], material=main)
    elif kind.endswith("1D"):
        fld = cls(x_samples=spec["nx"], x_delta=spec["dx"], t_samples=spec["nt"],
                  t_delta=spec["dt"], material=main)
    else:
        extra = (spec["flow"],) if kind == "AcousticFlow2D" else ()
        fld = cls(*extra, x_samples=spec["nx"], x_delta=spec["dx"], y_samples=spec["ny"],
                  y_delta=spec["dy"], t_samples=spec["nt"], t_delta=spec["dt"], material=main)
    for indices, params in mats[1:]:
        fld.add_material_region(reg.Region(list(map(int, indices)), "mat"),
                                _make_material(pyfds, kind, params))
    for name, v in (spec.get("init") or {}).items():
        getattr(fld, name).values = np.array(v, dtype=np.float64).copy()
    for name, blist in (spec.get("bounds") or {}).items():
        comp = getattr(fld, name)
        for b in blist:
            comp.boundaries.append(reg.Boundary(reg.Region(list(map(int, b["indices"])), "b"),
                                                value=b["value"],
                                                additive=b.get("additive", False)))
    for name, olist in (spec.get("outputs") or {}).items():
        comp = getattr(fld, name)
        for idx in olist:
            comp.outputs.append(reg.Output(reg.Region(list(map(int, idx)), "o")))
    return fld


def run_reference(spec, num_steps=None):
    """Run ``simulate(num_steps)`` on the reference; return (state, signals) like the oracle."""
    from .fds_oracle import components_of
    fld = build_reference_field(spec)
    fld.simulate(num_steps if num_steps else spec["nt"])
    state = {c: np.array(getattr(fld, c).values, dtype=np.float64) for c in components_of(spec["kind"])}
    signals = {}
    for c in components_of(spec["kind"]):
        comp = getattr(fld, c)
        signals[c] = [np.array(o.signals, dtype=np.float64).reshape(len(o.region.indices), -1)
                      for o in comp.outputs]
    return state, signals

"""Seeded scenario specs for parity tests (test infrastructure only).

A scenario spec is a plain dict understood by ``oracle.fds_oracle.simulate``, by
``oracle.ref_build.build_reference_field`` (reference, validation only) and by the
test helpers that build the same field through ``pyfds_gb300``. Every draw uses
``numpy.random.default_rng(seed)``.
"""
import numpy as np

ACOUSTIC_KINDS = ("Acoustic1D", "Acoustic2D", "Acoustic3DAxi")
THERMAL_KINDS = ("Thermal1D", "Thermal2D", "Thermal3DAxi")
ALL_KINDS = ACOUSTIC_KINDS + THERMAL_KINDS


def _components(kind):
    from .fds_oracle import components_of
    return components_of(kind)


def _random_material(rng, kind, mu):
    if kind.startswith("Acoustic"):
        c = float(rng.uniform(1000, 3000))
        rho = float(rng.uniform(800, 2000))
        return {"sound_velocity": c, "density": rho,
                "absorption_coef": float(rng.uniform(1e-4, 5e-3)) if mu else 0}
    k = float(rng.uniform(0.2, 200))
    aniso = rng.random() < 0.5
    return {"heat_capacity": float(rng.uniform(500, 1500)),
            "density": float(rng.uniform(1000, 3000)),
            "thermal_conductivity_x": k,
            "thermal_conductivity_y": float(rng.uniform(0.2, 200)) if aniso else k}


def _pulse(t, f, t0, sigma, amp=1.0):
    return amp * np.sin(2 * np.pi * f * t) * np.exp(-(t - t0) ** 2 / (2 * sigma ** 2))


def random_scenario(seed, kind, nx, ny=None, steps=40, mu=True, boundary_modes="all",
                    init_noise=True):
    """A small random scenario that exercises every boundary/output mode.

    - 1..3 extra material regions drawn over random cell subsets (later ones win),
    - Dirichlet scalar bounds, additive 1-D signals (with duplicate indices),
      per-point signal lists, 2-D ndarray signals, additive scalars,
    - outputs on every component, with duplicates,
    - random initial state so that every stencil term is active from step 0.
    """
    rng = np.random.default_rng(seed)
    is2d = not kind.endswith("1D")
    ny = (ny or 1) if is2d else 1
    n = nx * ny
    dx = 1e-4
    dy = dx * (float(rng.choice([1.0, 1.25])) if is2d else 1.0)
    mats = [(None, _random_material(rng, kind, mu))]
    for _ in range(int(rng.integers(1, 4))):
        cnt = int(rng.integers(1, max(2, n // 3)))
        idx = np.sort(rng.choice(n, size=cnt, replace=False))
        mats.append((idx.tolist(), _random_material(rng, kind, mu)))
    if kind.startswith("Acoustic"):
        cmax = max(m[1]["sound_velocity"] for m in mats)
        dt = 0.4 * min(dx, dy) / cmax / (np.sqrt(2) if is2d else 1.0)
    else:
        amax = max(max(m[1]["thermal_conductivity_x"], m[1]["thermal_conductivity_y"])
                   / (m[1]["density"] * m[1]["heat_capacity"]) for m in mats)
        dt = 0.2 * min(dx, dy) ** 2 / (4 * amax)
    nt = steps + 5
    t = np.arange(nt) * dt
    comps = _components(kind)
    bounds = {}
    outputs = {}
    f0 = 1.0 / (20 * dt)
    for ci, comp in enumerate(comps):
        bl = []
        modes = ["dirichlet", "signal", "list", "array2d", "scalar_add"]
        if boundary_modes != "all":
            modes = list(boundary_modes)
        for mode in modes:
            if rng.random() < 0.35 and mode != "dirichlet":
                continue
            cnt = int(rng.integers(1, min(6, n) + 1))
            idx = rng.integers(0, n, size=cnt).tolist()
            if mode == "dirichlet":
                # a fixed edge (first/last row or the two ends)
                if is2d:
                    edge = list(range(0, nx)) if rng.random() < 0.5 else list(range(0, n, nx))
                else:
                    edge = [0, n - 1]
                bl.append({"indices": edge, "value": float(rng.choice([0.0, 0.5])),
                           "additive": False})
            elif mode == "signal":
                if len(idx) > 1:
                    idx.append(idx[0])  # duplicate index: fancy assignment, last write wins
                bl.append({"indices": idx, "value": _pulse(t, f0, 10 * dt, 3 * dt),
                           "additive": bool(rng.random() < 0.8)})
            elif mode == "list":
                sigs = [_pulse(t, f0 * (1 + 0.1 * k), 8 * dt, 2 * dt, amp=1 + k)
                        for k in range(len(idx))]
                bl.append({"indices": idx, "value": sigs, "additive": bool(rng.random() < 0.5)})
            elif mode == "array2d":
                arr = rng.standard_normal((nt, len(idx))) * 0.1
                bl.append({"indices": idx, "value": arr, "additive": bool(rng.random() < 0.5)})
            elif mode == "scalar_add":
                bl.append({"indices": idx, "value": float(rng.uniform(-0.01, 0.01)),
                           "additive": True})
        if bl:
            bounds[comp] = bl
        ol = []
        for _ in range(int(rng.integers(1, 3))):
            cnt = int(rng.integers(1, min(5, n) + 1))
            idx = rng.integers(0, n, size=cnt).tolist()
            if cnt > 1 and rng.random() < 0.3:
                idx.append(idx[0])
            ol.append(idx)
        outputs[comp] = ol
    init = {}
    if init_noise:
        scale = {"pressure": 1.0, "velocity": 1e-6, "velocity_x": 1e-6, "velocity_y": 1e-6,
                 "temperature": 10.0, "heat_flux": 1.0, "heat_flux_x": 1.0, "heat_flux_y": 1.0}
        for comp in comps:
            base = 293.15 if comp == "temperature" else 0.0
            init[comp] = base + scale[comp] * rng.standard_normal(n)
    spec = {"kind": kind, "nx": nx, "dx": dx, "dt": dt, "nt": nt, "materials": mats,
            "bounds": bounds, "outputs": outputs, "init": init, "steps": steps}
    if is2d:
        spec["ny"] = ny
        spec["dy"] = dy
    return spec


def flow_scenario(seed, nx, ny, steps=60, flow="rows", mu=True):
    """A random Acoustic2D scenario with a moving medium (``AcousticFlow2D``,
    pyfds/acoustic_flow.py:13-57): the random_scenario of Acoustic2D plus a flow
    velocity, per row (``flow="rows"``: periods 1..9 steps, some rows negative and
    one row at rest) or one scalar (``flow="scalar"``)."""
    spec = random_scenario(seed, "Acoustic2D", nx, ny, steps=steps, mu=mu)
    rng = np.random.default_rng(seed + 7919)
    spec["kind"] = "AcousticFlow2D"
    if flow == "scalar":
        spec["flow"] = float(spec["dx"] / spec["dt"] / rng.integers(2, 7))
    else:
        periods = rng.integers(1, 10, size=ny).astype(np.float64)
        periods[rng.random(ny) < 0.2] *= -1
        v = spec["dx"] / spec["dt"] / (periods + 0.25)
        v[rng.integers(0, ny)] = 0.0
        spec["flow"] = v
    return spec


def nonlinear_scenario(seed, kind, nx, steps=60, convective=True, nl_state=True, mu=True):
    """A random 1-D nonlinear acoustic scenario (``IdealGas1D`` or
    ``Acoustic2ndOrder1D``, pyfds/nonlinear_acoustics.py): a gas (or liquid) with
    1..2 extra material regions, a small random initial density perturbation, a
    pressure source cell driven by a pulse, velocity held at 0 at both ends, and
    outputs on every component."""
    rng = np.random.default_rng(seed)
    dx = 1e-3
    liquid = kind == "Acoustic2ndOrder1D"

    def material():
        c = float(rng.uniform(1400, 1600) if liquid else rng.uniform(300, 360))
        rho = float(rng.uniform(900, 1100) if liquid else rng.uniform(1.0, 1.4))
        p = {"sound_velocity": c, "density": rho,
             "absorption_coef": float(rng.uniform(1e-4, 1e-2) * rho * c * dx) if mu else 0,
             "isobaric_heat_cap": float(rng.uniform(1.3, 1.7)), "isochoric_heat_cap": 1.0}
        if liquid:
            p["d_rho_p"] = c * c
            p["d_rho2_p"] = float(rng.uniform(1e6, 1e7))
        return p

    mats = [(None, material())]
    for _ in range(int(rng.integers(1, 3))):
        a, b = sorted(rng.integers(0, nx, size=2))
        mats.append((np.arange(a, b + 1), material()))
    cmax = max(m[1]["sound_velocity"] for m in mats)
    dt = 0.4 * dx / cmax
    rho0 = mats[0][1]["density"]
    # weak enough to stay finite over a few hundred steps (the reference's central
    # convective term grows slowly with forward Euler stepping)
    rel = 1e-5 if liquid else 1e-3
    init = {"density": rng.standard_normal(nx) * rel * rho0}
    t = np.arange(steps) * dt
    f0 = cmax / (12 * dx)
    amp = 10 * rel * rho0 * cmax ** 2
    src = int(rng.integers(1, nx - 1))
    spec = {"kind": kind, "nx": nx, "dx": dx, "dt": dt, "nt": steps, "steps": steps,
            "materials": mats, "init": init,
            "bounds": {"pressure": [{"indices": [src], "value": _pulse(t, f0, 4 / f0, 1 / f0, amp),
                                     "additive": False}],
                       "velocity": [{"indices": [0, nx - 1], "value": 0.0, "additive": False}]},
            "outputs": {"pressure": [[src, int(rng.integers(0, nx))]],
                        "velocity": [[int(rng.integers(0, nx)), int(rng.integers(0, nx))]],
                        "density": [[int(rng.integers(0, nx))]]}}
    if kind == "IdealGas1D":
        spec["convective"] = bool(convective)
        spec["nl_state"] = bool(nl_state)
    return spec


# ------------------------------------------------------------------ coupled fields

def coupled_scenario(seed, variant, nx=30, steps=40):
    """Coupled 1-D scenarios (pyfds/coupling.py, pyfds/coupled_fields.py):

    - "thermoacoustic" / "thermoacoustic3": ThermoAcoustic1D with a driven pressure
      cell (stepping 1, or 3 with accumulation);
    - "sync": Acoustic1D + Thermal1D in SynchronizedFields with a quadratic
      BoundaryCoupling of the pressure into the temperature (stepping 2, accumulated)
      and a power-law MaterialCoupling of the temperature into the sound velocity;
    - "sync_exp": the same with an exponential MaterialCoupling of the pressure into
      the thermal conductivity (change threshold 1e-9).
    """
    rng = np.random.default_rng(seed)
    dx = 1e-4
    ac_mat = {"sound_velocity": float(rng.uniform(1400, 1600)),
              "density": float(rng.uniform(900, 1100)),
              "absorption_coef": float(rng.uniform(1e-3, 1e-2))}
    th_mat = {"heat_capacity": float(rng.uniform(3000, 4500)),
              "density": float(rng.uniform(900, 1100)),
              "thermal_conductivity_x": float(rng.uniform(0.4, 0.7))}
    dt = 0.4 * dx / ac_mat["sound_velocity"]
    t = np.arange(steps) * dt
    f0 = ac_mat["sound_velocity"] / (10 * dx)
    src = int(rng.integers(1, nx - 1))
    bounds = {"pressure": [{"indices": [src], "value": _pulse(t, f0, 3 / f0, 1 / f0, 1e5),
                            "additive": True},
                           {"indices": [0, nx - 1], "value": 0.0, "additive": False}],
              "temperature": [{"indices": [0], "value": 293.15, "additive": False}]}
    outputs = {"pressure": [[int(rng.integers(0, nx)), src]],
               "velocity": [[int(rng.integers(0, nx))]],
               "temperature": [[int(rng.integers(0, nx)), src]]}
    init = {"temperature": 293.15 + rng.standard_normal(nx) * 0.01}
    if variant.startswith("thermoacoustic"):
        return {"kind": "ThermoAcoustic1D", "nx": nx, "dx": dx, "dt": dt, "nt": steps,
                "steps": steps, "acoustic_material": ac_mat, "thermal_material": th_mat,
                "stepping": 3 if variant == "thermoacoustic3" else 1,
                "bounds": bounds, "outputs": outputs, "init": init}
    base = {"nx": nx, "dx": dx, "dt": dt, "nt": steps}
    ac = dict(base, kind="Acoustic1D", materials=[(None, ac_mat)],
              bounds={"pressure": bounds["pressure"]},
              outputs={"pressure": outputs["pressure"], "velocity": outputs["velocity"]})
    th = dict(base, kind="Thermal1D", materials=[(None, th_mat)],
              bounds={"temperature": bounds["temperature"]},
              outputs={"temperature": outputs["temperature"]}, init=init)
    inter = [{"type": "boundary", "src": [0, "pressure"], "dst": [1, "temperature"],
              "fn": ["quad", 1e-12], "additive": True, "accumulate": True, "stepping": 2}]
    if variant == "sync":
        inter.append({"type": "material", "src": [1, "temperature"], "field": 0,
                      "param": "sound_velocity", "fn": ["power", 1, 1e-4], "rel": None,
                      "stepping": 2})
    else:
        inter.append({"type": "material", "src": [0, "pressure"], "field": 1,
                      "param": "thermal_conductivity_x", "fn": ["exp", 0.5, 1e-6],
                      "rel": 1e-9, "stepping": 1})
    return {"kind": "Synchronized", "nx": nx, "dt": dt, "nt": steps, "steps": steps,
            "fields": [ac, th], "interactions": inter}


def build_coupled(mod, spec, build_field, **field_kwargs):
    """The coupled object of ``spec`` from module ``mod`` (the reference package or
    pyfds_gb300): fields from ``build_field(field_spec)``, interactions from the
    library's coupling classes."""
    from .fds_oracle import transfer
    if spec["kind"] == "ThermoAcoustic1D":
        def mat(cls, p):
            p = dict(p)
            if cls is mod.AcousticMaterial:
                m = mod.AcousticMaterial(p.pop("sound_velocity"), p.pop("density"))
                for k, v in p.items():
                    setattr(m, k, v)
                return m
            return mod.ThermalMaterial(p["heat_capacity"], p["density"],
                                       p["thermal_conductivity_x"])
        obj = mod.ThermoAcoustic1D(spec["nx"], spec["dx"], spec["nt"], spec["dt"],
                                   mat(mod.ThermalMaterial, spec["thermal_material"]),
                                   mat(mod.AcousticMaterial, spec["acoustic_material"]),
                                   spec.get("stepping", 1), **field_kwargs)
        for name, v in (spec.get("init") or {}).items():
            getattr(obj, name).values = np.array(v, dtype=np.float64).copy()
        regmod = mod.regions
        for name, blist in (spec.get("bounds") or {}).items():
            for b in blist:
                getattr(obj, name).boundaries.append(regmod.Boundary(
                    regmod.Region(list(map(int, b["indices"])), "boundary"), value=b["value"],
                    additive=b.get("additive", False)))
        for name, olist in (spec.get("outputs") or {}).items():
            for idx in olist:
                getattr(obj, name).outputs.append(regmod.Output(
                    regmod.Region(list(map(int, idx)), "output")))
        return obj
    fields = [build_field(f, **field_kwargs) for f in spec["fields"]]
    inter = []
    for it in spec["interactions"]:
        if it["type"] == "boundary":
            fn = it["fn"]
            inter.append(mod.BoundaryCoupling(
                getattr(fields[it["src"][0]], it["src"][1]),
                getattr(fields[it["dst"][0]], it["dst"][1]),
                lambda x, fn=fn: transfer(fn, x), additive=it["additive"],
                accumulate=it["accumulate"], stepping=it["stepping"]))
        else:
            src = getattr(fields[it["src"][0]], it["src"][1])
            tgt = fields[it["field"]]
            fn = it["fn"]
            if fn[0] == "power":
                inter.append(mod.MaterialCouplingPowerLaw(src, tgt, it["param"], fn[1], fn[2],
                                                          rel_change_threshold=it["rel"],
                                                          stepping=it["stepping"]))
            elif fn[0] == "exp":
                inter.append(mod.MaterialCouplingExponential(src, tgt, it["param"], fn[1], fn[2],
                                                             rel_change_threshold=it["rel"],
                                                             stepping=it["stepping"]))
            else:
                inter.append(mod.MaterialCoupling(src, tgt, it["param"],
                                                  lambda x, fn=fn: transfer(fn, x),
                                                  rel_change_threshold=it["rel"],
                                                  stepping=it["stepping"]))
    return mod.SynchronizedFields(fields, inter)


def coupled_results(obj, kind_of):
    """([(state, signals)] per field) of a simulated coupled object."""
    out = []
    for f in obj.fields:
        kind = kind_of(f)
        from .fds_oracle import components_of
        st = {c: np.array(getattr(f, c).values, dtype=np.float64) for c in components_of(kind)}
        sig = {c: [np.array(o.signals, dtype=np.float64).reshape(
            len(np.asarray(o.region.indices).reshape(-1)), -1) for o in getattr(f, c).outputs]
            for c in components_of(kind)}
        out.append((st, sig))
    return out

"""Seeded synthetic workloads (plain scenario specs) and a builder for fields.

A scenario spec is a plain dict::

    {"kind": "Acoustic2D", "nx": .., "ny": .., "dx": .., "dy": .., "dt": .., "nt": ..,
     "steps": .., "materials": [(None | indices, params), ...],
     "init": {component: values}, "bounds": {component: [{indices, value, additive}]},
     "outputs": {component: [indices, ...]}}

``materials[0]`` (indices None) is the main material over the whole grid; later
entries overwrite their cells. ``build_field`` turns a spec into a pyfds_gb300
field; the same spec drives the CPU oracle in the tests.
"""
import numpy as np

from . import acoustic_flow, acoustics, nonlinear_acoustics, regions as reg, thermal

WATER = {"sound_velocity": 1500.0, "density": 1000.0, "absorption_coef": 0}
STEEL = {"sound_velocity": 5900.0, "density": 7850.0, "absorption_coef": 0}
ALUMINIUM = {"heat_capacity": 897.0, "density": 2700.0, "thermal_conductivity_x": 237.0,
             "thermal_conductivity_y": 237.0}
POLYMER = {"heat_capacity": 1470.0, "density": 1190.0, "thermal_conductivity_x": 0.19,
           "thermal_conductivity_y": 0.19}


def gauss_pulse(t, f, t0, sigma, amp=1.0):
    """Gaussian-modulated sine ``amp sin(2 pi f t) exp(-(t - t0)^2 / (2 sigma^2))``."""
    return amp * np.sin(2 * np.pi * f * t) * np.exp(-(t - t0) ** 2 / (2 * sigma ** 2))


def acoustic1d_water(nx=1000, nt=2000, additive=True):
    """Acoustic1D in water, dx = 1e-4 m, dt = 0.5 dx / c, 2000 steps.

    Pressure held at 0 at both ends; a 1 MHz Gaussian-modulated source (centre 2 us,
    sigma 0.5 us, 1 Pa) at index 100; a pressure output at index 800."""
    dx = 1e-4
    dt = 0.5 * dx / WATER["sound_velocity"]
    t = np.arange(nt) * dt
    return {"kind": "Acoustic1D", "nx": nx, "dx": dx, "dt": dt, "nt": nt, "steps": nt,
            "materials": [(None, dict(WATER))],
            "bounds": {"pressure": [
                {"indices": [0], "value": 0, "additive": False},
                {"indices": [nx - 1], "value": 0, "additive": False},
                {"indices": [100], "value": gauss_pulse(t, 1e6, 2e-6, 0.5e-6),
                 "additive": additive}]},
            "outputs": {"pressure": [[800]]}}


def acoustic2d_steel_block(n=2048, nt=4000, n_probes=64, seed=2):
    """Acoustic2D n x n (2048 by default), dx = dy = 5e-5 m, water with a steel block.

    The block covers x in [800, 1200), y in [1000, 1600) (scaled by n / 2048);
    dt = 0.5 dx / (5900 sqrt 2); zero-pressure edges; an additive line source along
    y = 200 for x = 512..1536 (scaled) with the 1 MHz pulse; n_probes pressure
    outputs drawn uniformly over interior cells."""
    dx = 5e-5
    s = n / 2048.0
    dt = 0.5 * dx / (STEEL["sound_velocity"] * np.sqrt(2))
    t = np.arange(nt) * dt
    xs = np.arange(int(800 * s), int(1200 * s))
    ys = np.arange(int(1000 * s), int(1600 * s))
    steel = (xs[:, None] + ys[None, :] * n).reshape(-1)
    edges = np.unique(np.concatenate([np.arange(n), (n - 1) * n + np.arange(n),
                                      np.arange(n) * n, np.arange(n) * n + n - 1]))
    line = int(200 * s) * n + np.arange(int(512 * s), int(1536 * s) + 1)
    rng = np.random.default_rng(seed)
    pr = rng.integers(1, n - 1, size=(n_probes, 2))
    probes = (pr[:, 0] + pr[:, 1] * n).tolist()
    return {"kind": "Acoustic2D", "nx": n, "ny": n, "dx": dx, "dy": dx, "dt": dt, "nt": nt,
            "steps": nt,
            "materials": [(None, dict(WATER)), (steel, dict(STEEL))],
            "bounds": {"pressure": [
                {"indices": edges, "value": 0, "additive": False},
                {"indices": line, "value": gauss_pulse(t, 1e6, 2e-6, 0.5e-6), "additive": True}]},
            "outputs": {"pressure": [probes]}}


def acoustic_flow_block(n=2048, nt=4000, n_probes=64, seed=2, period=10):
    """The water/steel Acoustic2D workload of ``acoustic2d_steel_block`` in a medium
    moving along x (AcousticFlow2D): flow = dx / (period + 0.5) / dt in every row, so
    every row moves one cell every ``period`` steps."""
    spec = acoustic2d_steel_block(n, nt, n_probes, seed)
    spec["kind"] = "AcousticFlow2D"
    spec["flow"] = float(spec["dx"] / (period + 0.5) / spec["dt"])
    return spec


def ideal_gas_column(n=1000, nt=20000, nl_state=True):
    """IdealGas1D: a 1 m air column (c = 343 m/s, rho = 1.2 kg/m^3, gamma = 1.4,
    light absorption), dx = 1 mm, dt at CFL 0.5; a finite-amplitude 10 kPa pressure
    pulse (5 kHz, Gaussian-modulated) driven at cell 1, velocity 0 at both ends,
    pressure outputs at the quarter points."""
    dx = 1e-3
    c, rho = 343.0, 1.2
    dt = 0.5 * dx / c
    t = np.arange(nt) * dt
    mat = {"sound_velocity": c, "density": rho, "absorption_coef": 1.8e-5,
           "isobaric_heat_cap": 1.4, "isochoric_heat_cap": 1.0}
    return {"kind": "IdealGas1D", "nx": n, "dx": dx, "dt": dt, "nt": nt, "steps": nt,
            "convective": True, "nl_state": nl_state,
            "materials": [(None, mat)],
            "bounds": {"pressure": [{"indices": [1],
                                     "value": gauss_pulse(t, 5e3, 4e-4, 1e-4, 1e4),
                                     "additive": False}],
                       "velocity": [{"indices": [0, n - 1], "value": 0.0, "additive": False}]},
            "outputs": {"pressure": [[n // 4, n // 2, 3 * n // 4]]}}


def axi_disc_source(nr=1024, nz=4096, nt=6000, disc=200, probe_every=64):
    """Acoustic3DAxi r x z = 1024 x 4096, dx = dz = 5e-5 m, water, 6000 steps.

    An additive disc source of radius ``disc`` cells at z = 0 driven by a 2 MHz
    Gaussian-modulated pulse (centre 1 us, sigma 0.25 us); on-axis pressure outputs
    every ``probe_every`` cells; dt = 0.5 dx / (1500 sqrt 2)."""
    dx = 5e-5
    dt = 0.5 * dx / (WATER["sound_velocity"] * np.sqrt(2))
    t = np.arange(nt) * dt
    src = np.arange(min(disc, nr))
    probes = (np.arange(0, nz, probe_every) * nr).tolist()
    return {"kind": "Acoustic3DAxi", "nx": nr, "ny": nz, "dx": dx, "dy": dx, "dt": dt,
            "nt": nt, "steps": nt, "materials": [(None, dict(WATER))],
            "bounds": {"pressure": [{"indices": src, "value": gauss_pulse(t, 2e6, 1e-6, 0.25e-6),
                                     "additive": True}]},
            "outputs": {"pressure": [probes]}}


def thermal2d_two_materials(n=4096, nt=50000, n_probes=64, seed=4):
    """Thermal2D n x n, dx = 1e-4 m: aluminium with a polymer part above a seeded
    sinusoidal interface y > n/2 + A sin(2 pi x / lambda + phi).

    Initial temperature 293.15 K, column x = 0 held at 373.15 K, dt at 0.2 of the
    explicit diffusion limit dx^2 / (4 alpha_max), n_probes seeded outputs."""
    dx = 1e-4
    rng = np.random.default_rng(seed)
    amp = rng.uniform(0.02, 0.1) * n
    lam = rng.uniform(0.2, 0.6) * n
    phi = rng.uniform(0, 2 * np.pi)
    x = np.arange(n)
    yint = n / 2 + amp * np.sin(2 * np.pi * x / lam + phi)
    yy = np.arange(n)
    mask = yy[None, :] > yint[:, None]  # [x, y]
    xi, yi = np.nonzero(mask)
    poly = (xi + yi * n).astype(np.int64)
    alpha = max(m["thermal_conductivity_x"] / (m["density"] * m["heat_capacity"])
                for m in (ALUMINIUM, POLYMER))
    dt = 0.2 * dx ** 2 / (4 * alpha)
    pr = rng.integers(1, n - 1, size=(n_probes, 2))
    probes = (pr[:, 0] + pr[:, 1] * n).tolist()
    return {"kind": "Thermal2D", "nx": n, "ny": n, "dx": dx, "dy": dx, "dt": dt, "nt": nt,
            "steps": nt, "materials": [(None, dict(ALUMINIUM)), (poly, dict(POLYMER))],
            "init": {"temperature": np.full(n * n, 293.15)},
            "bounds": {"temperature": [{"indices": np.arange(n) * n, "value": 373.15,
                                        "additive": False}]},
            "outputs": {"temperature": [probes]}}


def layered_media_batch(count=256, nt=2000, n_probes=16, seed=3, n_min=128, n_max=1024):
    """``count`` Acoustic2D scenarios of uneven size and media (seeded).

    Per instance: square side n = round(exp(U(ln n_min, ln n_max))); 3..8 horizontal
    layers with uniform-random thicknesses, c ~ U[1000, 3000] m/s, rho ~ U[800, 2000]
    kg/m^3; a point pressure source at a uniform interior cell driven by a
    Gaussian-modulated sine with f ~ U[0.5, 5] MHz (centre 2/f, sigma 0.5/f);
    dx = c_min / (20 f), dt = 0.4 dx / c_max; zero-pressure edges; ``n_probes``
    pressure outputs at uniform interior cells; ``nt`` steps."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(count):
        n = int(round(np.exp(rng.uniform(np.log(n_min), np.log(n_max)))))
        layers = int(rng.integers(3, 9))
        cuts = np.sort(rng.choice(np.arange(1, n), size=layers - 1, replace=False))
        bounds = np.concatenate([[0], cuts, [n]])
        cs = rng.uniform(1000, 3000, size=layers)
        rhos = rng.uniform(800, 2000, size=layers)
        f0 = rng.uniform(0.5e6, 5e6)
        dx = cs.min() / (20 * f0)
        dt = 0.4 * dx / cs.max()
        t = np.arange(nt) * dt
        xs = np.arange(n)
        mats = [(None, {"sound_velocity": float(cs[0]), "density": float(rhos[0]),
                        "absorption_coef": 0})]
        for k in range(1, layers):
            ys = np.arange(bounds[k], bounds[k + 1])
            idx = (xs[:, None] + ys[None, :] * n).reshape(-1)
            mats.append((idx, {"sound_velocity": float(cs[k]), "density": float(rhos[k]),
                               "absorption_coef": 0}))
        edges = np.unique(np.concatenate([np.arange(n), (n - 1) * n + np.arange(n),
                                          np.arange(n) * n, np.arange(n) * n + n - 1]))
        src = rng.integers(1, n - 1, size=2)
        pr = rng.integers(1, n - 1, size=(n_probes, 2))
        specs.append({
            "kind": "Acoustic2D", "nx": n, "ny": n, "dx": dx, "dy": dx, "dt": dt, "nt": nt,
            "steps": nt, "materials": mats,
            "bounds": {"pressure": [
                {"indices": edges, "value": 0, "additive": False},
                {"indices": [int(src[0] + src[1] * n)],
                 "value": gauss_pulse(t, f0, 2.0 / f0, 0.5 / f0), "additive": True}]},
            "outputs": {"pressure": [(pr[:, 0] + pr[:, 1] * n).tolist()]},
            "frequency": f0})
    return specs


def surrogate_media(count, seed, n=256, nt=4096, t_src=704):
    """``count`` Acoustic2D scenarios of the layered-media kind of
    ``layered_media_batch`` at a fixed n x n grid, for the learned surrogate.

    Same draws per instance (3..8 layers, c ~ U[1000, 3000], rho ~ U[800, 2000],
    f ~ U[0.5, 5] MHz, point source, dx = c_min / (20 f), dt = 0.4 dx / c_max,
    zero-pressure edges), without probes. The source pulse (centre 2/f, sigma
    0.5/f) is cut to exactly zero from step ``t_src`` on, so every later window
    is source-free (t_src = 704 covers centre + 5 sigma for any c_max / c_min <= 3).
    Each spec also carries the per-cell ``c`` and ``rho`` maps ([n][n], row y)."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(count):
        layers = int(rng.integers(3, 9))
        cuts = np.sort(rng.choice(np.arange(1, n), size=layers - 1, replace=False))
        bounds = np.concatenate([[0], cuts, [n]])
        cs = rng.uniform(1000, 3000, size=layers)
        rhos = rng.uniform(800, 2000, size=layers)
        f0 = rng.uniform(0.5e6, 5e6)
        dx = cs.min() / (20 * f0)
        dt = 0.4 * dx / cs.max()
        t = np.arange(nt) * dt
        sig = gauss_pulse(t, f0, 2.0 / f0, 0.5 / f0)
        sig[t_src:] = 0.0
        xs = np.arange(n)
        cmap = np.empty((n, n))
        rmap = np.empty((n, n))
        mats = [(None, {"sound_velocity": float(cs[0]), "density": float(rhos[0]),
                        "absorption_coef": 0})]
        cmap[:] = cs[0]
        rmap[:] = rhos[0]
        for k in range(1, layers):
            ys = np.arange(bounds[k], bounds[k + 1])
            idx = (xs[:, None] + ys[None, :] * n).reshape(-1)
            mats.append((idx, {"sound_velocity": float(cs[k]), "density": float(rhos[k]),
                               "absorption_coef": 0}))
            cmap[bounds[k]:bounds[k + 1], :] = cs[k]
            rmap[bounds[k]:bounds[k + 1], :] = rhos[k]
        edges = np.unique(np.concatenate([np.arange(n), (n - 1) * n + np.arange(n),
                                          np.arange(n) * n, np.arange(n) * n + n - 1]))
        src = rng.integers(1, n - 1, size=2)
        specs.append({
            "kind": "Acoustic2D", "nx": n, "ny": n, "dx": dx, "dy": dx, "dt": dt, "nt": nt,
            "steps": nt, "materials": mats,
            "bounds": {"pressure": [
                {"indices": edges, "value": 0, "additive": False},
                {"indices": [int(src[0] + src[1] * n)], "value": sig, "additive": True}]},
            "outputs": {},
            "frequency": f0, "c_map": cmap, "rho_map": rmap, "t_src": t_src})
    return specs


def _material(kind, params):
    p = dict(params)
    if kind.startswith("Acoustic") or kind == "IdealGas1D":
        mat = acoustics.AcousticMaterial(p.pop("sound_velocity"), p.pop("density"))
        for k, v in p.items():
            setattr(mat, k, v)
        return mat
    kx = p.pop("thermal_conductivity_x")
    ky = p.pop("thermal_conductivity_y", kx)
    return thermal.ThermalMaterial(p.pop("heat_capacity"), p.pop("density"), (kx, ky))


def build_field(spec, **kwargs):
    """A pyfds_gb300 field built from a scenario spec (extra kwargs go to the
    constructor, e.g. ``precision`` or ``exact``)."""
    kind = spec["kind"]
    cls = (getattr(acoustics, kind, None) or getattr(acoustic_flow, kind, None)
           or getattr(nonlinear_acoustics, kind, None) or getattr(thermal, kind))
    mats = spec["materials"]
    main = _material(kind, mats[0][1])
    if kind == "IdealGas1D":
        kwargs = dict(kwargs, convective=spec.get("convective", True),
                      nl_state=spec.get("nl_state", True))
    if kind.endswith("1D"):
        f = cls(x_samples=spec["nx"], x_delta=spec["dx"], t_samples=spec["nt"],
                t_delta=spec["dt"], material=main, **kwargs)
    else:
        extra = (spec["flow"],) if kind == "AcousticFlow2D" else ()
        f = cls(*extra, x_samples=spec["nx"], x_delta=spec["dx"], y_samples=spec["ny"],
                y_delta=spec["dy"], t_samples=spec["nt"], t_delta=spec["dt"], material=main,
                **kwargs)
    for idx, params in mats[1:]:
        f.add_material_region(reg.Region(np.asarray(idx, dtype=np.int64), "material"),
                              _material(kind, params))
    for name, v in (spec.get("init") or {}).items():
        getattr(f, name).values = np.array(v, dtype=np.float64)
    for name, blist in (spec.get("bounds") or {}).items():
        comp = getattr(f, name)
        for b in blist:
            comp.boundaries.append(reg.Boundary(reg.Region(b["indices"], "boundary"),
                                                value=b["value"],
                                                additive=b.get("additive", False)))
    for name, olist in (spec.get("outputs") or {}).items():
        comp = getattr(f, name)
        for idx in olist:
            comp.outputs.append(reg.Output(reg.Region(idx, "output")))
    return f

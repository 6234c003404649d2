"""CPU oracle for the staggered-grid FD time step of pyfds.

TEST INFRASTRUCTURE ONLY. This module is the checker: ``tests/``, the package's
``smoke()`` and the CPU-baseline leg of ``bench.py`` may import it; the product
path (``pyfds_gb300``) never does.

It restates, in plain numpy, the arithmetic that the reference performs through
``scipy.sparse.dia_matrix.dot`` (scipy 1.18, an un-vendored dependency of the
reference: ``pyproject.toml:16-20`` pins no version). The restatement follows
scipy's documented DIA layout: ``dia_matrix((data, offsets))`` stores
``data[k][j]`` at ``A[j - offsets[k], j]``, so every diagonal is indexed by the
*column* (the neighbour it multiplies), and the matrix-vector product
accumulates ``y[i] += data[k][i + o_k] * x[i + o_k]`` diagonal by diagonal in
storage order, starting from ``y = 0``. Sums of operators
(``(d_x2 + d_y2).todia()``) go through CSR addition (position-wise ``a + b`` in
operand order) and come back with their diagonals sorted by offset. Each of
these rules is reproduced below with the same floating-point operation order,
so on a machine whose scipy build does not contract multiply-adds (x86-64) the
oracle is bit-identical to the reference; the golden fixtures check this.

Parity status: pinned. ``tests/test_oracle_golden.py`` checks the oracle against
the operator known-answer matrices of the reference's own tests
(``test/test_acoustics.py:19-66``, ``test/test_fields.py:57-107``,
``test/test_coupling.py:113-118``) and against trajectories produced by the
unmodified reference (``tests/golden/make_golden.py``).
"""
import numpy as np

__all__ = [
    "dia_matvec", "d_x", "d_y", "d_x2", "d_y2", "dia_sum", "dia_to_dense",
    "material_vector", "apply_bounds", "write_outputs",
    "assemble", "sim_step", "simulate", "components_of",
]

# --------------------------------------------------------------------------------------
# DIA operators (pyfds/fields.py:158-202 for 1-D, :273-365 for 2-D)
# An operator is a list of (offset, data) pairs in storage order; len(data) == N.
# --------------------------------------------------------------------------------------


def _ones(n):
    # fields.py:172 / :287: np.array(1).repeat(N) -> integer ones
    return np.array(1).repeat(n)


def d_x(n, factors=None, variant="forward"):
    """``Field1D/Field2D.d_x`` (pyfds/fields.py:158-184, :273-299); x-step is 1 in flat order."""
    return _first_derivative(n, factors, variant, 1)


def d_y(n, nx, factors=None, variant="forward"):
    """``Field2D.d_y`` (pyfds/fields.py:301-328); y-step is ``x.samples`` in flat order."""
    return _first_derivative(n, factors, variant, nx)


def _first_derivative(n, factors, variant, step):
    if factors is None:
        factors = _ones(n)
    factors = np.asarray(factors)
    if variant == "forward":
        data = np.array([-factors, factors])
        offs = [0, step]
    elif variant == "central":
        data = np.array([-factors / 2, factors / 2])
        offs = [-step, step]
    elif variant == "backward":
        data = np.array([-factors, factors])
        offs = [-step, 0]
    else:
        raise ValueError("Unknown difference quotient variant {}.".format(variant))
    return [(o, data[k]) for k, o in enumerate(offs)]


def d_x2(n, factors=None):
    """``d_x2`` (pyfds/fields.py:186-202, :330-346)."""
    if factors is None:
        factors = _ones(n)
    factors = np.asarray(factors)
    data = np.array([factors, -2 * factors, factors])
    return [(-1, data[0]), (0, data[1]), (1, data[2])]


def d_y2(n, nx, factors=None):
    """``Field2D.d_y2`` (pyfds/fields.py:348-365)."""
    if factors is None:
        factors = _ones(n)
    factors = np.asarray(factors)
    data = np.array([factors, -2 * factors, factors])
    return [(-nx, data[0]), (0, data[1]), (nx, data[2])]


def _valid_mask(n, off):
    """Columns j that hold a stored entry of diagonal ``off`` in an n x n matrix."""
    j = np.arange(n)
    i = j - off
    return (i >= 0) & (i < n)


def dia_sum(*ops):
    """Sum of DIA operators as scipy computes ``(A + B + ...).todia()``.

    CSR addition combines coinciding entries position-wise, left operand first, and
    drops entries that come out exactly zero; ``todia`` then sorts the diagonals by
    offset. Dropped zeros only change results for non-finite inputs, which the
    oracle does not model, so they are kept as zeros here.
    """
    n = len(ops[0][0][1])
    acc = {}
    present = {}
    for op in ops:
        # entries of one operand: (offset -> per-column value), duplicates within one
        # dia_matrix are summed by tocsr in storage order.
        local = {}
        for off, data in op:
            m = _valid_mask(n, off)
            vals = np.where(m, np.asarray(data, dtype=np.float64), 0.0)
            if off in local:
                local[off] = (local[off][0] + vals, local[off][1] | m)
            else:
                local[off] = (vals, m)
        for off, (vals, m) in local.items():
            if off in acc:
                both = present[off] & m
                new = np.where(both, acc[off] + vals, np.where(m, vals, acc[off]))
                acc[off] = new
                present[off] = present[off] | m
            else:
                acc[off] = vals.copy()
                present[off] = m.copy()
    return [(off, acc[off]) for off in sorted(acc)]


def dia_matvec(op, x):
    """``dia_matrix.dot`` for one operator, same accumulation order as scipy."""
    x = np.asarray(x, dtype=np.float64)
    n = x.shape[0]
    y = np.zeros(n)
    for off, data in op:
        data = np.asarray(data, dtype=np.float64)
        if off >= 0:
            if off < n:
                y[: n - off] += data[off:] * x[off:]
        else:
            if -off < n:
                y[-off:] += data[: n + off] * x[: n + off]
    return y


def dia_to_dense(op, n):
    a = np.zeros((n, n))
    for off, data in op:
        for j in range(n):
            i = j - off
            if 0 <= i < n:
                a[i, j] += data[j]
    return a


# --------------------------------------------------------------------------------------
# Materials (pyfds/fields.py:34-57) and per-kind assembly
# --------------------------------------------------------------------------------------


def material_vector(n, material_regions, name):
    """``Field.material_vector`` (pyfds/fields.py:34-57).

    ``material_regions`` is a list of ``(indices, params)`` in insertion order where
    ``params`` is a dict of material parameters; later regions overwrite earlier ones.
    """
    vec = np.zeros(n)
    found = False
    for indices, params in material_regions:
        if name in params and params[name] is not None:
            # ``None`` stands for the main region, which covers every cell
            # (pyfds/fields.py:148-150, :265-267)
            idx = slice(None) if indices is None else np.asarray(indices, dtype=np.int64)
            vec[idx] = params[name]
            found = True
    if not found:
        raise KeyError("Material parameter {} not found in set materials.")
    return vec


def components_of(kind):
    """Field component names in the order the reference creates them."""
    return {
        "Acoustic1D": ["pressure", "velocity"],
        "Acoustic2D": ["pressure", "velocity_x", "velocity_y"],
        "AcousticFlow2D": ["pressure", "velocity_x", "velocity_y"],
        "Acoustic3DAxi": ["pressure", "velocity_x", "velocity_y"],
        "Thermal1D": ["temperature", "heat_flux"],
        "IdealGas1D": ["pressure", "velocity", "density"],
        "Acoustic2ndOrder1D": ["pressure", "velocity", "density"],
        "Thermal2D": ["temperature", "heat_flux_x", "heat_flux_y"],
        "Thermal3DAxi": ["temperature", "heat_flux_x", "heat_flux_y"],
    }[kind]


def _radii(nx, ny, dx):
    """``_radii`` (pyfds/acoustics.py:166-176, pyfds/thermal.py:132-142)."""
    return np.tile(np.arange(0, nx) * dx, ny) + dx / 2


def assemble(spec, scale=None):
    """Build the operators of one field (the ``assemble_matrices`` of each kind).

    ``spec`` keys: kind, nx, ny (2-D), dx, dy (2-D), dt, materials.
    Returns a dict of DIA operators plus the vectors ``sim_step`` needs every step.
    """
    kind = spec["kind"]
    dt, dx = spec["dt"], spec["dx"]
    nx = spec["nx"]
    ny = spec.get("ny", 1)
    dy = spec.get("dy", None)
    n = nx * ny
    mats = spec["materials"]

    def mv(name):
        # a MaterialCoupling multiplies one parameter by its transfer factors
        # (pyfds/coupling.py:181-196)
        if scale and name in scale:
            return material_vector(n, mats, name) * scale[name]
        return material_vector(n, mats, name)

    ops = {"n": n, "nx": nx}
    if kind == "AcousticFlow2D":
        kind = "Acoustic2D"  # pyfds/acoustic_flow.py:13: the Acoustic2D operators
    if kind in ("IdealGas1D", "Acoustic2ndOrder1D"):
        # pyfds/nonlinear_acoustics.py:38-53 and :124-138
        ops["a_d_v"] = d_x(n, dt / dx * np.ones(nx))
        ops["a_v_p"] = d_x(n, (dt / dx) * np.ones(nx), variant="backward")
        ops["a_v_v"] = d_x2(n, dt / dx ** 2 * mv("absorption_coef"))
        ops["a_v_v2"] = d_x(n, (dt / dx / 2) * np.ones(nx), variant="central")
        ops["stat_density"] = mv("density")
        if kind == "IdealGas1D":
            ops["sound_velocity"] = mv("sound_velocity")
            ops["heat_cap_ratio"] = mv("isobaric_heat_cap") / mv("isochoric_heat_cap")
            ops["convective"] = bool(spec.get("convective", True))
            ops["nl_state"] = bool(spec.get("nl_state", True))
        else:
            ops["d_rho_p"] = mv("d_rho_p")
            ops["d_rho2_p"] = mv("d_rho2_p")
            ops["convective"] = True
        return ops
    if kind == "Acoustic1D":
        # pyfds/acoustics.py:27-38
        ops["a_p_v"] = d_x(n, dt / dx * mv("sound_velocity") ** 2 * mv("density"))
        ops["a_v_p"] = d_x(n, dt / dx / mv("density"), variant="backward")
        ops["a_v_v"] = d_x2(n, dt / dx ** 2 * mv("absorption_coef") / mv("density"))
    elif kind == "Acoustic2D":
        # pyfds/acoustics.py:89-109
        ops["a_p_vx"] = d_x(n, dt / dx * mv("sound_velocity") ** 2 * mv("density"))
        ops["a_p_vy"] = d_y(n, nx, dt / dy * mv("sound_velocity") ** 2 * mv("density"))
        ops["a_vx_p"] = d_x(n, dt / dx / mv("density"), variant="backward")
        ops["a_vy_p"] = d_y(n, nx, dt / dy / mv("density"), variant="backward")
        ops["a_vx_vx"] = dia_sum(
            d_x2(n, dt / dx ** 2 * mv("absorption_coef") / mv("density")),
            d_y2(n, nx, dt / dy ** 2 * mv("absorption_coef") / mv("density")))
        ops["a_vy_vy"] = ops["a_vx_vx"]
    elif kind == "Acoustic3DAxi":
        # pyfds/acoustics.py:178-203
        r = _radii(nx, ny, dx)
        ops["radii"] = r
        ops["a_p_vx"] = d_x(n, dt / dx * mv("sound_velocity") ** 2 * mv("density") / r)
        ops["a_p_vy"] = d_y(n, nx, dt / dy * mv("sound_velocity") ** 2 * mv("density"))
        ops["a_vx_p"] = d_x(n, dt / dx / mv("density"), variant="backward")
        ops["a_vy_p"] = d_y(n, nx, dt / dy / mv("density"), variant="backward")
        ops["a_vx_vx"] = dia_sum(
            d_x2(n, dt / dx ** 2 * mv("absorption_coef") / mv("density")),
            d_y2(n, nx, dt / dy ** 2 * mv("absorption_coef") / mv("density")),
            d_x(n, dt / dx * mv("absorption_coef") / mv("density") / r, variant="central"))
        ops["a_vy_vy"] = ops["a_vx_vx"]
        # per-step explicit radial loss term (pyfds/acoustics.py:213-215)
        ops["mu"] = mv("absorption_coef")
        ops["rho"] = mv("density")
    elif kind == "Thermal1D":
        # pyfds/thermal.py:29-38
        ops["a_t_q"] = d_x(n, dt / dx / mv("density") / mv("heat_capacity"))
        ops["a_q_t"] = d_x(n, 1 / dx * mv("thermal_conductivity_x"), variant="backward")
    elif kind == "Thermal2D":
        # pyfds/thermal.py:75-90
        ops["a_t_qx"] = d_x(n, dt / dx / mv("density") / mv("heat_capacity"))
        ops["a_t_qy"] = d_y(n, nx, dt / dy / mv("density") / mv("heat_capacity"))
        ops["a_qx_t"] = d_x(n, 1 / dx * mv("thermal_conductivity_x"), variant="backward")
        ops["a_qy_t"] = d_y(n, nx, 1 / dy * mv("thermal_conductivity_y"), variant="backward")
    elif kind == "Thermal3DAxi":
        # pyfds/thermal.py:144-159
        r = _radii(nx, ny, dx)
        ops["radii"] = r
        ops["a_t_qx"] = d_x(n, dt / dx / mv("density") / mv("heat_capacity") / r)
        ops["a_t_qy"] = d_y(n, nx, dt / dy / mv("density") / mv("heat_capacity"))
        ops["a_qx_t"] = d_x(n, 1 / dx * mv("thermal_conductivity_x"), variant="backward")
        ops["a_qy_t"] = d_y(n, nx, 1 / dy * mv("thermal_conductivity_y"), variant="backward")
    else:
        raise ValueError("unknown field kind %r" % kind)
    return ops


# --------------------------------------------------------------------------------------
# Boundaries and outputs (pyfds/regions.py:125-165, pyfds/fields.py:591-611)
# --------------------------------------------------------------------------------------


def _boundary_new_values(value, additive, old, step):
    """``Boundary.apply`` (pyfds/regions.py:125-145)."""
    if np.ndim(value) == 0:
        return additive * old + value
    elif isinstance(value, np.ndarray):
        return additive * old + value[step]
    else:
        return [additive * old[ii] + signal[step] for ii, signal in enumerate(value)]


def apply_bounds(values, bounds, step):
    """``FieldComponent.apply_bounds`` (pyfds/fields.py:591-600): in list order, numpy
    fancy assignment (duplicate indices: the last write wins)."""
    for b in bounds:
        idx = b["indices"]
        values[idx] = _boundary_new_values(b["value"], b.get("additive", False),
                                           values[idx], step)


def write_outputs(values, outputs, signals):
    """``FieldComponent.write_outputs`` (pyfds/fields.py:602-611): one sample per index."""
    for k, idx in enumerate(outputs):
        sig = signals[k]
        for j, index in enumerate(idx):
            sig[j].append(values[index])


# --------------------------------------------------------------------------------------
# Time step per kind
# --------------------------------------------------------------------------------------


def sim_step(kind, ops, state, bounds, outputs, signals, step, dt=None, matvec=None,
             inplace=False):
    """One ``sim_step`` of the given kind, in place on ``state`` (dict name -> array).

    ``bounds``/``outputs``/``signals`` are dicts keyed by component name. ``matvec``
    (default: ``dia_matvec`` on the operator lists) lets the CPU-baseline worker run
    the operators as scipy matrices, the reference's own product. ``inplace``
    subtracts each update into the state array itself, as the reference's ``-=``
    does, instead of binding a new array (same values; the worker sets it so that
    its timing carries no extra allocation).
    """
    mv = matvec or dia_matvec

    def update(name, delta):
        """state[name] - delta."""
        if inplace:
            np.subtract(state[name], delta, out=state[name])
        else:
            state[name] = state[name] - delta

    def pre(name):
        apply_bounds(state[name], bounds.get(name, []), step)
        write_outputs(state[name], outputs.get(name, []), signals.setdefault(name, []))

    if kind in ("IdealGas1D", "Acoustic2ndOrder1D"):
        # pyfds/nonlinear_acoustics.py:55-90 and :140-163
        pre("pressure")
        rho0 = ops["stat_density"]
        v = state["velocity"]
        if ops["convective"]:
            state["velocity"] = v - (mv(ops["a_v_p"], state["pressure"]) / (rho0 + state["density"])
                                     + mv(ops["a_v_v2"], v)
                                     - mv(ops["a_v_v"], v) / (rho0 + state["density"]))
        else:
            state["velocity"] = v - (mv(ops["a_v_p"], state["pressure"]) / (rho0 + state["density"])
                                     - mv(ops["a_v_v"], v) / (rho0 + state["density"]))
        pre("velocity")
        state["density"] = state["density"] - mv(ops["a_d_v"],
                                                 (state["density"] + rho0) * state["velocity"])
        pre("density")
        d = state["density"]
        if kind == "IdealGas1D":
            c, g = ops["sound_velocity"], ops["heat_cap_ratio"]
            if ops["nl_state"]:
                state["pressure"] = rho0 * c ** 2 / g * (((rho0 + d) / rho0) ** g - 1)
            else:
                state["pressure"] = c ** 2 * d
        else:
            state["pressure"] = ops["d_rho_p"] * d + ops["d_rho2_p"] / 2 * d ** 2
    elif kind == "Acoustic1D":
        # pyfds/acoustics.py:40-52
        pre("pressure")
        update("velocity", mv(ops["a_v_p"], state["pressure"])
               - mv(ops["a_v_v"], state["velocity"]))
        pre("velocity")
        update("pressure", mv(ops["a_p_v"], state["velocity"]))
    elif kind == "Acoustic2D":
        # pyfds/acoustics.py:111-128
        pre("pressure")
        p = state["pressure"]
        update("velocity_x", mv(ops["a_vx_p"], p) - mv(ops["a_vx_vx"], state["velocity_x"]))
        update("velocity_y", mv(ops["a_vy_p"], p) - mv(ops["a_vy_vy"], state["velocity_y"]))
        pre("velocity_x")
        pre("velocity_y")
        update("pressure", mv(ops["a_p_vx"], state["velocity_x"])
               + mv(ops["a_p_vy"], state["velocity_y"]))
    elif kind == "Acoustic3DAxi":
        # pyfds/acoustics.py:205-225
        pre("pressure")
        p = state["pressure"]
        r = ops["radii"]
        vx = state["velocity_x"]
        update("velocity_x", mv(ops["a_vx_p"], p) - mv(ops["a_vx_vx"], vx)
               + dt * ops["mu"] / ops["rho"] * vx / r ** 2)
        update("velocity_y", mv(ops["a_vy_p"], p) - mv(ops["a_vy_vy"], state["velocity_y"]))
        pre("velocity_x")
        pre("velocity_y")
        update("pressure", mv(ops["a_p_vx"], state["velocity_x"] * r)
               + mv(ops["a_p_vy"], state["velocity_y"]))
    elif kind == "Thermal1D":
        # pyfds/thermal.py:40-51
        pre("temperature")
        state["heat_flux"] = -mv(ops["a_q_t"], state["temperature"])
        pre("heat_flux")
        update("temperature", mv(ops["a_t_q"], state["heat_flux"]))
    elif kind == "Thermal2D":
        # pyfds/thermal.py:92-107
        pre("temperature")
        t = state["temperature"]
        state["heat_flux_x"] = -mv(ops["a_qx_t"], t)
        state["heat_flux_y"] = -mv(ops["a_qy_t"], t)
        pre("heat_flux_x")
        pre("heat_flux_y")
        update("temperature", mv(ops["a_t_qx"], state["heat_flux_x"])
               + mv(ops["a_t_qy"], state["heat_flux_y"]))
    elif kind == "Thermal3DAxi":
        # pyfds/thermal.py:161-176
        pre("temperature")
        t = state["temperature"]
        r = ops["radii"]
        state["heat_flux_x"] = -mv(ops["a_qx_t"], t)
        state["heat_flux_y"] = -mv(ops["a_qy_t"], t)
        pre("heat_flux_x")
        pre("heat_flux_y")
        update("temperature", mv(ops["a_t_qx"], state["heat_flux_x"] * r)
               + mv(ops["a_t_qy"], state["heat_flux_y"]))
    else:
        raise ValueError("unknown field kind %r" % kind)


def flow_periods(spec):
    """``AcousticFlow2D.flow_t_deltas`` (pyfds/acoustic_flow.py:27-37): per row, the
    step period of the one-cell shift, ``int(dx / flow / dt)``."""
    flow, ny = spec["flow"], spec["ny"]
    if isinstance(flow, (list, np.ndarray)) and len(flow) == ny:
        f = np.asarray(flow)
    elif isinstance(flow, (float, int)):
        f = np.ones(ny) * flow
    else:
        raise ValueError('Flow must either be scalar or a vector with length of y_samples.')
    with np.errstate(divide="ignore", invalid="ignore"):
        return (spec["dx"] / f / spec["dt"]).astype(int)


def apply_flow(state, periods, step, nx):
    """``AcousticFlow2D.apply_flow`` (pyfds/acoustic_flow.py:49-57): rows whose period
    divides the step move one cell in +x, their first cell becomes 0."""
    for c in ("pressure", "velocity_x", "velocity_y"):
        v = state[c]
        for n, f in enumerate(periods):
            with np.errstate(divide="ignore", invalid="ignore"):
                due = step % f == 0
            if due:
                v[n * nx + 1:(n + 1) * nx] = v[n * nx:(n + 1) * nx - 1]
                v[n * nx:n * nx + 1] = 0


def simulate(spec, num_steps=None, state=None, step0=0):
    """Run ``num_steps`` steps of the scenario ``spec`` (``Field.simulate``,
    pyfds/fields.py:67-95: assemble once, then ``sim_step(); step += 1``).

    ``spec``: kind, nx, [ny], dx, [dy], dt, nt, materials, [init], [bounds], [outputs].
    Returns ``(state, signals)``; ``signals[name][k]`` is an array of shape
    ``(len(indices_k), steps)`` for output ``k`` of component ``name``.
    """
    kind = spec["kind"]
    ops = assemble(spec)
    n = ops["n"]
    if state is None:
        state = {c: np.zeros(n) for c in components_of(kind)}
        for c, v in (spec.get("init") or {}).items():
            state[c] = np.array(v, dtype=np.float64).copy()
    if num_steps is None:
        num_steps = spec["nt"]
    bounds = spec.get("bounds") or {}
    outputs = spec.get("outputs") or {}
    signals = {c: [[[] for _ in idx] for idx in outputs.get(c, [])] for c in components_of(kind)}
    periods = flow_periods(spec) if kind == "AcousticFlow2D" else None
    step_kind = "Acoustic2D" if kind == "AcousticFlow2D" else kind
    for s in range(step0, step0 + num_steps):
        sim_step(step_kind, ops, state, bounds, outputs, signals, s, dt=spec["dt"])
        if periods is not None:
            apply_flow(state, periods, s, ops["nx"])
    out = {c: [np.array(sig, dtype=np.float64).reshape(len(sig), -1) for sig in signals[c]]
           for c in signals}
    return state, out


# --------------------------------------------------------------------------------------
# Coupled fields (pyfds/coupling.py, pyfds/coupled_fields.py)
# --------------------------------------------------------------------------------------


def transfer(fn, values):
    """Transfer functions of the coupling scenarios: ("quad", c) -> c x^2,
    ("power", power, factor) -> 1 + factor x^power (pyfds/coupling.py:287-300),
    ("exp", a, b) -> a + (1 - a) exp(b x) (pyfds/coupling.py:243-254)."""
    if fn[0] == "quad":
        return fn[1] * values ** 2
    if fn[0] == "power":
        return 1 + fn[2] * values ** fn[1]
    if fn[0] == "exp":
        return fn[1] + (1 - fn[1]) * np.exp(fn[2] * values)
    raise ValueError(fn)


def thermoacoustic_spec_fields(spec):
    """The two field specs of ThermoAcoustic1D (pyfds/coupled_fields.py:18-39)."""
    base = {"nx": spec["nx"], "dx": spec["dx"], "dt": spec["dt"], "nt": spec["nt"]}
    ac = dict(base, kind="Acoustic1D", materials=[(None, spec["acoustic_material"])])
    th = dict(base, kind="Thermal1D", materials=[(None, spec["thermal_material"])])
    for f, names in ((ac, ("pressure", "velocity")), (th, ("temperature", "heat_flux"))):
        for key in ("bounds", "outputs", "init"):
            sub = {c: v for c, v in (spec.get(key) or {}).items() if c in names}
            if sub:
                f[key] = sub
    return [ac, th]


def coupled_interactions(spec):
    """Interaction list of a coupled spec; ThermoAcoustic1D's loss coupling is
    ("loss") from the acoustic velocity into the temperature."""
    if spec["kind"] == "ThermoAcoustic1D":
        st = spec.get("stepping", 1)
        return [{"type": "boundary", "src": [0, "velocity"], "dst": [1, "temperature"],
                 "fn": ["loss"], "additive": True, "accumulate": st > 1, "stepping": st}]
    return spec["interactions"]


def simulate_coupled(spec, num_steps=None):
    """``SynchronizedFields.simulate`` (pyfds/coupling.py:14-87 with
    pyfds/fields.py:67-95): assemble every field (material couplings apply their
    factors of the initial source values), then per step every field's sim_step in
    list order and every interaction's apply(step). Returns ([(state, signals) per
    field])."""
    fields = (thermoacoustic_spec_fields(spec) if spec["kind"] == "ThermoAcoustic1D"
              else spec["fields"])
    inter = coupled_interactions(spec)
    n = fields[0]["nx"] * fields[0].get("ny", 1)
    states = []
    for f in fields:
        st = {c: np.zeros(n) for c in components_of(f["kind"])}
        for c, v in (f.get("init") or {}).items():
            st[c] = np.array(v, dtype=np.float64).copy()
        states.append(st)
    scales = [dict() for _ in fields]

    def mat_factors(it):
        return transfer(it["fn"], states[it["src"][0]][it["src"][1]])

    for it in inter:
        if it["type"] == "material":
            scales[it["field"]][it["param"]] = mat_factors(it)
            it["_last"] = 0
    ops = [assemble(f, scales[k]) for k, f in enumerate(fields)]
    signals = []
    for f in fields:
        outs = f.get("outputs") or {}
        signals.append({c: [[[] for _ in idx] for idx in outs.get(c, [])]
                        for c in components_of(f["kind"])})
    acc = [0 for _ in inter]
    if num_steps is None:
        num_steps = spec["nt"]
    for s in range(num_steps):
        for k, f in enumerate(fields):
            sim_step(f["kind"], ops[k], states[k], f.get("bounds") or {}, f.get("outputs") or {},
                     signals[k], s, dt=f["dt"])
        for j, it in enumerate(inter):
            if it["type"] == "boundary":
                src = states[it["src"][0]][it["src"][1]]
                if it["fn"][0] == "loss":
                    # ThermoAcoustic1D._loss_coupling (pyfds/coupled_fields.py:45-65)
                    ac_f, th_f = fields
                    vd = dia_matvec(ops[0]["a_v_p"], src * material_vector(n, ac_f["materials"],
                                                                            "density"))
                    tf = lambda: (material_vector(n, ac_f["materials"], "absorption_coef")
                                  / material_vector(n, th_f["materials"], "density")
                                  / material_vector(n, th_f["materials"], "heat_capacity")
                                  * vd ** 2 * spec["dt"])
                else:
                    tf = lambda: transfer(it["fn"], src)
                dst = states[it["dst"][0]]
                name = it["dst"][1]
                if it["accumulate"] is True:
                    acc[j] += tf()
                if s % it["stepping"] == 0:
                    val = tf() if it["accumulate"] is False else acc[j]
                    if it["accumulate"] is not False:
                        acc[j] = 0
                    dst[name] = dst[name] + val if it["additive"] is True else val
            elif it["type"] == "material":
                if s % it["stepping"] == 0:
                    tf = mat_factors(it)
                    rel = max(abs((tf - it["_last"]) / tf))
                    if it.get("rel") is None or rel > it["rel"]:
                        scales[it["field"]][it["param"]] = tf
                        ops[it["field"]] = assemble(fields[it["field"]], scales[it["field"]])
                        it["_last"] = tf
    out = []
    for k, f in enumerate(fields):
        sig = {c: [np.array(x, dtype=np.float64).reshape(len(x), -1) for x in signals[k][c]]
               for c in signals[k]}
        out.append((states[k], sig))
    return out

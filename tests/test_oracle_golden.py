"""The CPU oracle, pinned: against the reference's own known-answer operator
matrices (test/test_acoustics.py:19-66, test/test_fields.py:57-107,
test/test_coupling.py:113-118) and against trajectories of the unmodified
reference stored in tests/golden (generated by tests/golden/make_golden.py)."""
import json
import os

import numpy as np
import pytest

from oracle import fds_oracle as O
from oracle import scenarios as S

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def dense(op, n):
    return O.dia_to_dense(op, n)


def test_known_answer_acoustic1d():
    # test/test_acoustics.py:19-26: c=700, rho=0.01, bulk viscosity 1 -> mu = 1
    spec = {"kind": "Acoustic1D", "nx": 3, "dx": 1, "dt": 1,
            "materials": [(None, {"sound_velocity": 700, "density": 0.01, "absorption_coef": 1})]}
    ops = O.assemble(spec)
    assert np.allclose(dense(ops["a_p_v"], 3), [[-4900, 4900, 0], [0, -4900, 4900], [0, 0, -4900]])
    assert np.allclose(dense(ops["a_v_p"], 3), [[100, 0, 0], [-100, 100, 0], [0, -100, 100]])
    assert np.allclose(dense(ops["a_v_v"], 3), [[-200, 100, 0], [100, -200, 100], [0, 100, -200]])


def test_known_answer_acoustic2d():
    # test/test_acoustics.py:29-46 (2 x 2, including the x wrap of cell 1 -> 2)
    spec = {"kind": "Acoustic2D", "nx": 2, "ny": 2, "dx": 1, "dy": 1, "dt": 1,
            "materials": [(None, {"sound_velocity": 700, "density": 0.01, "absorption_coef": 1})]}
    ops = O.assemble(spec)
    assert np.allclose(dense(ops["a_p_vx"], 4), [[-4900, 4900, 0, 0], [0, -4900, 4900, 0],
                                                 [0, 0, -4900, 4900], [0, 0, 0, -4900]])
    assert np.allclose(dense(ops["a_p_vy"], 4), [[-4900, 0, 4900, 0], [0, -4900, 0, 4900],
                                                 [0, 0, -4900, 0], [0, 0, 0, -4900]])
    assert np.allclose(dense(ops["a_vx_p"], 4), [[100, 0, 0, 0], [-100, 100, 0, 0],
                                                 [0, -100, 100, 0], [0, 0, -100, 100]])
    assert np.allclose(dense(ops["a_vy_p"], 4), [[100, 0, 0, 0], [0, 100, 0, 0],
                                                 [-100, 0, 100, 0], [0, -100, 0, 100]])
    expect = [[-400, 100, 100, 0], [100, -400, 100, 100], [100, 100, -400, 100],
              [0, 100, 100, -400]]
    assert np.allclose(dense(ops["a_vx_vx"], 4), expect)
    assert np.allclose(dense(ops["a_vy_vy"], 4), expect)


def test_known_answer_acoustic3d_axi():
    # test/test_acoustics.py:49-66 (radius column scaling, r = 0.5, 1.5)
    spec = {"kind": "Acoustic3DAxi", "nx": 2, "ny": 2, "dx": 1, "dy": 1, "dt": 1,
            "materials": [(None, {"sound_velocity": 1, "density": 1, "absorption_coef": 1})]}
    ops = O.assemble(spec)
    assert np.allclose(dense(ops["a_p_vx"], 4), [[-2, 2 / 3, 0, 0], [0, -2 / 3, 2, 0],
                                                 [0, 0, -2, 2 / 3], [0, 0, 0, -2 / 3]])
    assert np.allclose(dense(ops["a_p_vy"], 4), [[-1, 0, 1, 0], [0, -1, 0, 1],
                                                 [0, 0, -1, 0], [0, 0, 0, -1]])
    assert np.allclose(dense(ops["a_vx_p"], 4), [[1, 0, 0, 0], [-1, 1, 0, 0], [0, -1, 1, 0],
                                                 [0, 0, -1, 1]])
    assert np.allclose(dense(ops["a_vy_p"], 4), [[1, 0, 0, 0], [0, 1, 0, 0], [-1, 0, 1, 0],
                                                 [0, -1, 0, 1]])
    expect = [[-4, 4 / 3, 1, 0], [0, -4, 2, 1], [1, 2 / 3, -4, 4 / 3], [0, 1, 0, -4]]
    assert np.allclose(dense(ops["a_vx_vx"], 4), expect)
    assert np.allclose(dense(ops["a_vy_vy"], 4), expect)


def test_known_answer_thermal1d():
    # test/test_coupling.py:113-118
    spec = {"kind": "Thermal1D", "nx": 3, "dx": 1, "dt": 1,
            "materials": [(None, {"heat_capacity": 1, "density": 1,
                                  "thermal_conductivity_x": 1, "thermal_conductivity_y": 1})]}
    ops = O.assemble(spec)
    assert np.allclose(dense(ops["a_t_q"], 3), [[-1, 1, 0], [0, -1, 1], [0, 0, -1]])


def test_known_answer_derivative_operators():
    # test/test_fields.py:57-107
    assert np.allclose(dense(O.d_x(3), 3), [[-1, 1, 0], [0, -1, 1], [0, 0, -1]])
    assert np.allclose(dense(O.d_x(3, variant="backward"), 3), [[1, 0, 0], [-1, 1, 0], [0, -1, 1]])
    assert np.allclose(dense(O.d_x(3, variant="central"), 3),
                       [[0, 0.5, 0], [-0.5, 0, 0.5], [0, -0.5, 0]])
    assert np.allclose(dense(O.d_x2(3), 3), [[-2, 1, 0], [1, -2, 1], [0, 1, -2]])
    assert np.allclose(dense(O.d_x(4), 4), [[-1, 1, 0, 0], [0, -1, 1, 0], [0, 0, -1, 1],
                                            [0, 0, 0, -1]])
    assert np.allclose(dense(O.d_x(4, variant="central"), 4),
                       [[0, 0.5, 0, 0], [-0.5, 0, 0.5, 0], [0, -0.5, 0, 0.5], [0, 0, -0.5, 0]])
    assert np.allclose(dense(O.d_y(4, 2), 4), [[-1, 0, 1, 0], [0, -1, 0, 1], [0, 0, -1, 0],
                                               [0, 0, 0, -1]])
    assert np.allclose(dense(O.d_y(4, 2, variant="backward"), 4),
                       [[1, 0, 0, 0], [0, 1, 0, 0], [-1, 0, 1, 0], [0, -1, 0, 1]])
    assert np.allclose(dense(O.d_y(4, 2, variant="central"), 4),
                       [[0, 0, 0.5, 0], [0, 0, 0, 0.5], [-0.5, 0, 0, 0], [0, -0.5, 0, 0]])
    assert np.allclose(dense(O.d_y2(4, 2), 4), [[-2, 0, 1, 0], [0, -2, 0, 1], [1, 0, -2, 0],
                                                [0, 1, 0, -2]])
    with pytest.raises(ValueError):
        O.d_x(3, variant="sideways")


def test_boundary_semantics_known_answers():
    # test/test_fields.py:12-38
    v = np.random.default_rng(0).random(100)
    O.apply_bounds(v, [{"indices": [5, 6, 7], "value": 23}], step=0)
    assert np.allclose(v[[5, 6, 7]], 23)
    v = np.ones(100)
    O.apply_bounds(v, [{"indices": [5, 6, 7], "additive": True,
                        "value": [np.arange(3) * 23, np.arange(3) * 42, np.arange(3) * 23]}], step=1)
    assert np.allclose(v[[5, 6, 7]], [24, 43, 24])
    v = np.ones(100)
    O.apply_bounds(v, [{"indices": [5, 6, 7], "additive": True, "value": np.arange(3) * 23}],
                   step=2)
    assert np.allclose(v[[5, 6, 7]], [47, 47, 47])


def _load(name):
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.skip("fixture %s not generated" % name)
    return np.load(path)


def test_oracle_operators_match_golden():
    g = _load("operators.npz")
    kinds = sorted({k.split("/")[0] for k in g.files})
    assert len(kinds) == 6
    for kind in kinds:
        nx, ny, dx, dy, dt = g[kind + "/grid"]
        mats = [(None if i is None else np.array(i), p)
                for i, p in json.loads(str(g[kind + "/materials"]))]
        spec = {"kind": kind, "nx": int(nx), "ny": int(ny), "dx": dx, "dy": dy, "dt": dt,
                "materials": mats}
        ops = O.assemble(spec)
        n = int(nx * ny)
        for key in g.files:
            if not key.startswith(kind + "/a_"):
                continue
            name = key.split("/")[1]
            got = dense(ops[name], n)
            assert np.array_equal(got, g[key]), (kind, name)


def random_cases():
    g = _load("random_scenarios.npz")
    return json.loads(str(g["cases"])), g


def test_oracle_random_scenarios_bitwise():
    from golden_digest import spec_digest
    from golden_inputs import apply_inputs
    cases, g = random_cases()
    for case in cases:
        spec = S.random_scenario(case["seed"], case["kind"], case["nx"], case["ny"],
                                 steps=case["steps"], mu=case["mu"])
        prefix = "s%d/" % case["seed"]
        apply_inputs(spec, g, prefix)
        assert str(g[prefix + "digest"]) == spec_digest(spec), "scenario generator drifted"
        st, sig = O.simulate(spec, spec["steps"])
        for c in O.components_of(case["kind"]):
            assert np.array_equal(st[c], g[prefix + c + "/state"]), (case, c)
            for j, s in enumerate(sig[c]):
                assert np.array_equal(s, g[prefix + c + "/sig%d" % j]), (case, c, j)


def test_oracle_acoustic1d_water_bitwise():
    from pyfds_gb300 import workloads
    from golden_inputs import apply_inputs
    g = _load("acoustic1d_water.npz")
    spec = apply_inputs(workloads.acoustic1d_water(), g)
    st, sig = O.simulate(spec, spec["steps"])
    assert np.array_equal(sig["pressure"][0], g["pressure/sig0"])
    assert np.array_equal(st["pressure"], g["pressure/state"])
    assert np.array_equal(st["velocity"], g["velocity/state"])
    # the source pulse reaches the probe at index 800 with a peak |p| of 0.807
    assert abs(np.abs(sig["pressure"][0]).max() - 0.807) < 0.01


def test_oracle_thermal2d_small_bitwise():
    from pyfds_gb300 import workloads
    from golden_inputs import apply_inputs
    g = _load("thermal2d_512.npz")
    spec = apply_inputs(workloads.thermal2d_two_materials(512, 500, 64), g)
    st, sig = O.simulate(spec, spec["steps"])
    assert np.array_equal(sig["temperature"][0], g["temperature/sig0"])
    # reductions are summed in a platform-dependent order: compare to a few ulps
    assert np.allclose([np.linalg.norm(st["temperature"]), st["temperature"].sum()],
                       g["temperature/state_norm"], rtol=1e-13, atol=0)


@pytest.mark.slow
def test_oracle_axi_small_bitwise():
    from pyfds_gb300 import workloads
    from golden_inputs import apply_inputs
    g = _load("axi_disc_256x1024.npz")
    spec = apply_inputs(workloads.axi_disc_source(256, 1024, 500, disc=50, probe_every=32), g)
    st, sig = O.simulate(spec, spec["steps"])
    assert np.array_equal(sig["pressure"][0], g["pressure/sig0"])


def test_oracle_matches_live_reference():
    from oracle import ref_loader
    if not ref_loader.reference_available():
        pytest.skip("reference source tree not available")
    from oracle import ref_build
    for seed in (101, 102, 103, 104, 105, 106):
        kind = S.ALL_KINDS[seed % 6]
        spec = S.random_scenario(seed, kind, 6, None if kind.endswith("1D") else 5, steps=12)
        a = O.simulate(spec, spec["steps"])
        b = ref_build.run_reference(spec, spec["steps"])
        for c in a[0]:
            assert np.array_equal(a[0][c], b[0][c])


def test_oracle_flow_bitwise():
    """AcousticFlow2D (pyfds/acoustic_flow.py): the oracle against the reference's
    trajectories, bit for bit (per-row and scalar flows, periods 1..9, negative
    periods, a row at rest)."""
    import warnings
    from golden_digest import spec_digest
    from golden_inputs import apply_inputs
    g = _load("acoustic_flow.npz")
    for case in json.loads(str(g["cases"])):
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            spec = S.flow_scenario(case["seed"], case["nx"], case["ny"], steps=case["steps"],
                                   flow=case["flow"], mu=case["mu"])
        prefix = "f%d/" % case["seed"]
        apply_inputs(spec, g, prefix)
        assert str(g[prefix + "digest"]) == spec_digest(spec), "scenario generator drifted"
        st, sig = O.simulate(spec, spec["steps"])
        for c in O.components_of("AcousticFlow2D"):
            assert np.array_equal(st[c], g[prefix + c + "/state"]), (case, c)
            for j, s in enumerate(sig[c]):
                assert np.array_equal(s, g[prefix + c + "/sig%d" % j]), (case, c, j)


def test_oracle_flow_matches_live_reference():
    import warnings
    from oracle import ref_loader
    if not ref_loader.reference_available():
        pytest.skip("reference source tree not available")
    from oracle import ref_build
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        for seed in (301, 302):
            spec = S.flow_scenario(seed, 10, 6, steps=25, flow="rows" if seed % 2 else "scalar")
            a = O.simulate(spec, spec["steps"])
            b = ref_build.run_reference(spec, spec["steps"])
            for c in a[0]:
                assert np.array_equal(a[0][c], b[0][c])


def _nl_spec(case):
    return S.nonlinear_scenario(case["seed"], case["kind"], case["nx"], steps=case["steps"],
                                convective=case["convective"], nl_state=case["nl_state"],
                                mu=case["mu"])


def test_oracle_nonlinear_bitwise():
    """IdealGas1D / Acoustic2ndOrder1D (pyfds/nonlinear_acoustics.py): the oracle
    against the reference's trajectories, bit for bit."""
    from golden_digest import spec_digest
    from golden_inputs import apply_inputs
    g = _load("nonlinear_1d.npz")
    for case in json.loads(str(g["cases"])):
        spec = _nl_spec(case)
        prefix = "n%d/" % case["seed"]
        apply_inputs(spec, g, prefix)
        assert str(g[prefix + "digest"]) == spec_digest(spec), "scenario generator drifted"
        st, sig = O.simulate(spec, spec["steps"])
        for c in O.components_of(case["kind"]):
            assert np.array_equal(st[c], g[prefix + c + "/state"]), (case, c)
            for j, s in enumerate(sig[c]):
                assert np.array_equal(s, g[prefix + c + "/sig%d" % j]), (case, c, j)


def test_oracle_coupling_bitwise():
    """Coupled fields (pyfds/coupling.py, pyfds/coupled_fields.py): the oracle's
    SynchronizedFields stepping against the reference's trajectories, bit for bit."""
    from coupled_helpers import compare, coupled_spec
    from golden_digest import spec_digest
    g = _load("coupling.npz")
    for case in json.loads(str(g["cases"])):
        spec, prefix = coupled_spec(case, g)
        assert str(g[prefix + "digest"]) == spec_digest(spec), "scenario generator drifted"

        def check(a, b, where):
            assert np.array_equal(a, b), (case, where)
        compare(O.simulate_coupled(spec, spec["steps"]), g, prefix, check)


@pytest.mark.parametrize("kind", ["Acoustic1D", "Acoustic2D", "Acoustic3DAxi", "Thermal1D",
                                  "Thermal2D", "Thermal3DAxi"])
def test_baseline_worker_path_matches_the_oracle(kind):
    """The CPU-baseline worker's step (scipy DIA products, in-place updates) gives the
    oracle's values: bit for bit where scipy does not contract multiply-adds, within
    1e-13 otherwise."""
    from oracle import bench_worker as W
    nx, ny = (23, None) if kind.endswith("1D") else (11, 7)
    spec = S.random_scenario(31, kind, nx, ny, steps=6, mu=True)
    ops = O.assemble(spec)
    sops = W.scipy_operators(ops)
    runs = []
    for o, kw in ((ops, {}), (sops, {"matvec": W._dot, "inplace": True})):
        st = {c: np.array(v, dtype=np.float64) for c, v in (spec.get("init") or {}).items()}
        for c in O.components_of(kind):
            st.setdefault(c, np.zeros(ops["n"]))
        outs = spec.get("outputs") or {}
        sig = {c: [[[] for _ in idx] for idx in outs.get(c, [])] for c in st}
        for s in range(spec["steps"]):
            O.sim_step(kind, o, st, spec.get("bounds") or {}, outs, sig, s, dt=spec["dt"], **kw)
        runs.append((st, sig))
    (a, sa), (b, sb) = runs
    for c in a:
        scale = max(np.linalg.norm(a[c]), 1e-300)
        assert np.linalg.norm(a[c] - b[c]) <= 1e-13 * scale, c
        assert len(sa[c]) == len(sb[c])
        for x, y in zip(sa[c], sb[c]):  # one output each (outputs differ in size)
            x, y = np.asarray(x, dtype=float), np.asarray(y, dtype=float)
            assert x.shape == y.shape and np.allclose(x, y, rtol=1e-13, atol=0), c
